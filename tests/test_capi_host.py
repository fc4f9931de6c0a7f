"""C-ABI library: loads without a GPU, exports every symbol the public headers
declare, and its host-only logic and argument validation behave (no kernel
launches here)."""
import ctypes as C
import importlib
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADERS = sorted((ROOT / "include").glob("*.h"))


def _p3(v):
    import importlib
    return importlib.import_module("3deye_gb300").Point3i(v, v, v)


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tde_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(tde):
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(tde.lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "3deye_gb300" / "lib3deye_gb300.so")],
                         capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert names <= exported


def test_version_and_error_slot(tde):
    assert b"sm_103a" in tde.lib.tde_version()
    rc = tde.lib.tde_raycast(None, 0, None, None, None, None, 0.1, None, None, None, None)
    assert rc == -1
    assert "raycast" in tde.last_error()


def test_determine_extract_step(tde):
    step, n = C.c_uint(), C.c_uint()
    for depth, div, exp in [(512, 4, (64, 8)), (256, 4, (32, 8)), (128, 4, (16, 8)), (512, 2, (128, 4)),
                            (128, 1, (64, 2))]:
        assert tde.lib.tde_determine_extract_step(depth, div, C.byref(step), C.byref(n)) == 0
        assert (step.value, n.value) == exp
    assert tde.lib.tde_determine_extract_step(1024, 4, C.byref(step), C.byref(n)) == -7
    assert tde.lib.tde_determine_extract_step(512, 0, C.byref(step), C.byref(n)) == -1


def test_round_buffer_init_and_volume_bytes(tde):
    rb = tde.round_buffer((512, 512, 512), (3.0, 3.0, 3.0))
    assert rb.buffer_length == 512 ** 3 and rb.start_index == 0
    assert tuple(rb.volume_size.__getattribute__(a) for a in "xyz") == (3.0, 3.0, 3.0)
    assert tde.tsdf_volume_bytes(tde.TSDF_I16, rb) == 4 * 512 ** 3
    assert tde.tsdf_volume_bytes(tde.TSDF_F16, rb) == 4 * 512 ** 3
    assert tde.tsdf_volume_bytes(tde.TSDF_F32, rb) == 6 * 512 ** 3
    assert tde.tsdf_volume_bytes(7, rb) == 0
    bad = tde.round_buffer((1024, 1024, 4096), (1.0, 1.0, 1.0))
    assert tde.tsdf_volume_bytes(0, bad) == 0  # beyond int32 voxel addressing


_DUMMY = C.c_void_p(256)  # never dereferenced: each call below fails validation first


def _p3f(v):
    from importlib import import_module
    return import_module("3deye_gb300").Point3f(v, v, v)


def _light(number):
    from importlib import import_module
    t = import_module("3deye_gb300")
    return t.LightSource(t.Point3f(0.0, 0.0, 0.0), number)


@pytest.mark.parametrize("call", [
    lambda L, rb: L.tde_integrate_tsdf(None, None, 0, 0.03, None, None, None, None, C.byref(rb), 128, None),
    lambda L, rb: L.tde_tsdf_init(None, 0, C.byref(rb), None),
    lambda L, rb: L.tde_bilateral_filter(None, None, 64, 48, 4.5, 30.0, 4000, None),
    lambda L, rb: L.tde_normal_map(None, None, 0, 0, None),
    lambda L, rb: L.tde_extract_slice(None, 0, None, _p3(0), _p3(1), C.byref(rb), None, 0, None, None, None, 0,
                                      None, None),
    lambda L, rb: L.tde_clean_tsdf_slice(None, 0, _p3(0), _p3(0), C.byref(rb), None),
    lambda L, rb: L.tde_raycast(None, 5, None, None, None, None, 0.1, None, C.byref(rb), None, None),
    # whole-volume export, colour lookup, shading: refused before any device work
    lambda L, rb: L.tde_extract_tsdf_volume(None, 0, C.byref(rb), _p3f(0.1), None, 0, None, None, 0, None, None),
    lambda L, rb: L.tde_extract_tsdf_volume(_DUMMY, 0, C.byref(rb), _p3f(0.0), _DUMMY, 64, None, None, 0, _DUMMY,
                                            None),
    lambda L, rb: L.tde_extract_tsdf_volume(_DUMMY, 9, C.byref(rb), _p3f(0.1), _DUMMY, 64, None, None, 0, _DUMMY,
                                            None),
    lambda L, rb: L.tde_extract_color_volume(None, C.byref(rb), None, 0, _p3f(0.1), None, None),
    lambda L, rb: L.tde_extract_color_volume(_DUMMY, C.byref(rb), _DUMMY, 4, _p3f(float("nan")), _DUMMY, None),
    lambda L, rb: L.tde_generate_image(_DUMMY, _DUMMY, 4, 4, C.byref(_light(2)), _DUMMY, None),
    lambda L, rb: L.tde_generate_image(_DUMMY, _DUMMY, 0, 4, C.byref(_light(1)), _DUMMY, None),
    lambda L, rb: L.tde_generate_image(None, _DUMMY, 4, 4, C.byref(_light(1)), _DUMMY, None),
    # pipeline checkpoint / resume and pose-driven shifts without a pipeline
    lambda L, rb: L.tde_pipeline_checkpoint(None, None, 0),
    lambda L, rb: L.tde_pipeline_restore(None, None, 0),
    lambda L, rb: L.tde_pipeline_shift_needed_pose(None, None, 1.5, 0.4, None),
])
def test_invalid_arguments_are_reported(tde, call):
    importlib.import_module("3deye_gb300.pipeline")  # declares the pipeline entry points
    rb = tde.round_buffer((8, 8, 8), (1.0, 1.0, 1.0))
    assert call(tde.lib, rb) == -1


def test_checkpoint_size_without_pipeline(tde):
    importlib.import_module("3deye_gb300.pipeline")
    assert tde.lib.tde_pipeline_checkpoint_bytes(None) == 0


def test_host_icp_solve_matches_oracle(tde, orc):
    rng = np.random.default_rng(5)
    J = rng.normal(0, 1, (500, 6))
    r = rng.normal(0, 0.01, 500)
    A = J.T @ J
    b = J.T @ r
    sums = []
    for k in range(6):
        for j in range(k, 7):
            sums.append(b[k] if j == 6 else A[k, j])
    sums = np.array(sums, np.float32)
    R = np.eye(3)
    t = np.array([0.1, 0.2, 0.3])
    R1, t1, x = R.copy().ravel(), t.copy(), np.zeros(6)
    assert tde.lib.tde_icp_solve_update_host(sums.ctypes.data_as(C.c_void_p), R1.ctypes.data_as(C.c_void_p),
                                             t1.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p)) == 0
    st, R2, t2, x2 = orc.icp_solve(sums.astype(np.float64), R.ravel(), t)
    assert st == 0
    np.testing.assert_allclose(x, x2, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(R1, R2.ravel(), atol=1e-14)
    np.testing.assert_allclose(np.linalg.solve(A, b), x, rtol=1e-5)
    Rm = R1.reshape(3, 3)
    np.testing.assert_allclose(Rm @ Rm.T, np.eye(3), atol=1e-12)
