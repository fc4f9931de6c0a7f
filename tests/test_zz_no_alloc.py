"""tde_integrate_tsdf_noalloc: TSDF integration for callers that cannot
allocate device memory (its scratch is a fixed array in the library's static
device memory).  It must give exactly what tde_integrate_tsdf gives, call
after call, and refuse configurations whose scratch would not fit.

Kept in a file pytest collects last, so a run that stops at its first failure
has run every other test before this one."""
import ctypes as C
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _declare(tde):
    L = tde.lib
    L.tde_integrate_tsdf_noalloc.restype = C.c_int
    L.tde_integrate_tsdf_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.POINTER(tde.Matrix3f),
                                             C.POINTER(tde.Point3f), C.POINTER(tde.Intrinsics),
                                             C.POINTER(tde.Point3f), C.POINTER(tde.RoundBuffer), C.c_int, C.c_void_p]
    L.tde_integrate_tsdf_noalloc_max_scratch_bytes.restype = C.c_size_t
    L.tde_integrate_tsdf_scratch_bytes.restype = C.c_size_t
    L.tde_integrate_tsdf_scratch_bytes.argtypes = [C.c_int, C.c_int, C.POINTER(tde.RoundBuffer)]
    return L


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_noalloc_matches_integrate_on_consecutive_calls(tde, orc, cuda, fmt):
    import torch
    syn = importlib.import_module("3deye_gb300.synth")
    L = _declare(tde)
    cfg = syn.small_config("c1", frames=2, cols=160, rows=120, voxels=64, fmt=fmt)
    scene = syn.make_scene(cfg, 1000)
    traj = syn.make_trajectory(cfg, 2000)
    oi = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    ti = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    rb = tde.round_buffer((cfg.voxels,) * 3, (cfg.volume_m,) * 3, (9, 40, 3))
    ref = tde.new_volume(fmt, rb)
    out = tde.new_volume(fmt, rb)
    cell = (cfg.cell,) * 3
    for i in range(2):  # two calls in a row: the shared array carries the first call's contents
        depth = orc.apply_noise(orc.render_depth(scene, traj[i], oi), 3000, i)
        sd = tde.scale_depth(torch.from_numpy(depth).to(cuda), ti)
        R = traj[i, :9].reshape(3, 3).astype(np.float32)
        t = traj[i, 9:].astype(np.float32)
        tde.integrate_tsdf(sd, ref, fmt, cfg.trunc_m, R.T.copy(), t, ti, cell, rb, cfg.max_weight)
        Ri, tt, cs = tde.mat3(R.T.copy()), tde.vec3(t), tde.vec3(cell)
        tde.check(L.tde_integrate_tsdf_noalloc(sd.data_ptr(), out.data_ptr(), fmt, cfg.trunc_m, C.byref(Ri),
                                               C.byref(tt), C.byref(ti), C.byref(cs), C.byref(rb), cfg.max_weight,
                                               tde.stream_ptr()))
        torch.cuda.synchronize()
        assert torch.equal(out, ref), f"call {i + 1}: volume differs from tde_integrate_tsdf"
    assert (ref != 0).any()


def test_noalloc_at_its_advertised_capacity(tde, orc, cuda):
    """The largest configuration the fixed array is sized for: a 512^3 volume
    with 640x480 frames, two calls in a row, equal to tde_integrate_tsdf."""
    import torch
    syn = importlib.import_module("3deye_gb300.synth")
    L = _declare(tde)
    cfg = syn.CONFIGS["c2"]
    rb = tde.round_buffer((cfg.voxels,) * 3, (cfg.volume_m,) * 3, (100, 7, 300))
    ti = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    need = L.tde_integrate_tsdf_scratch_bytes(cfg.cols, cfg.rows, C.byref(rb))
    assert 0 < need <= L.tde_integrate_tsdf_noalloc_max_scratch_bytes()
    scene = syn.make_scene(cfg, 1000)
    traj = syn.make_trajectory(cfg, 2000, 2)
    oi = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    ref = tde.new_volume(cfg.tsdf_format, rb)
    out = tde.new_volume(cfg.tsdf_format, rb)
    cell = (np.float32(cfg.volume_m) / np.float32(cfg.voxels),) * 3
    for i in range(2):
        depth = orc.apply_noise(orc.render_depth(scene, traj[i], oi), 3000, i)
        sd = tde.scale_depth(torch.from_numpy(depth).to(cuda), ti)
        R = traj[i, :9].reshape(3, 3).astype(np.float32)
        t = traj[i, 9:].astype(np.float32)
        tde.integrate_tsdf(sd, ref, cfg.tsdf_format, cfg.trunc_m, R.T.copy(), t, ti, cell, rb, cfg.max_weight)
        Ri, tt, cs = tde.mat3(R.T.copy()), tde.vec3(t), tde.vec3(cell)
        tde.check(L.tde_integrate_tsdf_noalloc(sd.data_ptr(), out.data_ptr(), cfg.tsdf_format, cfg.trunc_m,
                                               C.byref(Ri), C.byref(tt), C.byref(ti), C.byref(cs), C.byref(rb),
                                               cfg.max_weight, tde.stream_ptr()))
        torch.cuda.synchronize()
        assert torch.equal(out, ref), f"call {i + 1}: volume differs from tde_integrate_tsdf"
    assert (ref.view(torch.int16)[1::2] != 0).sum() > 100000  # weights written
    del ref, out
    torch.cuda.empty_cache()


def test_noalloc_rejects_configurations_beyond_its_array(tde, cuda):
    L = _declare(tde)
    assert L.tde_integrate_tsdf_noalloc_max_scratch_bytes() == 3 << 19
    rb = tde.round_buffer((1024, 1024, 1024), (4.0, 4.0, 4.0))
    ti = tde.Intrinsics(525.0, 525.0, 319.5, 239.5, 640, 480)
    R, t, cs = tde.mat3(np.eye(3)), tde.vec3((0, 0, 0)), tde.vec3((4 / 1024,) * 3)
    rc = L.tde_integrate_tsdf_noalloc(None, None, 1, 0.03, C.byref(R), C.byref(t), C.byref(ti), C.byref(cs),
                                      C.byref(rb), 128, None)
    assert rc == -5
    assert "scratch" in tde.last_error()
