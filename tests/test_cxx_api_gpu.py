"""The reference-compatible C++ API (include/3deye/) exercised by a C++ caller
(tests/cxx/api_roundtrip.cpp) and compared with the CPU oracle."""
import importlib
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu
syn = importlib.import_module("3deye_gb300.synth")
IDENT12 = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)


def build_caller(tmp_path):
    exe = tmp_path / "api_roundtrip"
    lib = ROOT / "3deye_gb300"
    cxx = shutil.which("g++") or "g++"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include" / "3deye"), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cxx" / "api_roundtrip.cpp"), "-L", str(lib), "-l3deye_gb300",
                    f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    return exe


def bits_equal(a, b):
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


@pytest.mark.parametrize("fmt", [0, 1])
def test_cxx_api_roundtrip_matches_oracle(cuda, orc, tmp_path, fmt):
    cfg = syn.small_config("c1", frames=3, cols=160, rows=120, voxels=64, fmt=fmt)
    scene = syn.make_scene(cfg, 1000)
    traj = syn.make_trajectory(cfg, 2000)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    d0 = orc.apply_noise(orc.render_depth(scene, traj[0], intr), 3000, 0)
    d1 = orc.apply_noise(orc.render_depth(scene, traj[2], intr), 3000, 2)
    W, H, N = cfg.cols, cfg.rows, cfg.voxels
    bounds = np.array([20, -1000, -1000, 27, -1001, -1001], np.int32)
    with open(tmp_path / "input.bin", "wb") as f:
        np.array([W, H, N, 0, fmt], np.int32).tofile(f)
        np.array([cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.volume_m, cfg.trunc_m, cfg.dist_thresh, cfg.angle_thresh],
                 np.float32).tofile(f)
        traj[0].astype(np.float32).tofile(f)
        traj[1].astype(np.float32).tofile(f)
        d0.tofile(f)
        d1.tofile(f)
        bounds.tofile(f)
    exe = build_caller(tmp_path)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = (tmp_path / "output.bin").read_bytes()
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype, n, off)
        off += a.nbytes
        return a

    vm, nm = take(np.float32, W * H * 3).reshape(H, W, 3), take(np.float32, W * H * 3).reshape(H, W, 3)
    vm1, nm1 = take(np.float32, W * H * 3 // 4).reshape(H // 2, W // 2, 3), take(np.float32, W * H * 3 // 4).reshape(
        H // 2, W // 2, 3)
    A, b = take(np.float64, 36).reshape(6, 6), take(np.float64, 6)
    n = int(take(np.uint32, 1)[0])
    pts = take(np.float32, 4 * n).reshape(n, 4)
    rb = orc.make_rb((N,) * 3, (cfg.volume_m,) * 3)
    vol_bytes = orc.volume_bytes(fmt, rb)
    vol_after = take(np.uint8, vol_bytes)
    vc, nc = take(np.float32, W * H * 3).reshape(H, W, 3), take(np.float32, W * H * 3).reshape(H, W, 3)
    nw = int(take(np.uint32, 1)[0])
    whole = take(np.float32, 4 * nw).reshape(nw, 4)
    wcols = take(np.uint8, 4 * nw).reshape(nw, 4)
    img = take(np.uint8, W * H * 3).reshape(H, W, 3)
    ncs = int(take(np.uint32, 1)[0])
    cslab = take(np.uint8, 4 * ncs).reshape(ncs, 4)

    # oracle
    R = traj[0, :9].reshape(3, 3).astype(np.float32)
    t = traj[0, 9:].astype(np.float32)
    cell = np.full(3, cfg.volume_m / N, np.float32)
    vol = np.zeros(vol_bytes, np.uint8)
    orc.integrate(orc.scale_depth(d0, intr), vol, fmt, cfg.trunc_m, np.ascontiguousarray(R.T), t, intr, cell, rb)
    vmo, nmo = orc.raycast(vol, fmt, rb, intr, R, t, cfg.trunc_m, cell)
    assert bits_equal(vm, vmo) and bits_equal(nm, nmo)
    assert bits_equal(vm1, orc.resize_map(vmo, False)) and bits_equal(nm1, orc.resize_map(nmo, True))
    po, _, _, no = orc.extract_slice(vol, fmt, None, bounds[:3], bounds[3:], rb)
    assert n == no and n > 0 and np.array_equal(pts, po)
    # Extract_Tsdf_Volume, Extract_Color_Volume (the caller's colour pattern), Generate_Image
    wo, _, nwo = orc.extract_tsdf_volume(vol, fmt, rb, cell)
    assert nw == nwo and nw > 100 and bits_equal(whole, wo)
    i = np.arange(N ** 3, dtype=np.uint64)
    colour = np.stack([(i * 7) % 256, (i * 13) % 256, (i * 29) % 256, np.where(i % 5 == 0, 0, 200)],
                      axis=1).astype(np.uint8)
    assert np.array_equal(wcols, orc.extract_color_volume(colour, rb, wo, cell))
    # Extract_Color_Slice appends to the caller's one-entry cloud
    cso = orc.extract_color_slice(colour, bounds[:3], bounds[3:], rb)
    assert ncs == 1 + len(cso) and len(cso) > 100
    assert np.array_equal(cslab[0], [1, 2, 3, 4]) and np.array_equal(cslab[1:], cso)
    assert np.array_equal(img, orc.generate_image(vmo, nmo, t))
    orc.clean_tsdf_slice(vol, fmt, bounds[:3], bounds[3:], rb)
    assert np.array_equal(vol_after, vol)
    # Estimate_Combined: the oracle's FP64 sums on the caller's own maps
    R2 = traj[1, :9].reshape(3, 3).astype(np.float32)
    t2 = traj[1, 9:].astype(np.float32)
    pose = np.concatenate([R2.ravel(), t2, R.T.ravel(), t]).astype(np.float32)
    sums, _ = orc.icp_terms(vc, nc, vmo, nmo, pose, intr, cfg.dist_thresh, cfg.angle_thresh)
    assert sums[27] > 500
    k = 0
    for i in range(6):
        for j in range(i, 7):
            got = b[i] if j == 6 else A[i, j]
            assert abs(got - sums[k]) <= 1e-6 * max(1.0, abs(sums).max()), (i, j, got, sums[k])
            if j < 6:
                assert A[j, i] == A[i, j]
            k += 1


def test_cxx_rgbd_odometry_matches_oracle(cuda, orc, tmp_path):
    """Prepare_Data_For_RGBD .. Estimate_Isometry_By_RGBD called from C++
    (tests/cxx/rgbd_roundtrip.cpp) against the oracle on a rendered pair."""
    cfg = syn.small_config("c1", frames=3, cols=320, rows=240)
    scene = syn.make_scene(cfg, 7)
    traj = syn.make_trajectory(cfg, 7)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    W, H, L = cfg.cols, cfg.rows, 3
    frames = []
    with open(tmp_path / "rgbd_in.bin", "wb") as f:
        np.array([W, H, L], np.int32).tofile(f)
        np.array([cfg.fx, cfg.fy, cfg.cx, cfg.cy, 0.07], np.float32).tofile(f)
        for k in (0, 1):
            mm = np.rint(orc.render_depth(scene, traj[k], intr) * 1000).astype(np.uint16)
            rgb = orc.render_rgb(scene, traj[k], intr)
            mm.tofile(f)
            rgb.tofile(f)
            frames.append(orc.rgbd_levels(mm, rgb, L))
    src = ROOT / "tests" / "cxx" / "rgbd_roundtrip.cpp"
    exe = tmp_path / "rgbd_roundtrip"
    lib = ROOT / "3deye_gb300"
    subprocess.run([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I", str(ROOT / "include" / "3deye"), "-I",
                    str(ROOT / "include"), str(src), "-L", str(lib), "-l3deye_gb300", f"-Wl,-rpath,{lib}", "-o",
                    str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = (tmp_path / "rgbd_out.bin").read_bytes()
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype, n, off)
        off += a.nbytes
        return a
    for l in range(L):
        m = (W >> l) * (H >> l)
        i8, dm, gx, gy = take(np.uint8, m), take(np.float32, m), take(np.int16, m), take(np.int16, m)
        assert np.array_equal(i8, frames[0][l][0].ravel()) and np.array_equal(dm, frames[0][l][1].ravel())
        assert np.array_equal(gx, frames[1][l][2].ravel()) and np.array_equal(gy, frames[1][l][3].ravel())
    npts = int(take(np.int32, 1)[0])
    pts = take(np.int32, 2 * npts).reshape(npts, 2)
    want = orc.rgbd_points(frames[1][0][2], frames[1][0][3], (10 / 0.125) ** 2)
    assert npts == len(want) > 1000 and np.array_equal(pts, want)
    # the identity pairs of those points, without a gradient test (the list is already filtered)
    ncorr, s2 = int(take(np.int32, 1)[0]), float(take(np.float32, 1)[0])
    diff = take(np.float32, npts)
    n_o, kept, res, s2_o = orc.rgbd_pairs(frames[0][0], frames[1][0], intr, IDENT12, 0.0)
    lin = pts[:, 1] * W + pts[:, 0]
    on = kept.ravel()[lin] > 0
    assert ncorr == int(on.sum()) > 500
    assert np.array_equal(diff[on], res.ravel()[lin][on]) and np.all(diff[~on] == 100.0)
    assert s2 == np.float32(np.sum(res.ravel()[lin][on].astype(np.float64) ** 2))
    ok = int(take(np.int32, 1)[0])
    R, t = take(np.float32, 9), take(np.float32, 3)
    pose_o, failed = orc.rgbd_odometry(frames[0], frames[1], intr, [7, 7, 7][:L], [10.0] * L)
    assert ok == 1 and failed == 0
    np.testing.assert_allclose(R, pose_o[:9], rtol=0, atol=2e-5)
    np.testing.assert_allclose(t, pose_o[9:], rtol=0, atol=5e-5)
