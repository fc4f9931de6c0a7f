"""The CPU restatement of the dense RGB-D odometry (oracle/oracle_rgbd.c)
against the reference's own kernel and against known answers.

compute_least_squares_equation.cl (the per-correspondence coefficients) is
the one kernel of the path the reference ships that runs as written; its
outputs for seeded inputs, computed by the kernel compiled as C
(tests/golden/make_golden.py, gen_lsm), pin the oracle's row.  The other
stages' kernels are absent or broken (x and y both from get_global_id(0),
unsigned derivatives, an inverted depth test), so the oracle's preparation,
pyramid, derivatives and points are pinned to independent numpy statements
of the published method, and the whole odometry to a known rigid motion of
a rendered textured scene.
"""
import ctypes as C
import importlib

import numpy as np
import pytest

from conftest import GOLDEN

syn = importlib.import_module("3deye_gb300.synth")


def rel_pose(Tp, Tc):
    """Camera-to-world poses of two frames -> the pose mapping previous-frame
    camera points to current-frame ones."""
    Rp, tp = Tp[:9].reshape(3, 3), Tp[9:]
    Rc, tc = Tc[:9].reshape(3, 3), Tc[9:]
    return np.concatenate([(Rc.T @ Rp).ravel(), Rc.T @ (tp - tc)])


def pose_error(a, b):
    """(translation error in m, rotation error in degrees)."""
    Re = a[:9].reshape(3, 3) @ b[:9].reshape(3, 3).T
    ang = np.degrees(np.arccos(np.clip((np.trace(Re) - 1) / 2, -1, 1)))
    return float(np.linalg.norm(a[9:] - b[9:])), float(ang)


def test_row_pinned_to_reference_kernel(orc):
    g = np.load(GOLDEN / "rgbd_lsm.npz")
    fx, fy, cx, cy, W, H = g["intr"]
    intr = orc.Intr(fx, fy, cx, cy, int(W), int(H))
    for k in range(len(g["u"])):
        Rt = np.concatenate([g["R"][k].ravel(), g["t"][k]]).astype(np.float32)
        row = orc.rgbd_row_single(int(g["u"][k]), int(g["v"][k]), float(g["z"][k]), Rt, intr, float(g["dx"][k]),
                                  float(g["dy"][k]), float(g["diff"][k]), float(g["sigma"][k]))
        Cref, vec = g["C"][k], g["vec"][k]
        # the reference evaluates without fused operations: a few ulps apart
        scale = np.abs(Cref).max()
        np.testing.assert_allclose(row[:6], Cref, rtol=0, atol=4e-7 * scale)
        # b's contribution: the reference's C * diff * w is -C * row[6]
        np.testing.assert_allclose(-row[:6] * row[6], vec, rtol=0, atol=4e-7 * np.abs(vec).max())


def test_prepare_pyramid_sobel_points_known(orc):
    rng = np.random.default_rng(3)
    H, W = 37, 52
    mm = rng.integers(0, 6000, (H, W)).astype(np.uint16)
    rgb = rng.integers(0, 256, (H, W, 3)).astype(np.uint8)
    I8, D = orc.rgbd_prepare(mm, rgb)
    r, g, b = (rgb[..., k].astype(np.int64) for k in range(3))
    np.testing.assert_array_equal(I8, ((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14).astype(np.uint8))
    np.testing.assert_array_equal(D, mm.astype(np.float32) * np.float32(0.001))
    I2, D2 = orc.rgbd_pyramid(I8, D)
    a = I8[: H // 2 * 2, : W // 2 * 2].astype(np.int64)
    np.testing.assert_array_equal(I2, ((a[0::2, 0::2] + a[0::2, 1::2] + a[1::2, 0::2] + a[1::2, 1::2] + 2) >> 2))
    np.testing.assert_array_equal(D2, D[0:H // 2 * 2:2, 0:W // 2 * 2:2])
    dx, dy = orc.rgbd_sobel(I8)
    p = I8.astype(np.int64)
    ex = np.zeros((H, W), np.int64)
    ey = np.zeros((H, W), np.int64)
    ex[1:-1, 1:-1] = (p[:-2, 2:] + 2 * p[1:-1, 2:] + p[2:, 2:]) - (p[:-2, :-2] + 2 * p[1:-1, :-2] + p[2:, :-2])
    ey[1:-1, 1:-1] = (p[2:, :-2] + 2 * p[2:, 1:-1] + p[2:, 2:]) - (p[:-2, :-2] + 2 * p[:-2, 1:-1] + p[:-2, 2:])
    np.testing.assert_array_equal(dx, ex)
    np.testing.assert_array_equal(dy, ey)
    scale = (10 / 0.125) ** 2
    pts = orc.rgbd_points(dx, dy, scale)
    ys, xs = np.nonzero((ex * ex + ey * ey).astype(np.float32) >= np.float32(scale))
    np.testing.assert_array_equal(pts, np.stack([xs, ys], 1))


@pytest.fixture(scope="module")
def scene_frames(orc):
    cfg = syn.CONFIGS["c2"]
    scene = syn.make_scene(cfg, 5)
    traj = syn.make_trajectory(cfg, 5, 12)
    intr = orc.Intr(*syn.intrinsics_tuple(cfg))

    def frame(T):
        mm = np.rint(orc.render_depth(scene, T, intr) * 1000).astype(np.uint16)
        return orc.rgbd_levels(mm, orc.render_rgb(scene, T, intr), 4)
    frames = {k: frame(traj[k]) for k in (0, 1, 10, 11)}
    return cfg, scene, traj, intr, frames


def test_identity_pairs_have_zero_residual(orc, scene_frames):
    _, _, _, intr, frames = scene_frames
    f = frames[0][0]
    I = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)
    n, kept, res, s = orc.rgbd_pairs(f, f, intr, I, 10.0)
    # every pixel with valid depth and enough gradient pairs with itself
    g2 = f[2].astype(np.int64) ** 2 + f[3].astype(np.int64) ** 2
    want = (f[1] > 0) & (f[1] < 35) & (g2.astype(np.float32) >= np.float32((10 / 0.125) ** 2))
    assert n == int(want.sum()) > 10000
    idx = np.arange(f[1].size).reshape(f[1].shape) + 1
    np.testing.assert_array_equal(kept, np.where(want, idx, 0))
    assert s == 0.0 and not res.any()
    sums, sigma = orc.rgbd_lsm(f, f, intr, I, 10.0)
    assert sigma == 0.0 and sums[27] == n
    assert np.all(sums[[6, 12, 17, 21, 24, 26]] == 0)  # b = -sum w r C = 0


@pytest.mark.parametrize("k", [0, 10])
def test_odometry_recovers_known_motion(orc, scene_frames, k):
    _, _, traj, intr, frames = scene_frames
    gt = rel_pose(traj[k], traj[k + 1])
    step_t, step_r = pose_error(gt, np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64))
    pose, failed = orc.rgbd_odometry(frames[k], frames[k + 1], intr, [7, 7, 7, 10], [10.0] * 4)
    assert failed == 0
    et, er = pose_error(pose, gt)
    # a 13 mm / 0.46 degree step, recovered to within a fifth of it
    assert step_t > 0.01 and step_r > 0.3
    assert et < 3e-3 and et < 0.2 * step_t, (et, step_t)
    assert er < 0.1 and er < 0.2 * step_r, (er, step_r)


def test_odometry_without_texture_keeps_pose(orc):
    H, W = 96, 128
    mm = np.full((H, W), 1500, np.uint16)
    rgb = np.full((H, W, 3), 120, np.uint8)
    lv = orc.rgbd_levels(mm, rgb, 3)
    intr = orc.Intr(100.0, 100.0, 63.5, 47.5, W, H)
    init = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0.01, -0.02, 0.005], np.float64)
    pose, failed = orc.rgbd_odometry(lv, lv, intr, [2, 2, 2], [10.0] * 3, init_pose12=init)
    assert failed == 6
    np.testing.assert_array_equal(pose, init)


def test_rgbd_c_abi_refuses_bad_arguments(tde):
    """Host-side refusals of the odometry entry point (no device work)."""
    rg = importlib.import_module("3deye_gb300.rgbd")
    lib = tde._capi.lib
    intr = tde._capi.Intrinsics(525.0, 525.0, 319.5, 239.5, 640, 480)
    p = rg.default_params()
    frame = rg.RgbdFrameC()
    scratch = C.c_void_p(0x1000)
    nb = lib.tde_rgbd_odometry_scratch_bytes(640, 480)
    assert nb > 0 and nb % 256 == 0
    # a missing level buffer
    rc = lib.tde_rgbd_odometry(C.byref(frame), C.byref(frame), C.byref(intr), C.byref(p), None, C.c_void_p(0x100),
                               C.c_void_p(0x200), scratch, nb, None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG
    assert "missing" in tde._capi.last_error()
    # five levels
    p.levels = 5
    rc = lib.tde_rgbd_odometry(C.byref(frame), C.byref(frame), C.byref(intr), C.byref(p), None, C.c_void_p(0x100),
                               C.c_void_p(0x200), scratch, nb, None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG
    # every level present, but iterations out of range / scratch too small
    p.levels = 2
    bufs = [C.c_void_p(0x1000 + 0x100 * k) for k in range(8)]
    for l in range(2):
        frame.intensity[l], frame.depth[l], frame.dx[l], frame.dy[l] = bufs[4 * l: 4 * l + 4]
    p.iters[1] = 101
    rc = lib.tde_rgbd_odometry(C.byref(frame), C.byref(frame), C.byref(intr), C.byref(p), None, C.c_void_p(0x100),
                               C.c_void_p(0x200), scratch, nb, None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG and "iters" in tde._capi.last_error()
    p.iters[1] = 7
    rc = lib.tde_rgbd_odometry(C.byref(frame), C.byref(frame), C.byref(intr), C.byref(p), None, C.c_void_p(0x100),
                               C.c_void_p(0x200), scratch, nb - 256, None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG and "scratch" in tde._capi.last_error()
    # a frame too small for its levels
    small = tde._capi.Intrinsics(50.0, 50.0, 7.5, 5.5, 16, 12)
    p.levels = 3
    rc = lib.tde_rgbd_odometry(C.byref(frame), C.byref(frame), C.byref(small), C.byref(p), None, C.c_void_p(0x100),
                               C.c_void_p(0x200), scratch, nb, None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG
    # the stage entry points refuse null buffers and sizes before any device work
    assert lib.tde_rgbd_prepare(None, None, 640, 480, None, None, None) == tde._capi.TDE_ERR_INVALID_ARG
    assert lib.tde_rgbd_pyramid(C.c_void_p(1), C.c_void_p(2), 1, 480, C.c_void_p(3), C.c_void_p(4), None) == \
        tde._capi.TDE_ERR_INVALID_ARG
    assert lib.tde_rgbd_derivatives(None, 640, 480, C.c_void_p(1), C.c_void_p(2), None) == tde._capi.TDE_ERR_INVALID_ARG
    assert lib.tde_rgbd_points_scratch_bytes(0, 480) == 0 and lib.tde_rgbd_odometry_scratch_bytes(640, 0) == 0
    pts_sb = lib.tde_rgbd_points_scratch_bytes(640, 480)
    assert pts_sb >= 480 * 4 and pts_sb % 256 == 0
    rc = lib.tde_rgbd_points_of_interest(C.c_void_p(1), C.c_void_p(2), 640, 480, 1.0, scratch, pts_sb - 256,
                                         C.c_void_p(3), 10, C.c_void_p(4), None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG and "scratch" in tde._capi.last_error()
    proj = (C.c_float * 12)()
    rc = lib.tde_rgbd_correspondences(C.c_void_p(1), C.c_void_p(2), C.c_void_p(3), C.c_void_p(4), C.c_void_p(5),
                                      None, 640, 480, None, 0, proj, 0.07, 35.0, 10.0, C.c_void_p(6), C.c_void_p(7),
                                      C.c_void_p(8), C.c_void_p(9), C.c_void_p(10), None)
    assert rc == tde._capi.TDE_ERR_INVALID_ARG  # dx without dy
    d = rg.default_params()
    assert d.levels == 4 and list(d.iters) == [7, 7, 7, 10] and list(d.min_gradient) == [10.0] * 4
    assert abs(d.max_depth_diff - 0.07) < 1e-7 and d.max_depth == 35.0
    # the projective form on the host, against the oracle's
    from oracle import oracle as orc
    pose = np.array([0.99, -0.1, 0.05, 0.1, 0.99, 0.02, -0.05, -0.02, 0.998, 0.1, -0.05, 0.02])
    got = rg.projective(pose, intr)
    want = np.zeros(12, np.float32)
    orc.lib.or_rgbd_projective(orc._p(pose[:9].copy()), orc._p(pose[9:].copy()), C.byref(orc.Intr(525.0, 525.0,
                               319.5, 239.5, 640, 480)), orc._p(want))
    np.testing.assert_array_equal(got, want)
