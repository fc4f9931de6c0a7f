"""Dense RGB-D odometry on the GPU (3deye_gb300/csrc/k_rgbd.cu through the
C-ABI) against the CPU oracle (oracle/oracle_rgbd.c) on the same frames.

Integer stages (intensity, pyramid, Sobel derivatives, points of interest)
and the pair search (kept pairs, their pixels and residuals, count, sum of
squared residuals, sigma) are bit-exact: both sides evaluate the same IEEE
operations.  The 27 sums of [A | b] differ only by accumulation order
(FP32 per thread and warp, FP64 across warps and blocks on the GPU; FP64 per
pair on the CPU): 2e-5 of the largest diagonal term.  The odometry then
agrees with the oracle's to 0.05 mm and 0.002 degrees over the 31 steps.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

syn = importlib.import_module("3deye_gb300.synth")

IDENT = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)


def rel_pose(Tp, Tc):
    Rp, tp = Tp[:9].reshape(3, 3), Tp[9:]
    Rc, tc = Tc[:9].reshape(3, 3), Tc[9:]
    return np.concatenate([(Rc.T @ Rp).ravel(), Rc.T @ (tp - tc)])


def pose_error(a, b):
    Re = a[:9].reshape(3, 3) @ b[:9].reshape(3, 3).T
    ang = np.degrees(np.arccos(np.clip((np.trace(Re) - 1) / 2, -1, 1)))
    return float(np.linalg.norm(a[9:] - b[9:])), float(ang)


@pytest.fixture(scope="module")
def setup(cuda, orc, tde):
    import torch
    rg = importlib.import_module("3deye_gb300.rgbd")
    cfg = syn.CONFIGS["c2"]
    scene = syn.make_scene(cfg, 5)
    traj = syn.make_trajectory(cfg, 5, 12)
    intr_o = orc.Intr(*syn.intrinsics_tuple(cfg))
    intr = tde.Intrinsics(*syn.intrinsics_tuple(cfg))
    d_scene = torch.from_numpy(np.ascontiguousarray(scene, np.float64)).to(cuda)
    cpu, gpu = {}, {}
    for k in (0, 1, 10, 11):
        mm = np.rint(orc.render_depth(scene, traj[k], intr_o) * 1000).astype(np.uint16)
        rgb = orc.render_rgb(scene, traj[k], intr_o)
        cpu[k] = dict(mm=mm, rgb=rgb, levels=orc.rgbd_levels(mm, rgb, 4))
        g_rgb = torch.empty((cfg.rows, cfg.cols, 3), dtype=torch.uint8, device=cuda)
        rg.synth_rgb(d_scene, scene.shape[0], traj[k], intr, g_rgb)
        g_mm = torch.from_numpy(mm.view(np.int16)).to(cuda)
        gpu[k] = dict(rgb=g_rgb, frame=rg.RgbdFrame(cfg.cols, cfg.rows, 4, cuda).load(g_mm, g_rgb))
    torch.cuda.synchronize()
    return dict(rg=rg, cfg=cfg, traj=traj, intr=intr, intr_o=intr_o, cpu=cpu, gpu=gpu)


def test_synthetic_colour_camera_matches_oracle(setup):
    for k, c in setup["cpu"].items():
        np.testing.assert_array_equal(setup["gpu"][k]["rgb"].cpu().numpy(), c["rgb"])


def test_prepare_pyramid_derivatives_bit_exact(setup):
    for k, c in setup["cpu"].items():
        f = setup["gpu"][k]["frame"]
        for l, (I8, D, dx, dy) in enumerate(c["levels"]):
            np.testing.assert_array_equal(f.I[l].cpu().numpy(), I8)
            np.testing.assert_array_equal(f.D[l].cpu().numpy().view(np.uint32), D.view(np.uint32))
            np.testing.assert_array_equal(f.dx[l].cpu().numpy(), dx)
            np.testing.assert_array_equal(f.dy[l].cpu().numpy(), dy)


@pytest.mark.parametrize("scale", [0.0, (10 / 0.125) ** 2, 1e9])
def test_points_of_interest_match_oracle(setup, orc, scale):
    rg = setup["rg"]
    for l in (0, 2):
        f = setup["gpu"][0]["frame"]
        pts, n = rg.points_of_interest(f.dx[l], f.dy[l], scale)
        want = orc.rgbd_points(f.dx[l].cpu().numpy(), f.dy[l].cpu().numpy(), scale)
        assert n == len(want)
        np.testing.assert_array_equal(pts.cpu().numpy(), want)


@pytest.mark.parametrize("k,level", [(0, 0), (10, 1), (10, 3)])
def test_correspondences_bit_exact(setup, orc, k, level):
    rg = setup["rg"]
    gt = rel_pose(setup["traj"][k], setup["traj"][k + 1])
    pose = IDENT.copy()
    pose[:9] = (0.5 * (gt[:9].reshape(3, 3) + np.eye(3))).ravel()  # part way: residuals are non-zero
    u, s, vt = np.linalg.svd(pose[:9].reshape(3, 3))
    pose[:9] = (u @ vt).ravel()
    pose[9:] = 0.5 * gt[9:]
    prev, curr = setup["gpu"][k]["frame"], setup["gpu"][k + 1]["frame"]
    cp, cc, diff, n, s2 = rg.correspondences(prev, curr, level, pose, setup["intr"])
    P, Cc = setup["cpu"][k]["levels"][level], setup["cpu"][k + 1]["levels"][level]
    n_o, kept, res, s2_o = orc.rgbd_pairs(P, Cc, setup["intr_o"].level(level), pose, 10.0)
    assert n == n_o and s2 == s2_o
    H, W = kept.shape
    kept = kept.ravel()
    on = kept > 0
    cp, cc, diff = cp.cpu().numpy(), cc.cpu().numpy(), diff.cpu().numpy()
    idx = np.arange(H * W)
    np.testing.assert_array_equal(cp[on], np.stack([idx[on] % W, idx[on] // W], 1))
    np.testing.assert_array_equal(cc[on], np.stack([(kept[on] - 1) % W, (kept[on] - 1) // W], 1))
    np.testing.assert_array_equal(diff[on], res.ravel()[on])
    assert np.all(diff[~on] == 100.0) and not cp[~on].any() and not cc[~on].any()
    # the list form over the points of interest of the previous frame's grid
    pts, npts = rg.points_of_interest(curr.dx[level], curr.dy[level], 0.0)
    assert npts == H * W
    cp2, cc2, diff2, n2, s22 = rg.correspondences(prev, curr, level, pose, setup["intr"], points=pts)
    assert n2 == n and s22 == s2
    np.testing.assert_array_equal(diff2.cpu().numpy(), diff)


@pytest.mark.parametrize("level", [0, 2])
def test_lsm_matches_oracle(setup, orc, level):
    rg = setup["rg"]
    k = 10
    gt = rel_pose(setup["traj"][k], setup["traj"][k + 1])
    pose = IDENT.copy()
    pose[9:] = 0.5 * gt[9:]
    prev, curr = setup["gpu"][k]["frame"], setup["gpu"][k + 1]["frame"]
    sums, sigma = rg.lsm(prev, curr, level, pose, setup["intr"])
    P, Cc = setup["cpu"][k]["levels"][level], setup["cpu"][k + 1]["levels"][level]
    sums_o, sigma_o = orc.rgbd_lsm(P, Cc, setup["intr_o"].level(level), pose, 10.0)
    assert sigma == sigma_o and sums[27] == sums_o[27] > 100
    diag = sums_o[[0, 7, 13, 18, 22, 25]].max()
    np.testing.assert_allclose(sums, sums_o, rtol=0, atol=2e-5 * diag)


@pytest.mark.parametrize("k", [0, 10])
def test_odometry_matches_oracle_and_ground_truth(setup, orc, k):
    rg = setup["rg"]
    od = rg.RgbdOdometry(setup["intr"])
    pose, status = od.estimate(setup["gpu"][k]["frame"], setup["gpu"][k + 1]["frame"])
    assert status == rg.STATUS_SOLVED
    pose_o, failed = orc.rgbd_odometry(setup["cpu"][k]["levels"], setup["cpu"][k + 1]["levels"], setup["intr_o"],
                                       [7, 7, 7, 10], [10.0] * 4)
    assert failed == 0
    et, er = pose_error(pose, pose_o)
    assert et < 5e-5 and er < 2e-3, (et, er)
    gt = rel_pose(setup["traj"][k], setup["traj"][k + 1])
    et, er = pose_error(pose, gt)
    assert et < 3e-3 and er < 0.1, (et, er)
    # from an initial estimate: the first step of a one-level run equals the oracle's
    p1 = rg.default_params(1)
    p1.iters[0] = 1
    od1 = rg.RgbdOdometry(setup["intr"], p1)
    init = IDENT.copy()
    init[9:] = gt[9:] * 0.8
    pose1, st1 = od1.estimate(setup["gpu"][k]["frame"], setup["gpu"][k + 1]["frame"], init)
    pose1_o, f1 = orc.rgbd_odometry(setup["cpu"][k]["levels"][:1], setup["cpu"][k + 1]["levels"][:1],
                                    setup["intr_o"], [1], [10.0], init_pose12=init)
    assert st1 == rg.STATUS_SOLVED and f1 == 0
    np.testing.assert_allclose(pose1, pose1_o, rtol=0, atol=1e-7)


def test_odometry_without_texture_reports_failed_solves(cuda, tde):
    import torch
    rg = importlib.import_module("3deye_gb300.rgbd")
    H, W = 96, 128
    intr = tde.Intrinsics(100.0, 100.0, 63.5, 47.5, W, H)
    mm = torch.full((H, W), 1500, dtype=torch.int16, device=cuda)
    rgb = torch.full((H, W, 3), 120, dtype=torch.uint8, device=cuda)
    f = rg.RgbdFrame(W, H, 3, cuda).load(mm, rgb)
    od = rg.RgbdOdometry(intr, rg.default_params(3))
    init = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0.01, -0.02, 0.005], np.float64)
    pose, status = od.estimate(f, f, init)
    assert status == rg.STATUS_SOLVE_FAILED
    np.testing.assert_array_equal(pose, init)
