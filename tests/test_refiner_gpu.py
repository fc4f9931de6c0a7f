"""The learned depth refiner on the GPU (tcgen05 convolutions, weight
gradients, routing kernels, AdamW) against the FP64 CPU oracle of the same
network (oracle/unet.py, bf16 rounding emulated at the GPU's storage points).

Tolerances: bf16 storage rounds to 8 significant bits (relative step 2^-8 to
2^-7); the GPU accumulates in FP32 and the oracle in FP64, so an element whose
FP32 and FP64 sums straddle a bf16 rounding boundary differs by one bf16 step.
Activations: every element within 2% of the tensor's largest magnitude and
99% within one bf16 step (2^-7 relative + 1e-3 of the largest magnitude).
Gradients: per parameter block, |g_gpu - g_ref| <= 3e-2 |g_ref| (2-norm) and
cosine similarity >= 0.999.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, H, W = 2, 24, 160  # 160 px rows: one full and one partial 128-pixel tile


def make_batch(seed, n=N, h=H, w=W):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    out, tgt = [], []
    for _ in range(n):
        a, b, c = rng.uniform(-0.004, 0.004, 3)
        base = 1.6 + a * xx + b * yy + 0.2 * np.sin(xx / (7 + 10 * abs(c) * 1e3)) * np.cos(yy / 9.0)
        gt = np.round(base * 1000.0)
        noisy = gt + rng.normal(0.0, 4.0, gt.shape)
        raw = np.clip(np.round(noisy), 0, 32767)
        raw[rng.random(gt.shape) < 0.04] = 0
        t = gt.copy()
        t[rng.random(gt.shape) < 0.03] = 0
        out.append(raw)
        tgt.append(t)
    return np.array(out, np.uint16), np.array(tgt, np.uint16)


@pytest.fixture(scope="module")
def U():
    from oracle import unet
    return unet


@pytest.fixture(scope="module")
def rf():
    return importlib.import_module("3deye_gb300.refiner")


def close_bf16(name, g, r):
    scale = float(np.abs(r).max()) + 1e-30
    d = np.abs(g - r)
    step = np.abs(r) * 2.0 ** -7 + 1e-3 * scale
    frac_bad = float((d > step).mean())
    assert d.max() <= 0.02 * scale, (name, float(d.max()), scale)
    assert frac_bad <= 1e-2, (name, frac_bad)


def test_forward_matches_oracle_layer_by_layer(cuda, U, rf):
    raw, _ = make_batch(1)
    R = rf.Refiner(N, H, W, seed=7)
    d = U.unflatten(R.get_params())
    d["head.w"] = np.random.default_rng(1).normal(0, 0.2, 16)  # a residual of a few mm
    theta = U.f32(U.flatten(d)).astype(np.float32)
    R.set_params(theta)
    out_mm, out_m = R.forward(raw)
    assert R.status() == 0
    _, (A, _, _) = U.forward(theta.astype(np.float64), raw)
    for name in rf.ACTIVATIONS:
        close_bf16(name, R.tensor(name), A[name])
    ref = A["out"]
    valid = raw > 0
    assert np.all(out_m[~valid] == 0)
    # the head on the GPU's own d0 (FP32 on the GPU, FP64 here)
    d0 = R.tensor("d0")
    head = np.where(valid, A["depth"] + 0.01 * (d0 @ d["head.w"] + d["head.b"][0]), 0.0)
    np.testing.assert_allclose(out_m, head, rtol=0, atol=2e-6)
    # and against the oracle: one bf16 step per channel of d0 bounds the difference
    bound = 0.01 * (np.abs(A["d0"]) @ np.abs(d["head.w"])) * 2.0 ** -6 + 2e-6
    assert np.all(np.abs(out_m - ref) <= bound)
    exp_mm = np.clip(np.rint(out_m * 1000.0), 0, 32767).astype(np.uint16)
    assert np.array_equal(out_mm, exp_mm)
    R.close()


def test_gradients_match_oracle(cuda, U, rf):
    raw, tgt = make_batch(2)
    R = rf.Refiner(N, H, W, seed=11)
    theta = R.get_params().astype(np.float64)
    # a larger head so that every layer receives a sizeable gradient
    d = U.unflatten(theta)
    d["head.w"] = np.random.default_rng(0).normal(0, 0.05, 16)
    theta = U.f32(U.flatten(d))
    R.set_params(theta.astype(np.float32))
    loss_g, g = R.loss_grad(raw, tgt)
    assert R.status() == 0
    loss_r, gr, _ = U.loss_and_grad(theta, raw, tgt)
    assert abs(loss_g - loss_r) <= 1e-4 * loss_r
    o = 0
    for name, shape in U.param_layout():
        n = int(np.prod(shape))
        a, b = g[o:o + n].astype(np.float64), gr[o:o + n]
        o += n
        nb = np.linalg.norm(b)
        assert nb > 0, name
        assert np.linalg.norm(a - b) <= 3e-2 * nb, (name, np.linalg.norm(a - b) / nb)
        assert a @ b / (np.linalg.norm(a) * nb) >= 0.999, name
    R.close()


def test_adamw_step_matches_oracle(cuda, U, rf):
    import torch
    raw, tgt = make_batch(3)
    R = rf.Refiner(N, H, W, seed=5)
    theta = R.get_params()
    _, g = R.loss_grad(raw, tgt)
    R.set_params(theta)
    r = torch.from_numpy(raw.view(np.int16)).cuda()
    t = torch.from_numpy(tgt.view(np.int16)).cuda()
    R.train_step_ptr(r.data_ptr(), t.data_ptr(), N, 1e-3)
    after = R.get_params()
    exp, _, _ = U.adamw(theta, g, np.zeros_like(theta), np.zeros_like(theta), 1, 1e-3)
    np.testing.assert_allclose(after, exp, rtol=1e-6, atol=1e-9)
    R.close()


def test_training_reduces_error_against_ground_truth(cuda, rf):
    """500 AdamW steps on noisy synthetic depth: the refined depth
    ends closer to the noise-free depth than the raw input is."""
    import torch
    h, w, n = 48, 64, 8
    R = rf.Refiner(n, h, w, seed=3)
    first = last = None
    for it in range(500):
        raw, gt = make_batch(100 + it, n, h, w)
        r = torch.from_numpy(raw.view(np.int16)).cuda()
        t = torch.from_numpy(gt.view(np.int16)).cuda()
        R.train_step_ptr(r.data_ptr(), t.data_ptr(), n, 2e-3)
        if it == 0:
            first = R.last_loss()
    last = R.last_loss()
    assert R.status() == 0
    assert last[0] < 0.75 * first[0], (first, last)
    raw, gt = make_batch(999, n, h, w)
    _, out_m = R.forward(raw)
    m = (raw > 0) & (gt > 0)
    err_raw = np.abs(raw[m] / 1000.0 - gt[m] / 1000.0).mean()
    err_ref = np.abs(out_m[m] - gt[m] / 1000.0).mean()
    assert err_ref < 0.8 * err_raw, (err_ref, err_raw)
    R.close()


def test_pipeline_with_identity_refiner(cuda, rf):
    """The refiner in place of the bilateral stage: an untrained refiner (zero
    head) is the identity on valid depth, so the pipeline's level-0 depth is
    the raw frame, tracking still follows the ground truth, and the frame
    runs 11 more kernels (the refiner's convolutions and the vertex map
    instead of the fused bilateral kernel)."""
    import ctypes as C
    from oracle import oracle as orc
    tde = importlib.import_module("3deye_gb300")
    syn = importlib.import_module("3deye_gb300.synth")
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg = syn.small_config("c1", frames=10, cols=160, rows=120, voxels=96, fmt=1)
    scene = syn.make_scene(cfg, 1000)
    traj = syn.make_trajectory(cfg, 2000)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    depths = [orc.apply_noise(orc.render_depth(scene, traj[i], intr), 3000, i) for i in range(cfg.frames)]
    plain = pl.Pipeline(cfg, traj[0])
    n_plain = plain.launches_per_frame()
    plain.close()
    R = rf.Refiner(1, cfg.rows, cfg.cols, seed=1)
    p = pl.Pipeline(cfg, traj[0])
    p.set_refiner(R)
    assert p.launches_per_frame() == n_plain + 11
    poses = []
    for d in depths:
        pose, st = p.process(d)
        assert st == 0
        poses.append(pose)
        dptr, _, _ = p.frame_maps(0)
        got = np.zeros((cfg.rows, cfg.cols), np.uint16)
        tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        tde.check(tde.lib.tde_memcpy(got.ctypes.data_as(C.c_void_p), dptr, got.nbytes, 1))
        assert np.array_equal(got, d)
    assert pl.ate_rmse(np.array(poses), traj[:cfg.frames]) < 0.02
    assert R.status() == 0
    p.set_refiner(None)
    assert p.launches_per_frame() == n_plain
    p.close()
    R.close()
