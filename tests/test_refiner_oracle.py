"""CPU checks of the refiner oracle (oracle/unet.py): its backward pass
against central finite differences in FP64, its bf16 rounding, and the
library's parameter count."""
import numpy as np
import pytest

from oracle import unet as U


def _batch(seed, n=2, h=16, w=24):
    rng = np.random.default_rng(seed)
    raw = rng.uniform(500, 3000, (n, h, w)).astype(np.uint16)
    raw[rng.random(raw.shape) < 0.05] = 0
    tgt = np.clip(raw.astype(np.int32) + rng.integers(-6, 7, raw.shape), 0, 65535).astype(np.uint16)
    tgt[rng.random(raw.shape) < 0.05] = 0
    return raw, tgt


def test_backward_matches_finite_differences():
    raw, tgt = _batch(0)
    th = U.init_params(1)
    d = U.unflatten(th)
    d["head.w"] = np.random.default_rng(2).normal(0.0, 0.05, 16)  # every layer gets a gradient
    th = U.flatten(d)
    _, g, _ = U.loss_and_grad(th, raw, tgt, emulate_bf16=False)
    rng = np.random.default_rng(1)
    o = 0
    for name, shape in U.param_layout():
        n = int(np.prod(shape))
        for i in (o + rng.integers(n, size=2)):
            e = np.zeros_like(th)
            e[i] = 1e-6
            lp, _, _ = U.loss_and_grad(th + e, raw, tgt, emulate_bf16=False)
            lm, _, _ = U.loss_and_grad(th - e, raw, tgt, emulate_bf16=False)
            fd = (lp - lm) / 2e-6
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 2e-4 * abs(g[i]) + 1e-12, (name, fd, g[i])
        o += n


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-3], np.float64)
    r = U.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 1e-3) <= 1e-3 * 2 ** -8


def test_param_count_matches_library(tde):
    import importlib
    rf = importlib.import_module("3deye_gb300.refiner")
    assert rf.param_count() == U.param_count() == 194401


def test_invalid_shapes_are_rejected(tde):
    import ctypes as C
    import importlib
    importlib.import_module("3deye_gb300.refiner")  # declares the signatures
    cap = importlib.import_module("3deye_gb300._capi")
    h = C.c_void_p()
    # argument checks run before any device call
    assert cap.lib.tde_refiner_create(1, 30, 64, 0, C.byref(h)) == cap.TDE_ERR_INVALID_ARG
    assert cap.lib.tde_refiner_create(0, 32, 64, 0, C.byref(h)) == cap.TDE_ERR_INVALID_ARG
