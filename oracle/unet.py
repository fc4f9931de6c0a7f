"""CPU oracle for the learned depth refiner (numpy, FP64 arithmetic).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU
refiner (3deye_gb300/csrc/k_refiner.cu); never called by the product path.

The refiner has no counterpart in the reference: it is a new stage that
replaces the bilateral filter (compute_bilateral_filtering.cl:8-57,
opencl_wrappers.cpp:216-235) when enabled.  This module fixes its exact
semantics -- the layer list, the parameter layout, where the GPU rounds to
bf16, how gradients are routed through pooling, upsampling and skips -- and
computes the forward pass, the masked L1 loss and every parameter gradient.

With ``emulate_bf16=True`` values are rounded to bf16 (round to nearest even)
at the points where the GPU stores bf16 tensors; accumulation stays FP64, so
the remaining difference from the GPU is its FP32 accumulation.  With
``emulate_bf16=False`` everything is FP64, which is what the finite-difference
check of the backward pass uses.

Network (NHWC, H and W divisible by 8; 3x3 convolutions with zero padding):

    in   = per tap t of the 3x3 window around p, three channels:
           [100 (d(p+t) - d(p)) if both valid else 0, valid(p+t), d(p+t)]
    c1 : in            -> 16, ReLU   = e0a          L0 (CUDA cores, fp32)
    c2 : e0a           -> 16, ReLU   = e0           L0
    c3 : pool(e0)      -> 32, ReLU   = e1a          L1
    c4 : e1a           -> 32, ReLU   = e1           L1
    c5 : pool(e1)      -> 48, ReLU   = e2a          L2
    c6 : e2a           -> 48, ReLU   = e2           L2
    c7 : pool(e2)      -> 64, ReLU   = b3a          L3
    c8 : b3a           -> 64, ReLU   = b3           L3
    c9 : up(b3) | e2   -> 48, ReLU   = d2           L2 (112 input channels)
    c10: up(d2) | e1   -> 32, ReLU   = d1           L1 (80)
    c11: up(d1) | e0   -> 16, ReLU   = d0           L0 (48)
    head: r = w . d0 + b (1x1, fp32);  out = depth_m + 0.01 r where valid, else 0

The input is relative depth in centimetres: bf16 keeps 8 significant bits,
so absolute depth (~1-4 m) would lose the millimetre noise the network has
to see at the first bf16 store; differences to the centre pixel do not.

pool = 2x2 max (gradient to the first maximum in the order (0,0), (0,1),
(1,0), (1,1)); up = 2x nearest; "|" = channel concatenation.
Loss = sum over pixels valid in both input and target of |out - target|,
divided by N*H*W.
"""
from __future__ import annotations

import numpy as np

# (name, level, source A, channels A, mode A, source B, channels B, Cout)
DIRECT, POOL, UP = 0, 1, 2
CONVS = [
    ("c2", 0, "e0a", 16, DIRECT, None, 0, 16, "e0"),
    ("c3", 1, "e0", 16, POOL, None, 0, 32, "e1a"),
    ("c4", 1, "e1a", 32, DIRECT, None, 0, 32, "e1"),
    ("c5", 2, "e1", 32, POOL, None, 0, 48, "e2a"),
    ("c6", 2, "e2a", 48, DIRECT, None, 0, 48, "e2"),
    ("c7", 3, "e2", 48, POOL, None, 0, 64, "b3a"),
    ("c8", 3, "b3a", 64, DIRECT, None, 0, 64, "b3"),
    ("c9", 2, "b3", 64, UP, "e2", 48, 48, "d2"),
    ("c10", 1, "d2", 48, UP, "e1", 32, 32, "d1"),
    ("c11", 0, "d1", 32, UP, "e0", 16, 16, "d0"),
]
C1_IN, C1_OUT, HEAD_IN = 3, 16, 16
DEPTH_SCALE = np.float32(0.001)
DIFF_SCALE = 100.0      # input depth differences in cm
RESIDUAL_SCALE = 0.01   # head output in cm


def param_layout():
    """[(name, shape)] in the order of the flat fp32 parameter vector."""
    out = [("c1.w", (C1_OUT, 9, C1_IN)), ("c1.b", (C1_OUT,))]
    for name, _, _, ca, _, _, cb, co, _ in CONVS:
        out += [(name + ".w", (co, 9, ca + cb)), (name + ".b", (co,))]
    out += [("head.w", (HEAD_IN,)), ("head.b", (1,))]
    return out


def param_count() -> int:
    return int(sum(np.prod(s) for _, s in param_layout()))


def unflatten(theta: np.ndarray) -> dict:
    d, o = {}, 0
    for name, shape in param_layout():
        n = int(np.prod(shape))
        d[name] = np.asarray(theta[o:o + n], np.float64).reshape(shape)
        o += n
    return d


def flatten(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in param_layout()])


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bf16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def f32(x):
    return np.asarray(x, np.float32).astype(np.float64)


class _R:
    """Rounding policy: bf16/fp32 emulation or identity."""

    def __init__(self, emulate: bool):
        self.on = emulate

    def b(self, x):
        return bf16(x) if self.on else x

    def f(self, x):
        return f32(x) if self.on else x


# ---------------------------------------------------------------------------
# primitives (NHWC, float64)
# ---------------------------------------------------------------------------
TAPS = [(dy, dx) for dy in range(3) for dx in range(3)]  # tap t = 3*dy + dx, offsets dy-1, dx-1


def conv3x3(x, w, b=None):
    """x [N,H,W,Ci], w [Co,9,Ci] -> [N,H,W,Co]."""
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((n, h, wd, w.shape[0]))
    for t, (dy, dx) in enumerate(TAPS):
        out += xp[:, dy:dy + h, dx:dx + wd, :] @ w[:, t, :].T
    if b is not None:
        out += b
    return out


def conv3x3_dgrad(dz, w):
    """Gradient of conv3x3 with respect to its input."""
    n, h, wd, _ = dz.shape
    gp = np.zeros((n, h + 2, wd + 2, w.shape[2]))
    for t, (dy, dx) in enumerate(TAPS):
        gp[:, dy:dy + h, dx:dx + wd, :] += dz @ w[:, t, :]
    return gp[:, 1:h + 1, 1:wd + 1, :]


def conv3x3_wgrad(x, dz):
    """Gradients of conv3x3 with respect to w [Co,9,Ci] and b [Co]."""
    n, h, wd, ci = x.shape
    co = dz.shape[3]
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((co, 9, ci))
    dzf = dz.reshape(-1, co)
    for t, (dy, dx) in enumerate(TAPS):
        dw[:, t, :] = dzf.T @ xp[:, dy:dy + h, dx:dx + wd, :].reshape(-1, ci)
    return dw, dzf.sum(0)


def pool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).max(axis=(2, 4))


def pool2_back(x, g):
    """Route g (at half resolution) to the first maximum of each 2x2 block of x."""
    n, h, w, c = x.shape
    blk = x.reshape(n, h // 2, 2, w // 2, 2, c).transpose(0, 1, 3, 5, 2, 4).reshape(n, h // 2, w // 2, c, 4)
    first = np.argmax(blk == blk.max(axis=-1, keepdims=True), axis=-1)  # first index attaining the max
    out = np.zeros((n, h // 2, w // 2, c, 4))
    np.put_along_axis(out, first[..., None], g[..., None], axis=-1)
    return out.reshape(n, h // 2, w // 2, c, 2, 2).transpose(0, 1, 4, 2, 5, 3).reshape(n, h, w, c)


def up2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up2_back(g):
    n, h, w, c = g.shape
    return g.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


# ---------------------------------------------------------------------------
# forward / backward
# ---------------------------------------------------------------------------
def inputs(raw_mm: np.ndarray):
    """raw uint16 mm [N,H,W] -> (depth_m fp32-as-f64 [N,H,W], valid bool,
    c1 input [N,H,W,9,3]: per tap (difference to the centre in cm, valid, depth))."""
    d = (raw_mm.astype(np.float32) * DEPTH_SCALE).astype(np.float64)
    valid = raw_mm > 0
    n, h, w = raw_mm.shape
    dz = np.where(valid, d, 0.0)
    dp = np.pad(dz, ((0, 0), (1, 1), (1, 1)))
    vp = np.pad(valid, ((0, 0), (1, 1), (1, 1)))
    x = np.zeros((n, h, w, 9, 3))
    for t, (dy, dx) in enumerate(TAPS):
        dt, vt = dp[:, dy:dy + h, dx:dx + w], vp[:, dy:dy + h, dx:dx + w]
        both = vt & valid
        # FP32 arithmetic, as the GPU: (d_t - d_c) * 100
        x[..., t, 0] = np.where(both, ((dt.astype(np.float32) - dz.astype(np.float32)) * np.float32(DIFF_SCALE)), 0.0)
        x[..., t, 1] = vt
        x[..., t, 2] = dt
    return d, valid, x


def conv_in(x, w, b):
    """First convolution: x [N,H,W,9,Ci] (taps pre-gathered), w [Co,9,Ci]."""
    return np.einsum("nhwtc,otc->nhwo", x, w) + b


def conv_in_wgrad(x, dz):
    return np.einsum("nhwtc,nhwo->otc", x, dz), dz.reshape(-1, dz.shape[-1]).sum(0)


def forward(theta, raw_mm, emulate_bf16=True):
    R = _R(emulate_bf16)
    p = unflatten(theta)
    d, valid, x = inputs(raw_mm)
    A = {"x": x}
    A["e0a"] = R.b(np.maximum(conv_in(x, p["c1.w"], p["c1.b"]), 0.0))
    wq = {}
    for name, _, sa, _, mode, sb, _, _, out in CONVS:
        src = A[sa]
        src = pool2(src) if mode == POOL else up2(src) if mode == UP else src
        if sb is not None:
            src = np.concatenate([src, A[sb]], axis=-1)
        A["in_" + name] = src
        wq[name] = R.b(p[name + ".w"])
        A[out] = R.b(np.maximum(conv3x3(src, wq[name], p[name + ".b"]), 0.0))
    r = A["d0"] @ p["head.w"] + p["head.b"][0]
    A["out"] = R.f(np.where(valid, d + RESIDUAL_SCALE * r, 0.0))
    A["depth"], A["valid"] = d, valid
    return A["out"], (A, wq, p)


def loss_and_grad(theta, raw_mm, target_mm, emulate_bf16=True):
    """(loss, flat gradient, out) for one batch."""
    R = _R(emulate_bf16)
    out, (A, wq, p) = forward(theta, raw_mm, emulate_bf16)
    n, h, w = raw_mm.shape
    t = (target_mm.astype(np.float32) * DEPTH_SCALE).astype(np.float64)
    m = A["valid"] & (target_mm > 0)
    inv = 1.0 / (n * h * w)
    diff = out - t
    loss = np.abs(diff[m]).sum() * inv
    dr = np.where(m, np.sign(diff), 0.0) * inv * RESIDUAL_SCALE  # gradient with respect to r
    g = {"head.w": np.einsum("nhw,nhwc->c", dr, A["d0"]), "head.b": np.array([dr.sum()])}
    dz = R.b(dr[..., None] * p["head.w"] * (A["d0"] > 0))
    gin = {}  # gradient reaching each stored tensor through skips
    for name, _, sa, ca, mode, sb, cb, _, out_name in reversed(CONVS):
        g[name + ".w"], g[name + ".b"] = conv3x3_wgrad(A["in_" + name], dz)
        gx = R.b(conv3x3_dgrad(dz, wq[name]))
        if sb is not None:
            gin[sb] = gx[..., ca:]
            ga = gx[..., :ca]
        else:
            ga = gx
        if mode == UP:
            dz = R.b(up2_back(ga) * (A[sa] > 0))
        elif mode == POOL:
            dz = R.b((gin.pop(sa) + pool2_back(A[sa], ga)) * (A[sa] > 0))
        else:
            # the dgrad output of a direct ReLU input is masked in place (the
            # mask is 0/1, so masking before or after the rounding agrees)
            dz = gx * (A[sa] > 0)
    g["c1.w"], g["c1.b"] = conv_in_wgrad(A["x"], dz)
    return loss, flatten(g), out


def init_params(seed: int) -> np.ndarray:
    """He-normal weights, zero biases, zero head (a numpy generator, for
    oracle-only experiments; the library initialises its own)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in param_layout():
        if name == "head.w":
            d[name] = np.zeros(shape)
        elif name.endswith(".w"):
            d[name] = rng.normal(0.0, np.sqrt(2.0 / (9 * shape[2])), shape)
        else:
            d[name] = np.zeros(shape)
    return f32(flatten(d))


def adamw(theta, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, wd=0.01):
    """One AdamW step (decoupled weight decay on weights, not on biases) in
    float32, as the GPU does; returns (theta, m, v)."""
    th = theta.astype(np.float32)
    g = grad.astype(np.float32)
    m = (np.float32(beta1) * m.astype(np.float32) + np.float32(1 - beta1) * g).astype(np.float32)
    v = (np.float32(beta2) * v.astype(np.float32) + np.float32(1 - beta2) * g * g).astype(np.float32)
    bc1 = np.float32(1 - beta1 ** step)
    bc2 = np.float32(1 - beta2 ** step)
    decay = weight_decay_mask().astype(np.float32) * np.float32(wd)
    upd = (m / bc1) / (np.sqrt(v / bc2) + np.float32(eps))
    th = th - np.float32(lr) * (upd + decay * th)
    return th.astype(np.float32), m, v


def weight_decay_mask() -> np.ndarray:
    return np.concatenate([np.full(int(np.prod(s)), 1.0 if n.endswith(".w") else 0.0) for n, s in param_layout()])
