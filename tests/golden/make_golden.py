"""Generate the golden vectors under tests/golden/ from the reference's own
OpenCL kernels compiled as C (oracle/_ref, built by oracle/build_ref.sh from
a checkout of the reference).  Run where a reference checkout exists:

    TDE_REFERENCE=<reference checkout> bash oracle/build_ref.sh
    python tests/golden/make_golden.py

Inputs are seeded; every fixture stores its inputs and the reference outputs.
The slab clouds are also written in the reference's text format
(slices_c*_points.txt, slices_c*_colors.txt).
The reference ships no golden vectors or tests of its own, so these fixtures
are what pins the oracle (tests/test_oracle_golden.py) and, through it, the
CUDA kernels.

Harness conventions (mirroring the reference host code):
  * raycast: one work-item per pixel, as Raycast (opencl_wrappers.cpp:66-95).
  * bilateral: the kernel writes convert_ushort_rte(sum1) (a reference bug);
    the shim records the argument of its convert_int_rte, sum1/sum2, from
    which the intended output rte(sum1/sum2), clamp, truncation follows
    (compute_bilateral_filtering.cl:49-53).  Both are stored.
  * slab extraction: per z chunk of determine_extract_step(depth, 4) the scan
    kernel, an exclusive prefix sum, and the extract kernel, as Extract_Slice
    (opencl_wrappers.cpp:856-964).  Slots of zero predicates point at a dump
    slot past the end, so the extract kernel's chunk-boundary +z writes
    (extract_slice_as_cloud.cl:369 tests z+1 < voxels_size.z where the scan
    tested z+1 < Max_Size) cannot overwrite a real point: the stored output
    is the reference's result on the scan's predicate set.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent


def p(a):
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------------------
# analytic scene -> int16 TSDF volume
# ---------------------------------------------------------------------------
def scene_sdf(pts: np.ndarray, V: float) -> np.ndarray:
    c = V / 2
    d = np.full(pts.shape[:-1], 1e9)
    d = np.minimum(d, (c + 0.3 * V) - pts[..., 1])                       # ground plane (y down)
    for cc, r in (((c, c + 0.1 * V, c), 0.18 * V), ((c - 0.22 * V, c + 0.15 * V, c + 0.1 * V), 0.12 * V),
                  ((c + 0.2 * V, c + 0.05 * V, c - 0.15 * V), 0.1 * V)):
        d = np.minimum(d, np.linalg.norm(pts - np.array(cc), axis=-1) - r)
    bmin, bmax = np.array([c - 0.35 * V, c, c - 0.3 * V]), np.array([c - 0.15 * V, c + 0.3 * V, c - 0.1 * V])
    q = np.abs(pts - (bmin + bmax) / 2) - (bmax - bmin) / 2
    box = np.linalg.norm(np.maximum(q, 0), axis=-1) + np.minimum(q.max(axis=-1), 0)
    return np.minimum(d, box)


def tsdf_volume_i16(N: int, V: float, trunc: float, origin=(0, 0, 0), weight=5):
    """Logical voxel (x,y,z) holds the field at its centre; stored at the
    cyclic address for `origin` (raycast.cl:29-47 with start_index 0)."""
    cs = V / N
    idx = (np.arange(N) + 0.5) * cs
    Z, Y, X = np.meshgrid(idx, idx, idx, indexing="ij")
    sdf = scene_sdf(np.stack([X, Y, Z], axis=-1), V)
    f = np.clip(sdf / trunc, -1.0, 1.0).astype(np.float32)
    v = np.trunc(f * np.float32(32767)).astype(np.int32).clip(-32767, 32767).astype(np.int16)
    w = np.where(sdf < -trunc, 0, weight).astype(np.int16)
    logical = np.stack([v, w], axis=-1)                                    # [z, y, x, 2]
    ox, oy, oz = origin
    stored = np.empty_like(logical)
    zz = (np.arange(N) + oz) % N
    yy = (np.arange(N) + oy) % N
    xx = (np.arange(N) + ox) % N
    stored[np.ix_(zz, yy, xx)] = logical
    return np.ascontiguousarray(stored.reshape(-1, 2))


def look(eye, tgt):
    zc = tgt - eye
    zc /= np.linalg.norm(zc)
    xc = np.cross([0.0, 1.0, 0.0], zc)
    xc /= np.linalg.norm(xc)
    yc = np.cross(zc, xc)
    return np.stack([xc, yc, zc], axis=1).astype(np.float32)


def gen_raycast():
    out = {}
    N, V = 64, 2.0
    trunc = 3 * V / N
    cases = []
    for ci, (origin, eye, tgt, W, H) in enumerate([
            ((0, 0, 0), (1.0, 0.55, -0.4), (1.0, 1.2, 1.0), 80, 60),
            ((5, 9, 3), (2.3, 0.7, 0.3), (0.9, 1.15, 1.05), 96, 72),
            ((60, 1, 33), (1.5, 0.5, 0.5), (0.9, 1.2, 1.4), 64, 48)]):        # camera inside the volume
        vol = tsdf_volume_i16(N, V, trunc, origin)
        rb = orc.make_rb((N, N, N), (V, V, V), origin)
        f = W * 0.82
        intr = orc.Intr(f, f, (W - 1) / 2.0, (H - 1) / 2.0, W, H)
        R = look(np.array(eye), np.array(tgt))
        t = np.array(eye, np.float32)
        cell = np.full(3, V / N, np.float32)
        vm = np.zeros((H, W, 3), np.float32)
        nm = np.zeros((H, W, 3), np.float32)
        orc.ref("raycast").ref_raycast(p(vol), p(vm), p(nm), p(t), p(R), C.c_float(trunc), C.byref(intr),
                                       C.byref(rb), p(cell))
        cases.append(dict(vol=vol, origin=np.array(origin, np.int32), intr=np.array([intr.fx, intr.fy, intr.cx,
                          intr.cy, W, H], np.float64), R=R, t=t, trunc=np.float32(trunc), N=N, V=V, vmap=vm,
                          nmap=nm))
    for i, c in enumerate(cases):
        for k, v in c.items():
            out[f"c{i}_{k}"] = v
    out["ncases"] = len(cases)
    np.savez_compressed(OUT / "raycast.npz", **out)
    return {i: int(np.isfinite(c["vmap"][..., 0]).sum()) for i, c in enumerate(cases)}


def gen_bilateral():
    rng = np.random.default_rng(7)
    W, H = 96, 72
    yy, xx = np.mgrid[0:H, 0:W]
    depth = (1200 + 400 * np.sin(xx / 13.0) + 250 * (yy > 40) + rng.normal(0, 6, (H, W))).astype(np.int32)
    depth[rng.uniform(size=(H, W)) < 0.05] = 0
    depth[10:20, 30:45] = 0
    depth = np.clip(depth, 0, 65535).astype(np.uint16)
    out = {"src": depth}
    for name, maxd in (("a", 32767), ("b", 1500)):
        dst = np.zeros_like(depth)
        ratio = np.zeros((H, W), np.float32)
        orc.ref("bilateral").ref_bilateral(p(depth), p(dst), W, H, C.c_uint(maxd), p(ratio))
        res = np.clip(np.where(np.isnan(ratio), 0, np.rint(ratio)), 0, 32767).astype(np.int32)
        res[res > maxd] = 0
        out[f"{name}_maxd"] = np.int32(maxd)
        out[f"{name}_literal"] = dst
        out[f"{name}_ratio"] = ratio
        out[f"{name}_intended"] = res.astype(np.uint16)
    np.savez_compressed(OUT / "bilateral.npz", **out)


def gen_transform_map():
    rng = np.random.default_rng(11)
    W, H = 40, 32
    vs = rng.normal(0, 1, (H, W, 3)).astype(np.float32)
    ns = rng.normal(0, 1, (H, W, 3)).astype(np.float32)
    vs[rng.uniform(size=(H, W)) < 0.1, 0] = np.nan
    ns[rng.uniform(size=(H, W)) < 0.1, 0] = np.nan
    ang = 0.3
    R = np.array([[np.cos(ang), -np.sin(ang), 0], [np.sin(ang), np.cos(ang), 0], [0, 0, 1]], np.float32)
    t = np.array([0.1, -0.2, 0.3], np.float32)
    vd, nd = np.zeros_like(vs), np.zeros_like(ns)
    orc.ref("transform_map").ref_transform_map(p(vs), p(ns), p(R), p(t), W, H, p(vd), p(nd))
    np.savez_compressed(OUT / "transform_map.npz", vs=vs, ns=ns, R=R, t=t, vd=vd, nd=nd)


def gen_transform_estimation():
    rng = np.random.default_rng(13)
    gbuf = rng.normal(0, 1, 27 * 1200).astype(np.float32)
    out = {"gbuf": gbuf}
    for L in (1200, 300, 19):
        o = np.zeros(27, np.float32)
        orc.ref("transform_estimation").ref_transform_estimation(p(gbuf), p(o), L)
        out[f"out_{L}"] = o
    cb = rng.normal(0, 1, 27 * 300).astype(np.float32)
    out["clean_in"] = cb.copy()
    orc.ref("clean_buff").ref_clean_buff(p(cb), 300)
    out["clean_out"] = cb
    np.savez_compressed(OUT / "transform_estimation.npz", **out)


def gen_slices():
    W, H, D, V = 32, 32, 128, 2.0
    trunc = 3 * V / W
    origin = (3, 5, 7)
    rng = np.random.default_rng(17)
    # anisotropic volume: cell size differs per axis
    cs = np.array([V / W, V / H, V / D], np.float32)
    idx = [(np.arange(n) + 0.5) * c for n, c in ((W, cs[0]), (H, cs[1]), (D, cs[2]))]
    Z, Y, X = np.meshgrid(idx[2], idx[1], idx[0], indexing="ij")
    sdf = scene_sdf(np.stack([X, Y, Z], axis=-1), V)
    f = np.clip(sdf / trunc, -1, 1).astype(np.float32)
    v = np.trunc(f * np.float32(32767)).astype(np.int32).clip(-32767, 32767).astype(np.int16)
    w = np.where(rng.uniform(size=f.shape) < 0.05, 0, 3).astype(np.int16)
    logical = np.stack([v, w], axis=-1)
    stored = np.empty_like(logical)
    stored[np.ix_((np.arange(D) + origin[2]) % D, (np.arange(H) + origin[1]) % H,
                  (np.arange(W) + origin[0]) % W)] = logical
    tsdf = np.ascontiguousarray(stored.reshape(-1, 2))
    color = np.zeros((D * H * W, 4), np.uint8)
    sel = rng.uniform(size=D * H * W) < 0.03
    color[sel] = rng.integers(1, 255, size=(sel.sum(), 4), dtype=np.uint8)
    rb = orc.make_rb((W, H, D), (V, V, V), origin)
    step = 16                                                   # determine_extract_step(128, 4)
    cases = [((3, -100, -100), (9, -101, -101)),                 # x slab
             ((-100, 30, -100), (-101, 36, -101)),               # y slab, wrapping past H
             ((-100, -100, 40), (-101, -101, 70)),               # z slab across chunks
             ((0, 33, 100), (4, 34, 134))]                       # all three axes
    out = {"tsdf": tsdf, "color": color, "origin": np.array(origin, np.int32), "dims": np.array([W, H, D], np.int32),
           "cell": cs, "ncases": len(cases)}
    for ci, (mn, mx) in enumerate(cases):
        mn_a, mx_a = np.array(mn, np.int32), np.array(mx, np.int32)
        pts_all, cols_all, count_kernel, dumps = [], [], 0, 0
        pred = np.zeros(4 * W * H * step, np.uint32)
        for i in range(D // step):
            lo, hi = i * step, (i + 1) * step
            num = np.zeros(1, np.uint32)
            orc.ref("scan_slice").ref_scan_slice(p(tsdf), p(color), p(mn_a), p(mx_a), lo, hi, C.byref(rb), p(pred),
                                                 p(num))
            cnt = int(pred.sum())
            assert cnt == int(num[0]), (cnt, int(num[0]))
            count_kernel += int(num[0])
            if cnt == 0:
                continue
            excl = np.concatenate([[0], np.cumsum(pred.astype(np.int64))[:-1]]).astype(np.uint32)
            slots = np.where(pred != 0, excl, cnt).astype(np.uint32)
            pts = np.zeros((cnt + 1, 4), np.float32)
            cols = np.zeros((cnt + 1, 4), np.uint8)
            orc.ref("extract_slice").ref_extract_slice(p(slots), p(tsdf), p(color), lo, hi, p(cs), p(mn_a), p(mx_a),
                                                       C.byref(rb), p(pts), p(cols))
            dumps += int(np.any(pts[cnt] != 0))
            pts_all.append(pts[:cnt])
            cols_all.append(cols[:cnt])
        out[f"c{ci}_mn"], out[f"c{ci}_mx"] = mn_a, mx_a
        out[f"c{ci}_points"] = np.concatenate(pts_all) if pts_all else np.zeros((0, 4), np.float32)
        out[f"c{ci}_colors"] = np.concatenate(cols_all) if cols_all else np.zeros((0, 4), np.uint8)
        out[f"c{ci}_count"] = np.int64(count_kernel)
        out[f"c{ci}_boundary_writes"] = np.int64(dumps)
        cc = color.copy()
        orc.ref("clean_color_slice").ref_clean_color_slice(p(cc), p(mn_a), p(mx_a), C.byref(rb))
        out[f"c{ci}_color_cleaned"] = cc
    np.savez_compressed(OUT / "slices.npz", **out)
    return {ci: int(out[f"c{ci}_count"]) for ci in range(len(cases))}


def gen_lsm():
    """compute_least_squares_equation.cl, one correspondence per call (n = 1:
    the kernel writes Indexes[id + k], so larger n overlaps rows): the six
    coefficients C and the vector C * diff * w, for seeded poses, pixels,
    depths, derivatives (its derivative buffers are unsigned char), residuals
    and sigmas."""
    rng = np.random.default_rng(17)
    W, H = 64, 48
    intr = orc.Intr(58.5, 61.25, 31.7, 24.3, W, H)
    lib = orc.ref("lsm")
    sz = np.zeros(4, np.int32)
    lib.ref_lsm_sizes(p(sz))
    assert sz[1] == 8 and sz[2] == 24 and sz[3] == 36, sz
    n = 96
    cases = {k: [] for k in ("u", "v", "z", "R", "t", "dx", "dy", "diff", "sigma", "C", "vec")}
    ip = np.zeros(W * H * max(int(sz[0]), 1), np.uint8)
    for _ in range(n):
        u, v = int(rng.integers(0, W)), int(rng.integers(0, H))
        uc, vc = int(rng.integers(0, W)), int(rng.integers(0, H))
        z = np.float32(rng.uniform(0.4, 6.0))
        w = rng.normal(0, 0.05, 3)
        th = np.linalg.norm(w)
        K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]]) / max(th, 1e-12)
        R = (np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K).astype(np.float32)
        t = rng.normal(0, 0.05, 3).astype(np.float32)
        dxv, dyv = int(rng.integers(0, 256)), int(rng.integers(0, 256))
        diff = np.float32(rng.integers(-120, 121))
        sigma = np.float32(rng.uniform(0.5, 40.0))
        dp = np.zeros(W * H, np.float32)
        dp[v * W + u] = z
        gx = np.zeros(W * H, np.uint8)
        gy = np.zeros(W * H, np.uint8)
        gx[vc * W + uc], gy[vc * W + uc] = dxv, dyv
        cp = np.array([u, v], np.int32)
        cc = np.array([uc, vc], np.int32)
        df = np.array([diff], np.float32)
        idx = np.zeros(6, np.float32)
        vec = np.zeros(6, np.float32)
        lib.ref_lsm(p(ip), p(dp), p(ip), p(gx), p(gy), p(cp), p(cc), p(df), C.c_float(sigma), p(R), p(t),
                    C.byref(intr), 1, p(idx), p(vec))
        for k, val in (("u", u), ("v", v), ("z", z), ("R", R), ("t", t), ("dx", dxv), ("dy", dyv), ("diff", diff),
                       ("sigma", sigma), ("C", idx), ("vec", vec)):
            cases[k].append(val)
    out = {k: np.asarray(v) for k, v in cases.items()}
    out["intr"] = np.array([intr.fx, intr.fy, intr.cx, intr.cy, W, H], np.float64)
    np.savez_compressed(OUT / "rgbd_lsm.npz", **out)


def gen_text_fixtures():
    """The slab clouds of slices.npz again in the reference's own text format
    (matrix<Point_XYZI> / matrix<Point_Color>::Save_To_File,
    common/inc/impl/matrix.hpp:413-476), as a reference caller would save them."""
    import importlib
    fmt = importlib.import_module("3deye_gb300.formats")
    g = np.load(OUT / "slices.npz")
    for ci in range(int(g["ncases"])):
        fmt.write_cloud(OUT / f"slices_c{ci}_points.txt", points=g[f"c{ci}_points"])
        fmt.write_cloud(OUT / f"slices_c{ci}_colors.txt", colors=g[f"c{ci}_colors"])


def main():
    if not orc.ref_available():
        sys.exit("oracle/_ref is not built: run TDE_REFERENCE=<reference checkout> bash oracle/build_ref.sh")
    print("raycast hits", gen_raycast())
    gen_bilateral()
    gen_transform_map()
    gen_transform_estimation()
    gen_lsm()
    print("slice counts", gen_slices())
    gen_text_fixtures()
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
