"""The CPU oracle against the golden vectors produced by the reference's own
kernels (tests/golden/make_golden.py).  Runs without a GPU."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return np.array_equal(a.view(np.uint32), b.view(np.uint32)) or (
        np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)]))


def raycast_cases(orc):
    g = np.load(GOLDEN / "raycast.npz")
    for i in range(int(g["ncases"])):
        k = lambda s: g[f"c{i}_{s}"]
        N, V = int(k("N")), float(k("V"))
        fx, fy, cx, cy, W, H = k("intr")
        intr = orc.Intr(fx, fy, cx, cy, int(W), int(H))
        rb = orc.make_rb((N, N, N), (V, V, V), tuple(int(v) for v in k("origin")))
        yield dict(vol=np.ascontiguousarray(k("vol")), rb=rb, intr=intr, R=k("R"), t=k("t"),
                   trunc=float(k("trunc")), cell=np.full(3, V / N, np.float32), vmap=k("vmap"), nmap=k("nmap"))


def test_raycast_oracle_bit_exact(orc):
    n = 0
    for c in raycast_cases(orc):
        vm, nm = orc.raycast(c["vol"], 0, c["rb"], c["intr"], c["R"], c["t"], c["trunc"], c["cell"])
        assert same_bits(vm, c["vmap"]), "vertex map differs from the reference kernel"
        assert same_bits(nm, c["nmap"]), "normal map differs from the reference kernel"
        n += int(np.isfinite(vm[..., 0]).sum())
    assert n > 5000  # the cases actually hit surfaces


def test_bilateral_oracle_matches_intended(orc):
    g = np.load(GOLDEN / "bilateral.npz")
    src = g["src"]
    for name in ("a", "b"):
        out, ratio = orc.bilateral(src, 4.5, 30.0, int(g[f"{name}_maxd"]), want_ratio=True)
        ref = g[f"{name}_intended"].astype(np.int32)
        d = np.abs(out.astype(np.int32) - ref)
        # same window and weights; the oracle accumulates sum1 with fma
        assert d.max() <= 1
        assert (d == 0).mean() >= 0.999
        fin = np.isfinite(g[f"{name}_ratio"])
        assert np.allclose(ratio[fin], g[f"{name}_ratio"][fin], rtol=1e-5, atol=1e-3)


def test_bilateral_reference_literal_output_is_sum1(orc):
    """Documents the reference quirk: the kernel stores rte(sum1), not the
    filtered depth (compute_bilateral_filtering.cl:55)."""
    g = np.load(GOLDEN / "bilateral.npz")
    lit = g["a_literal"].astype(np.int64)
    intended = g["a_intended"].astype(np.int64)
    assert (lit != intended).mean() > 0.5


def test_transform_maps_oracle_bit_exact(orc):
    g = np.load(GOLDEN / "transform_map.npz")
    vd, nd = orc.transform_maps(g["vs"], g["ns"], g["R"], g["t"])
    assert same_bits(vd, g["vd"]) and same_bits(nd, g["nd"])


def test_transform_estimation_oracle(orc):
    g = np.load(GOLDEN / "transform_estimation.npz")
    for L in (1200, 300, 19):
        out = orc.transform_estimation(g["gbuf"], L, 1200)
        np.testing.assert_allclose(out, g[f"out_{L}"], rtol=1e-4, atol=1e-4)
    co = g["clean_out"]
    assert np.all(co[:27 * 300] == 0)


def slice_inputs(orc):
    g = np.load(GOLDEN / "slices.npz")
    W, H, D = (int(v) for v in g["dims"])
    V = 2.0
    rb = orc.make_rb((W, H, D), (V, V, V), tuple(int(v) for v in g["origin"]))
    return g, rb


def test_extract_slice_oracle_bit_exact(orc):
    g, rb = slice_inputs(orc)
    tsdf = np.ascontiguousarray(g["tsdf"])
    color = np.ascontiguousarray(g["color"])
    for ci in range(int(g["ncases"])):
        mn, mx = g[f"c{ci}_mn"], g[f"c{ci}_mx"]
        pts, cols, _, n = orc.extract_slice(tsdf, 0, color, mn, mx, rb)
        assert n == int(g[f"c{ci}_count"])
        assert np.array_equal(pts.view(np.uint32), g[f"c{ci}_points"].view(np.uint32))
        assert np.array_equal(cols, g[f"c{ci}_colors"])


def test_extract_color_slice_is_the_colour_plane_of_the_pinned_slab_scan(orc):
    """Extract_Color_Slice's restatement equals the colour plane of the
    golden-pinned slab scan: with every TSDF weight zero the scan's +x/+y/+z
    predicates never fire (scan_slice_of_both_volumes.cl:108-135 need w != 0),
    so its output is the colour plane alone, chunk after chunk."""
    g, rb = slice_inputs(orc)
    tsdf = np.ascontiguousarray(g["tsdf"]).copy()
    tsdf[:, 1] = 0
    color = np.ascontiguousarray(g["color"])
    total = 0
    for ci in range(int(g["ncases"])):
        mn, mx = g[f"c{ci}_mn"], g[f"c{ci}_mx"]
        _, cols, _, n = orc.extract_slice(tsdf, 0, color, mn, mx, rb)
        got = orc.extract_color_slice(color, mn, mx, rb)
        assert len(got) == n and np.array_equal(got, cols)
        total += n
    assert total > 1000


def test_extract_slice_reference_boundary_writes_documented(orc):
    """The reference's extract kernel writes +z points at chunk ends that its
    scan never counted (extract_slice_as_cloud.cl:369 vs
    scan_slice_of_both_volumes.cl:160); the z-slab case crosses chunk ends."""
    g, _ = slice_inputs(orc)
    assert sum(int(g[f"c{ci}_boundary_writes"]) for ci in range(int(g["ncases"]))) > 0


def test_clean_color_slice_oracle(orc):
    g, rb = slice_inputs(orc)
    for ci in range(int(g["ncases"])):
        c = np.ascontiguousarray(g["color"]).copy()
        orc.clean_color_slice(c, g[f"c{ci}_mn"], g[f"c{ci}_mx"], rb)
        assert np.array_equal(c, g[f"c{ci}_color_cleaned"])


def test_float_half_roundtrip(orc):
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.normal(0, 1, 5000), rng.uniform(-70000, 70000, 2000), rng.uniform(-1e-6, 1e-6, 2000),
                         [0.0, -0.0, 65504.0, 65519.99, 65520.0, 2 ** -24, 2 ** -25, 3 * 2 ** -26, np.inf, -np.inf]])
    for x in xs.astype(np.float32):
        h = orc.lib.or_float_to_half(C.c_float(float(x)))
        ref = np.array([x], np.float32).astype(np.float16).view(np.uint16)[0]
        assert h == ref, (x, h, ref)
        assert orc.lib.or_half_to_float(h) == np.float32(np.array([h], np.uint16).view(np.float16)[0])


def test_voxel_address_matches_reference_rule(orc):
    rb = orc.make_rb((8, 6, 4), (1.0, 1.0, 1.0), (3, 5, 1))
    for x, y, z in [(0, 0, 0), (7, 5, 3), (5, 1, 3), (4, 0, 2)]:
        a = orc.lib.or_voxel_address(x, y, z, C.byref(rb))
        px, py, pz = (x + 3) % 8, (y + 5) % 6, (z + 1) % 4
        assert a == 8 * 6 * pz + 8 * py + px
