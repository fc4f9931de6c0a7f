"""CPU checks of the oracle's restatements for the model export and shading
rows (Extract_Tsdf_Volume, Extract_Color_Volume, Generate_Image), whose
kernels the reference does not ship: known answers worked out by hand, and
consistency with the golden-pinned slab extraction."""
import numpy as np

from conftest import GOLDEN


def golden_slices(orc):
    g = np.load(GOLDEN / "slices.npz")
    dims = tuple(int(v) for v in g["dims"])
    rb = orc.make_rb(dims, (2.0, 2.0, 2.0), tuple(int(v) for v in g["origin"]))
    return g, dims, rb


def test_whole_volume_export_is_the_pinned_slab_scan_over_every_voxel(orc):
    """With a depth whose divisor-2 and divisor-4 chunks coincide (not in the
    determine_extract_step table: 64-voxel chunks), the whole-volume export
    equals the golden-pinned slab extraction over a zone covering every
    voxel, moved to voxel centres in metres."""
    g, dims, _ = golden_slices(orc)
    W, H, D = dims
    assert orc.chunk_depth(64, 2) == orc.chunk_depth(64, 4) == 64
    # the first 64 slices of the golden volume as their own 32x32x64 volume (origin 0)
    tsdf = np.ascontiguousarray(g["tsdf"]).reshape(D, H, W, 2)[:64].copy()
    rb = orc.make_rb((W, H, 64), (2.0, 2.0, 1.0), (0, 0, 0))
    cell = np.array([2.0 / W, 2.0 / H, 1.0 / 64], np.float32)
    whole, wts, n = orc.extract_tsdf_volume(tsdf.reshape(-1, 2), 0, rb, cell, weights=True)
    slab, _, swts, sn = orc.extract_slice(tsdf.reshape(-1, 2), 0, None, (-10**6,) * 3, (10**6,) * 3, rb,
                                          weights=True)
    assert n == sn and n > 100
    expect = slab.copy()
    expect[:, :3] = (expect[:, :3] + np.float32(0.5)) * cell  # float32 ops, as the restatement
    assert np.array_equal(whole.view(np.uint32), expect.astype(np.float32).view(np.uint32))
    assert np.array_equal(wts, swts) and (wts > 0).all()


def test_color_lookup_known_answers(orc):
    g, dims, rb = golden_slices(orc)
    W, H, D = dims
    cell = np.array([2.0 / W, 2.0 / H, 2.0 / D], np.float32)
    color = np.ascontiguousarray(g["color"])
    org = np.array([int(v) for v in g["origin"]])
    rng = np.random.default_rng(4)
    idx = np.stack([rng.integers(0, W, 200), rng.integers(0, H, 200), rng.integers(0, D, 200)], axis=1)
    pts = np.zeros((200 + 4, 4), np.float32)
    pts[:200, :3] = (idx + 0.5) * cell  # voxel centres
    pts[200] = (-1e-3, 0.5, 0.5, 1)     # outside (x < 0)
    pts[201] = (2.0, 0.5, 0.5, 1)       # on the far face: floor(2/cell) = W, outside
    pts[202] = (np.nan, 0.5, 0.5, 1)
    pts[203] = (0.0, 0.0, 0.0, 1)       # the corner voxel
    out = orc.extract_color_volume(color, rb, pts, cell)
    phys = (idx + org) % np.array([W, H, D])
    addr = phys[:, 0] + W * (phys[:, 1] + H * phys[:, 2])
    assert np.array_equal(out[:200], color[addr])
    assert not out[200:203].any()
    assert np.array_equal(out[203], color[org[0] + W * (org[1] + H * org[2])])


def test_shading_known_answers(orc):
    # a plane z = 1 facing the camera, normals (0, 0, -1), light at the origin
    H, W = 5, 7
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float32)
    v = np.stack([(xs - 3) * 0.25, (ys - 2) * 0.25, np.ones_like(xs)], axis=-1).astype(np.float32)
    n = np.zeros_like(v)
    n[..., 2] = -1.0
    v[0, 0] = np.nan                       # no surface
    n[4, 6] = (np.nan, np.nan, np.nan)     # no normal
    img = orc.generate_image(v, n, (0.0, 0.0, 0.0))
    assert img.shape == (H, W, 3) and (img[..., 0] == img[..., 1]).all() and (img[..., 1] == img[..., 2]).all()
    assert img[2, 3, 0] == 255             # straight below the light: w = 1
    assert img[0, 0, 0] == 0 and img[4, 6, 0] == 0
    # w = cos of the angle to the light: 1 / |v| on this plane
    for (y, x) in [(2, 5), (0, 3), (4, 1)]:
        w = 1.0 / np.linalg.norm(v[y, x].astype(np.float64))
        assert abs(int(img[y, x, 0]) - (int(205 * w) + 50)) <= 1
    # no light: every valid pixel is white
    flat = orc.generate_image(v, n, (0.0, 0.0, 0.0), 0)
    valid = ~np.isnan(v[..., 0]) & ~np.isnan(n[..., 0])
    assert (flat[valid] == 255).all() and not flat[~valid].any()


def test_color_integration_known_answers(orc):
    """Integrate_Colors as restated (KinectFusion colour averaging): a camera
    looking along +z at a model plane through the centres of voxel slice
    z = 8; only that slice is within the truncation distance of the model
    surface.  Colours are running means rounded half to even; the weight
    stops at max_weight."""
    N, cellv, trunc = 16, 0.1, 0.06
    rb = orc.make_rb((N, N, N), (N * cellv,) * 3, (0, 0, 0))
    cell = np.full(3, cellv, np.float32)
    W = H = 16
    intr = orc.Intr(20.0, 20.0, 7.5, 7.5, W, H)
    t = np.array([0.8, 0.8, -1.0], np.float32)
    Ri = np.eye(3, dtype=np.float32)
    plane_z = np.float32(8.5 * cellv)
    vs, us = np.mgrid[0:H, 0:W].astype(np.float32)
    depth = plane_z - t[2]
    vmap = np.stack([(us - 7.5) / 20.0 * depth + t[0], (vs - 7.5) / 20.0 * depth + t[1],
                     np.full_like(us, plane_z)], axis=-1).astype(np.float32)
    color = np.zeros((N ** 3, 4), np.uint8)
    z_of = np.arange(N ** 3) // (N * N)

    def rgb(r, g, b):
        return np.broadcast_to(np.array([r, g, b], np.uint8), (H, W, 3)).copy()

    n1 = orc.integrate_colors(color, rgb(10, 200, 253), vmap, trunc, Ri, t, intr, cell, rb, max_weight=2)
    hit = color[:, 3] > 0
    assert n1 == hit.sum() > 50 and (z_of[hit] == 8).all()
    assert (color[hit] == [10, 200, 253, 1]).all() and not color[~hit].any()
    # a second frame: means (10+20)/2 = 15, (200+100)/2 = 150, (253+0)/2 = 126.5 -> 126 (ties to even)
    orc.integrate_colors(color, rgb(20, 100, 0), vmap, trunc, Ri, t, intr, cell, rb, max_weight=2)
    assert (color[hit] == [15, 150, 126, 2]).all()
    # at max_weight the mean keeps weight 2: (15*2 + 30)/3 = 20, (150*2 + 0)/3 = 100, (126*2 + 3)/3 = 85
    orc.integrate_colors(color, rgb(30, 0, 3), vmap, trunc, Ri, t, intr, cell, rb, max_weight=2)
    assert (color[hit] == [20, 100, 85, 2]).all()
    # no model surface: nothing changes
    before = color.copy()
    assert orc.integrate_colors(color, rgb(1, 2, 3), np.full_like(vmap, np.nan), trunc, Ri, t, intr, cell, rb) == 0
    assert np.array_equal(color, before)
