"""Known answers for the oracle stages whose reference kernels are absent.

The reference does not ship the kernels of scale/integrate, the depth
pyramid, the vertex and normal maps, ICP association and clean_tsdf_slice, so
golden vectors cannot pin them.  These tests pin the CPU restatement to the
published method itself -- KinectFusion (Newcombe et al. 2011) with the
point-to-plane linearisation (Low 2004) -- on analytic inputs whose right
answer is known independently of the code: a fronto-parallel plane, a sphere,
a tilted plane, constant depth, a known rigid motion, a known slab.  The CUDA
kernels equal these oracle stages bit for bit (tests/test_kernels_gpu.py), so
the known answers hold for them too.

Conventions of the reference these answers use: voxel centres at
(i + 1/2) * cell (raycast.cl:9-27 encoding, opencl_wrappers.cpp:21-64), the
pyramid intrinsics of intrinsics.cpp:7-18, the 27-term [A | b] layout of
opencl_wrappers.cpp:426-437 and the black zone of
scan_slice_of_both_volumes.cl:63-74.
"""
import importlib

import numpy as np
import pytest

syn = importlib.import_module("3deye_gb300.synth")

# storage step of one TSDF value, per format (int16: 1/32767; fp16: half ulp
# at 1; fp32: float rounding of depth and distance)
STEP = {0: 1.0 / 32767, 1: 2.0 ** -11, 2: 1e-6}


def decode(vol, fmt, n):
    """TSDF value and weight per voxel (physical order) of a volume buffer."""
    if fmt == 0:
        r = vol.view(np.int16).reshape(-1, 2)
        return r[:, 0].astype(np.float64) / 32767.0, r[:, 1].astype(np.int64)
    if fmt == 1:
        r = vol.view(np.uint16).reshape(-1, 2)
        return r[:, 0].view(np.float16).astype(np.float64), r[:, 1].astype(np.int64)
    f = vol[: 4 * n].view(np.float32).astype(np.float64)
    w = vol[4 * n: 6 * n].view(np.uint16).astype(np.int64)
    return f, w


def centres(N, cell):
    k = (np.arange(N, dtype=np.float64) + 0.5) * cell
    z, y, x = np.meshgrid(k, k, k, indexing="ij")
    return x.ravel(), y.ravel(), z.ravel()


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_integrate_fronto_parallel_plane(orc, fmt):
    """Camera at (c, c, 0) looking along +z at the plane z = d: a voxel whose
    centre g projects to pixel (u, v) gets sdf = D(u, v) - |g - t|, D the
    distance along the ray of pixel (u, v) to the plane, d * |K^-1 [u v 1]|;
    f = min(1, sdf / trunc) with weight 1 where sdf >= -trunc, nothing
    elsewhere."""
    N, V, W, H = 48, 1.2, 80, 60
    fx = fy = 70.0
    cx, cy = (W - 1) / 2.0, (H - 1) / 2.0
    d_mm = 737
    trunc = 3 * V / N
    cell = V / N
    intr = orc.Intr(fx, fy, cx, cy, W, H)
    rb = orc.make_rb((N,) * 3, (V,) * 3)
    vol = np.zeros(orc.volume_bytes(fmt, rb), np.uint8)
    t = np.array([V / 2, V / 2, 0.0], np.float32)
    depth = np.full((H, W), d_mm, np.uint16)
    sd = orc.scale_depth(depth, intr)
    orc.integrate(sd, vol, fmt, trunc, np.eye(3, dtype=np.float32), t, intr, np.full(3, cell, np.float32), rb)
    f, w = decode(vol, fmt, N ** 3)

    gx, gy, gz = centres(N, np.float32(cell))
    px, py, pz = gx - t[0], gy - t[1], gz - t[2]
    ue, ve = fx * px / pz + cx, fy * py / pz + cy
    u, v = np.rint(ue), np.rint(ve)
    inside = (u >= 0) & (u < W) & (v >= 0) & (v < H)
    D = d_mm / 1000.0 * np.sqrt(((u - cx) / fx) ** 2 + ((v - cy) / fy) ** 2 + 1.0)
    sdf = D - np.sqrt(px ** 2 + py ** 2 + pz ** 2)
    upd = inside & (sdf >= -trunc)
    # away from the cut-off sdf = -trunc and from projections half way between
    # two pixels, where float rounding may go either way
    half = lambda a: np.abs(a - np.floor(a) - 0.5) < 1e-3
    clear = (np.abs(sdf + trunc) > 1e-5) & ~half(ue) & ~half(ve)
    assert np.array_equal(w[clear] == 1, upd[clear]) and np.all(w[clear & ~upd] == 0)
    want = np.minimum(1.0, sdf / trunc)
    sel = upd & clear
    err = np.abs(f[sel] - want[sel])
    assert err.max() <= STEP[fmt] + 1e-5, err.max()
    # the surface: voxels straddling z = d change sign there
    band = sel & (np.abs(sdf) < trunc)
    assert band.sum() > 1000 and (f[band & (sdf > cell)] > 0).all() and (f[band & (sdf < -cell)] < 0).all()


def test_integrate_sphere_is_truncated_euclidean_distance(orc):
    """A sphere ahead of the camera, rendered as float depth along each
    pixel's ray: near the optical axis (where the viewing ray is within 6 deg
    of the surface normal) the fused value is the truncated Euclidean signed
    distance to the sphere, up to the cos(angle) and pixel-quantisation
    difference between a projective and a Euclidean distance."""
    N, V, W, H = 96, 1.6, 160, 120
    fx = fy = 150.0
    cx, cy = (W - 1) / 2.0, (H - 1) / 2.0
    cell = V / N
    trunc = 3 * cell
    intr = orc.Intr(fx, fy, cx, cy, W, H)
    rb = orc.make_rb((N,) * 3, (V,) * 3)
    c = np.array([V / 2, V / 2, 1.0])
    r = 0.35
    t = np.array([V / 2, V / 2, 0.0])
    # depth along the ray (what scale_depth hands to the integration), metres
    uu, vv = np.meshgrid(np.arange(W), np.arange(H))
    dirs = np.stack([(uu - cx) / fx, (vv - cy) / fy, np.ones_like(uu, dtype=np.float64)], -1)
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    oc = t - c
    b = dirs @ oc
    disc = b ** 2 - (oc @ oc - r * r)
    dist = np.where(disc > 0, -b - np.sqrt(np.maximum(disc, 0)), 0.0).astype(np.float32)
    vol = np.zeros(orc.volume_bytes(2, rb), np.uint8)
    orc.integrate(dist, vol, 2, trunc, np.eye(3, dtype=np.float32), t.astype(np.float32), intr,
                  np.full(3, cell, np.float32), rb)
    f, w = decode(vol, 2, N ** 3)
    gx, gy, gz = centres(N, cell)
    g = np.stack([gx, gy, gz], -1)
    sd = r - np.linalg.norm(g - c, axis=-1)          # > 0 outside... negative inside the sphere
    sd = -sd                                         # signed distance: + in front (outside), - inside
    axis = np.hypot(gx - c[0], gy - c[1]) < r * np.sin(np.radians(6.0))
    near = axis & (gz < c[2]) & (np.abs(sd) < 0.8 * trunc) & (w == 1)
    assert near.sum() >= 20
    err = np.abs(f[near] - sd[near] / trunc)
    assert err.max() < 0.02, err.max()
    # in front of the sphere, further than the truncation: free space (f = 1)
    free = axis & (gz < c[2]) & (sd > 1.5 * trunc) & (w == 1)
    assert free.sum() > 10 and np.all(f[free] == 1.0)
    # behind the surface, past the truncation: untouched
    behind = axis & (sd < -1.5 * trunc) & (gz < c[2] + r)
    assert behind.sum() > 10 and np.all(w[behind] == 0)


def test_vertex_and_normal_maps_of_a_tilted_plane(orc):
    """Depth of the plane n.p = d seen from the origin: the vertex map is
    z * K^-1 [u v 1] of the stored depth, and the PCA normals equal n facing
    the camera (n.v < 0) up to the 1 mm depth rounding."""
    W, H = 160, 120
    fx = fy = 131.25
    cx, cy = (W - 1) / 2.0, (H - 1) / 2.0
    intr = orc.Intr(fx, fy, cx, cy, W, H)
    n = np.array([0.3, -0.2, -1.0])
    n /= np.linalg.norm(n)
    d = -1.1  # n.p = d with p ahead of the camera
    uu, vv = np.meshgrid(np.arange(W, dtype=np.float64), np.arange(H, dtype=np.float64))
    ray = np.stack([(uu - cx) / fx, (vv - cy) / fy, np.ones_like(uu)], -1)
    z = d / (ray @ n)
    depth = np.rint(z * 1000.0).astype(np.uint16)
    vm = orc.vertex_map(depth, intr)
    zq = depth.astype(np.float64) / 1000.0
    np.testing.assert_allclose(vm[..., 2], zq, rtol=0, atol=1e-6)
    np.testing.assert_allclose(vm[..., 0], zq * (uu - cx) / fx, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(vm[..., 1], zq * (vv - cy) / fy, rtol=1e-6, atol=1e-6)
    nm = orc.normal_map(vm)
    ok = ~np.isnan(nm[..., 0])
    assert ok.mean() > 0.9
    facing = n if (n @ np.array([0.0, 0.0, 1.0])) < 0 else -n
    ang = np.degrees(np.arccos(np.clip(nm[ok] @ facing, -1, 1)))
    assert np.median(ang) < 0.5 and np.percentile(ang, 99) < 2.0, (np.median(ang), np.percentile(ang, 99))
    # an invalid pixel has no vertex; the image border lacks the 24 neighbours
    depth[10, 10] = 0
    assert np.isnan(orc.vertex_map(depth, intr)[10, 10]).all()
    assert np.isnan(nm[0, 0]).all()


def test_depth_pyramid_of_constant_depth_and_holes(orc):
    """Every level of a constant frame is the same constant (halved size);
    holes (0) stay holes and do not enter a neighbour's average; a pixel
    beyond 3 sigma_color of the block centre is left out."""
    H, W = 120, 160
    d = np.full((H, W), 1234, np.uint16)
    p1 = orc.pyramid(d, 30.0)
    p2 = orc.pyramid(p1, 30.0)
    assert p1.shape == (60, 80) and p2.shape == (30, 40)
    assert (p1 == 1234).all() and (p2 == 1234).all()
    d[40, 40] = 0              # centre of output (20, 20) invalid -> 0
    d[41, 41] = 5000           # outlier next to a valid centre, beyond 3 * 30 mm
    p = orc.pyramid(d, 30.0)
    assert p[20, 20] == 0
    assert p[20, 21] == 1234 and p[21, 20] == 1234
    d2 = np.full((H, W), 1000, np.uint16)
    d2[:, 1::2] = 1040         # within 3 sigma: averaged
    p = orc.pyramid(d2, 30.0)
    # the 5x5 window at an even column holds 3 columns of 1000 and 2 of 1040
    assert p[30, 30] == (3 * 1000 + 2 * 1040 + 2) // 5


def _rot(axis, deg):
    a = np.asarray(axis, np.float64)
    a /= np.linalg.norm(a)
    th = np.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def test_icp_recovers_a_known_rigid_motion(orc):
    """Point-to-plane ICP (Low 2004) with projective association, coarse to
    fine, as the per-frame loop runs it: model maps are frame A's maps in the
    world frame, the current maps are frame B's, rendered from a pose moved
    by a known 1.5 cm / 1.2 deg step; the solve recovers that pose."""
    from oracle.pipeline import OraclePipeline
    cfg = syn.small_config("c1", frames=2, cols=320, rows=240, voxels=64, fmt=2)
    scene = syn.make_scene(cfg, 1000)
    T0 = syn.make_trajectory(cfg, 2000)[0]
    R0, t0 = T0[:9].reshape(3, 3), T0[9:]
    dR = _rot([0.3, 1.0, -0.2], 1.2)
    R1 = R0 @ dR
    t1 = t0 + R0 @ np.array([0.012, -0.006, 0.0065])
    T1 = np.concatenate([R1.ravel(), t1])
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    dA = np.rint(orc.render_depth(scene, T0, intr) * 1000.0).astype(np.uint16)
    dB = np.rint(orc.render_depth(scene, T1, intr) * 1000.0).astype(np.uint16)
    op = OraclePipeline(cfg, T0)
    _, vA, nA = op.frame_maps(dA)
    for l in range(op.levels):
        op.vmod[l], op.nmod[l] = orc.transform_maps(vA[l], nA[l], R0.astype(np.float32), t0.astype(np.float32))
    _, vB, nB = op.frame_maps(dB)
    assert op.track(vB, nB)
    dt = np.linalg.norm(op.t - t1)
    dang = np.degrees(np.arccos(np.clip((np.trace(op.R.T @ R1) - 1) / 2, -1, 1)))
    assert dt < 1e-3 and dang < 0.05, (dt, dang)
    # and the step it had to find was a real one
    assert np.linalg.norm(t1 - t0) > 0.01


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_clean_tsdf_slice_zeroes_exactly_the_black_zone(orc, fmt):
    """Voxels whose global index (logical + origin_GRID) lies in [min, max] on
    any axis are reset to (0, weight 0); every other record keeps its bits."""
    N = (24, 20, 28)
    origin = (5, 17, 3)
    rb = orc.make_rb(N, (1.0, 1.0, 1.0), origin)
    rng = np.random.default_rng(4)
    vol = rng.integers(0, 256, orc.volume_bytes(fmt, rb), dtype=np.uint8)
    n = int(np.prod(N))
    if fmt == 2:
        vol[: 4 * n] = rng.uniform(-1, 1, n).astype(np.float32).view(np.uint8)
        vol[4 * n: 6 * n] = rng.integers(1, 100, n).astype(np.uint16).view(np.uint8)
    before = vol.copy()
    # x in [8, 10], no y, z in [25, 26]; the test is on logical + origin, unwrapped
    mn, mx = (8, -50, 25), (10, -60, 26)
    orc.clean_tsdf_slice(vol, fmt, mn, mx, rb)
    f, w = decode(vol, fmt, n)
    f0, w0 = decode(before, fmt, n)
    z, y, x = np.meshgrid(np.arange(N[2]), np.arange(N[1]), np.arange(N[0]), indexing="ij")
    zone = ((x + origin[0] >= 8) & (x + origin[0] <= 10)) | ((z + origin[2] >= 25) & (z + origin[2] <= 26))
    addr = orc.voxel_addresses(rb, x, y, z).ravel()
    zone_phys = np.zeros(n, bool)
    zone_phys[addr] = zone.ravel()
    assert zone_phys.sum() == 3 * N[1] * N[2] + 2 * N[0] * N[1] - 2 * 3 * N[1]
    assert np.all(f[zone_phys] == 0) and np.all(w[zone_phys] == 0)
    keep = ~zone_phys
    assert np.array_equal(np.nan_to_num(f[keep]), np.nan_to_num(f0[keep])) and np.array_equal(w[keep], w0[keep])
