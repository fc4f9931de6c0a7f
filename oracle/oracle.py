"""Python access to the CPU oracle (liboracle.so) and, when built, to the
reference's own kernels compiled as C (oracle/_ref/*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's CPU-baseline leg.  Operates on numpy arrays.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"


class Intr(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("cols", C.c_int), ("rows", C.c_int)]

    def level(self, l):
        d = float(1 << l)
        return Intr(self.fx / d, self.fy / d, self.cx / d, self.cy / d, self.cols >> l, self.rows >> l)


class RB(C.Structure):
    _fields_ = [("start_index", C.c_int), ("end_index", C.c_int), ("buffer_length", C.c_int),
                ("origin_GRID", C.c_int * 3), ("origin_GRID_global", C.c_float * 3),
                ("origin_metric", C.c_float * 3), ("volume_size", C.c_float * 3), ("voxels_size", C.c_int * 3)]


def make_rb(voxels, metric, origin=(0, 0, 0)) -> RB:
    rb = RB()
    rb.voxels_size[:] = list(voxels)
    rb.volume_size[:] = [float(v) for v in metric]
    rb.origin_GRID[:] = list(origin)
    rb.buffer_length = int(voxels[0]) * int(voxels[1]) * int(voxels[2])
    return rb


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} missing: run __graft_entry__.build()")
    return C.CDLL(str(LIB_PATH))


lib = _load()
P, I, F, SZ = C.c_void_p, C.c_int, C.c_float, C.c_size_t
pI, pRB = C.POINTER(Intr), C.POINTER(RB)
_sigs = {
    "or_voxel_address": (SZ, [I, I, I, pRB]),
    "or_float_to_half": (C.c_uint16, [F]),
    "or_half_to_float": (F, [C.c_uint16]),
    "or_raycast": (I, [P, I, P, P, P, P, F, pI, pRB, P]),
    "or_bilateral": (I, [P, P, I, I, F, F, C.c_uint32, P]),
    "or_pyramid": (I, [P, P, I, I, F]),
    "or_scale_depth": (I, [P, P, pI]),
    "or_vertex_map": (I, [P, P, pI]),
    "or_normal_map": (I, [P, P, I, I]),
    "or_icp_terms": (I, [P, P, P, P, P, pI, F, F, P, P]),
    "or_icp_solve": (I, [P, P, P, P]),
    "or_integrate": (I, [P, P, I, F, P, P, pI, P, pRB, I, P]),
    "or_resize_map": (I, [P, P, I, I, I]),
    "or_transform_maps": (I, [P, P, P, P, P, P, I, I]),
    "or_transform_estimation": (I, [P, P, I, I]),
    "or_extract_slice": (C.c_int64, [P, I, P, P, P, pRB, I, P, P, P, C.c_int64]),
    "or_extract_tsdf_volume": (C.c_int64, [P, I, pRB, I, P, P, P, C.c_int64]),
    "or_extract_color_volume": (None, [P, pRB, P, C.c_int64, P, P]),
    "or_generate_image": (None, [P, P, C.c_int64, P, I, P]),
    "or_clean_tsdf_slice": (I, [P, I, P, P, pRB]),
    "or_clean_color_slice": (I, [P, P, P, pRB]),
    "or_integrate_colors": (I, [P, P, P, F, P, P, pI, P, pRB, I, P]),
    "or_set_threads": (I, [I]),
    "or_raycast_records": (C.c_int64, [P, I, P, P, P, P, F, pI, pRB, P, P]),
    "or_scale_depth_f64": (I, [P, P, pI]),
    "or_integrate_f64": (I, [P, P, P, C.c_double, P, P, pI, P, pRB, I]),
    "or_raycast_f64": (I, [P, P, P, P, P, C.c_double, pI, pRB, P]),
    "or_icp_terms_f64": (I, [P, P, P, P, P, P, P, P, pI, C.c_double, C.c_double, P]),
    "or_render_depth": (I, [P, I, P, pI, P]),
    "or_apply_noise": (I, [P, P, I, I, C.c_uint32, C.c_uint32, F, F]),
    "or_render_rgb": (I, [P, I, P, pI, P]),
    "or_rgbd_prepare": (I, [P, P, I, I, P, P]),
    "or_rgbd_pyramid": (I, [P, P, I, I, P, P]),
    "or_rgbd_sobel": (I, [P, I, I, P, P]),
    "or_rgbd_points": (I, [P, P, I, I, F, P, I]),
    "or_rgbd_projective": (None, [P, P, pI, P]),
    "or_rgbd_pairs": (I, [P, P, P, P, P, P, pI, P, P, F, F, F, P, P, P]),
    "or_rgbd_lsm": (I, [P, P, P, P, P, P, pI, P, P, F, F, F, P, P]),
    "or_rgbd_row_single": (I, [I, I, F, P, pI, F, F, F, F, P]),
    "or_rgbd_odometry": (I, [P, P, P, P, P, P, pI, I, P, F, F, P, P]),
}
for _n, (_r, _a) in _sigs.items():
    _f = getattr(lib, _n)
    _f.restype, _f.argtypes = _r, _a

F32 = np.float32


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def volume_bytes(fmt, rb: RB) -> int:
    n = rb.voxels_size[0] * rb.voxels_size[1] * rb.voxels_size[2]
    return n * (6 if fmt == 2 else 4)


def raycast_records(vol, fmt, rb, intr, R, t, trunc, cell):
    """Distinct voxel records the reference raycast reads (and its maps)."""
    vm = np.empty((intr.rows, intr.cols, 3), F32)
    nm = np.empty_like(vm)
    n = int(rb.voxels_size[0]) * int(rb.voxels_size[1]) * int(rb.voxels_size[2])
    bits = np.zeros((n + 31) // 32, np.uint32)
    cnt = lib.or_raycast_records(_p(vol), fmt, _p(vm), _p(nm), _p(f32(t)), _p(f32(R)), trunc, C.byref(intr),
                                 C.byref(rb), _p(f32(cell)), _p(bits))
    return int(cnt), vm, nm


def set_threads(n: int) -> int:
    return lib.or_set_threads(n)


def raycast(vol, fmt, rb, intr, R, t, trunc, cell):
    vm = np.empty((intr.rows, intr.cols, 3), F32)
    nm = np.empty_like(vm)
    lib.or_raycast(_p(vol), fmt, _p(vm), _p(nm), _p(f32(t)), _p(f32(R)), trunc, C.byref(intr), C.byref(rb),
                   _p(f32(cell)))
    return vm, nm


def bilateral(src, sigma_space=4.5, sigma_color=30.0, max_mm=32767, want_ratio=False):
    H, W = src.shape
    dst = np.empty_like(src)
    ratio = np.empty((H, W), F32) if want_ratio else None
    lib.or_bilateral(_p(np.ascontiguousarray(src)), _p(dst), W, H, sigma_space, sigma_color, max_mm, _p(ratio))
    return (dst, ratio) if want_ratio else dst


def pyramid(src, sigma_color=30.0):
    H, W = src.shape
    dst = np.empty((H >> 1, W >> 1), np.uint16)
    lib.or_pyramid(_p(np.ascontiguousarray(src)), _p(dst), W, H, sigma_color)
    return dst


def scale_depth(depth, intr):
    out = np.empty((intr.rows, intr.cols), F32)
    lib.or_scale_depth(_p(np.ascontiguousarray(depth)), _p(out), C.byref(intr))
    return out


def vertex_map(depth, intr):
    out = np.empty((intr.rows, intr.cols, 3), F32)
    lib.or_vertex_map(_p(np.ascontiguousarray(depth)), _p(out), C.byref(intr))
    return out


def normal_map(vmap):
    H, W, _ = vmap.shape
    out = np.empty_like(vmap)
    lib.or_normal_map(_p(f32(vmap)), _p(out), W, H)
    return out


def icp_terms(vcur, ncur, vprev, nprev, pose24, intr, dist=0.1, angle=0.34202014):
    sums = np.zeros(28, np.float64)
    mask = np.zeros((intr.rows, intr.cols), np.uint8)
    lib.or_icp_terms(_p(f32(vcur)), _p(f32(ncur)), _p(f32(vprev)), _p(f32(nprev)), _p(f32(pose24)), C.byref(intr),
                     dist, angle, _p(sums), _p(mask))
    return sums, mask


def icp_solve(sums, R, t):
    R = np.ascontiguousarray(R, np.float64).copy()
    t = np.ascontiguousarray(t, np.float64).copy()
    x = np.zeros(6, np.float64)
    st = lib.or_icp_solve(_p(np.ascontiguousarray(sums, np.float64)), _p(R), _p(t), _p(x))
    return st, R, t, x


def integrate(depth_scaled, vol, fmt, trunc, R_inv, t, intr, cell, rb, max_weight=128):
    stats = np.zeros(2, np.uint64)
    lib.or_integrate(_p(f32(depth_scaled)), _p(vol), fmt, trunc, _p(f32(R_inv)), _p(f32(t)), C.byref(intr),
                     _p(f32(cell)), C.byref(rb), max_weight, _p(stats))
    return stats


def resize_map(src, normal):
    H, W, _ = src.shape
    dst = np.empty((H >> 1, W >> 1, 3), F32)
    lib.or_resize_map(_p(f32(src)), _p(dst), W, H, int(normal))
    return dst


def transform_maps(vs, ns, R, t):
    H, W, _ = vs.shape
    vd, nd = np.empty_like(vs), np.empty_like(ns)
    lib.or_transform_maps(_p(f32(vs)), _p(f32(ns)), _p(vd), _p(nd), _p(f32(R)), _p(f32(t)), W, H)
    return vd, nd


def transform_estimation(gbuf, length, stride=1200):
    out = np.empty(27, F32)
    lib.or_transform_estimation(_p(f32(gbuf)), _p(out), length, stride)
    return out


def chunk_depth(depth: int, divisor: int = 4) -> int:
    """determine_extract_step(depth, divisor) of common/src/mem_utils.cpp:43-85
    (step = {512: 256, 256: 128, 128: 64}[depth] / divisor); 64-voxel chunks
    for other depths divisible by 64, else one chunk."""
    table = {512: 256, 256: 128, 128: 64}
    if depth in table:
        return table[depth] // divisor
    return 64 if depth % 64 == 0 else depth


def extract_slice(vol, fmt, color, mn, mx, rb, capacity=None, weights=False):
    step = chunk_depth(rb.voxels_size[2])
    mn_a, mx_a = np.array(mn, np.int32), np.array(mx, np.int32)
    cp = _p(np.ascontiguousarray(color)) if color is not None else None
    n = lib.or_extract_slice(_p(vol), fmt, cp, _p(mn_a), _p(mx_a), C.byref(rb), step, None, None, None, 0)
    cap = n if capacity is None else capacity
    pts = np.zeros((max(cap, 1), 4), F32)
    cols = np.zeros((max(cap, 1), 4), np.uint8)
    wts = np.zeros(max(cap, 1), F32) if weights else None
    lib.or_extract_slice(_p(vol), fmt, cp, _p(mn_a), _p(mx_a), C.byref(rb), step, _p(pts), _p(cols), _p(wts), cap)
    k = min(n, cap)
    return pts[:k], cols[:k], (wts[:k] if weights else None), n


def voxel_addresses(rb, x, y, z):
    """calculate_address (scan_slice_of_both_volumes.cl:17-35): physical index
    of logical voxels, the start_index shift with its `>` wrap test."""
    N = [int(v) for v in rb.voxels_size]
    o = [int(v) for v in rb.origin_GRID]
    px, py, pz = ((np.asarray(c, np.int64) + o[k]) % N[k] for k, c in enumerate((x, y, z)))
    a = N[0] * N[1] * pz + N[0] * py + px + int(rb.start_index)
    L = int(rb.buffer_length)
    return np.where(a > L, a % L, a)


def extract_color_slice(color, mn, mx, rb):
    """Extract_Color_Slice (common/src/opencl_wrappers.cpp:687-782; its scan
    and extract kernels are absent): for logical voxels in (z, y, x) raster
    order -- what the wrapper's z chunks of determine_extract_step(depth, 2)
    give for one plane -- those in the black zone
    (check_whether_it_within_the_black_zone, scan_slice_of_both_volumes.cl:63-74)
    whose colour is set (Color_Point_Is_Set, :53-58) contribute their colour."""
    W, H, D = (int(v) for v in rb.voxels_size)
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    o = [int(v) for v in rb.origin_GRID]
    zone = (((x + o[0] >= mn[0]) & (x + o[0] <= mx[0])) | ((y + o[1] >= mn[1]) & (y + o[1] <= mx[1])) |
            ((z + o[2] >= mn[2]) & (z + o[2] <= mx[2])))
    c = np.asarray(color, np.uint8).reshape(-1, 4)[voxel_addresses(rb, x, y, z).ravel()]
    keep = zone.ravel() & (c != 0).any(axis=1)
    return np.ascontiguousarray(c[keep])


def extract_tsdf_volume(vol, fmt, rb, cell, capacity=None, weights=False):
    """Extract_Tsdf_Volume (common/src/opencl_wrappers.cpp:440-543): the slab
    scan with every voxel in the zone, no colour plane, z chunks of
    determine_extract_step(depth, divisor 2), and points at the metric centre
    (i + 0.5) * cell of the voxel they name.  Its kernels are not in the
    reference's sources; this follows the shipped slab kernels
    (scan_slice_of_both_volumes.cl:76-208, extract_slice_as_cloud.cl:72-201)."""
    step = chunk_depth(rb.voxels_size[2], 2)
    c = np.asarray(cell, F32)
    n = lib.or_extract_tsdf_volume(_p(vol), fmt, C.byref(rb), step, _p(c), None, None, 0)
    cap = n if capacity is None else capacity
    pts = np.zeros((max(cap, 1), 4), F32)
    wts = np.zeros(max(cap, 1), F32) if weights else None
    lib.or_extract_tsdf_volume(_p(vol), fmt, C.byref(rb), step, _p(c), _p(pts), _p(wts), cap)
    k = min(n, cap)
    return pts[:k], (wts[:k] if weights else None), n


def extract_color_volume(color, rb, points, cell):
    """Extract_Color_Volume (common/src/opencl_wrappers.cpp:545-581): colour of
    voxel floor(p / cell) for each point; zero outside the volume."""
    pts = np.ascontiguousarray(points, F32)
    out = np.zeros((len(pts), 4), np.uint8)
    lib.or_extract_color_volume(_p(np.ascontiguousarray(color)), C.byref(rb), _p(pts), len(pts),
                                _p(np.asarray(cell, F32)), _p(out))
    return out


def generate_image(vmap, nmap, light, nlights=1):
    """Generate_Image (common/src/opencl_wrappers.cpp:967-992): grey shading,
    uint8 [rows, cols, 3] for [rows, cols, 3] vertex and normal maps."""
    v = np.ascontiguousarray(vmap, F32)
    nm = np.ascontiguousarray(nmap, F32)
    out = np.zeros(v.shape[:-1] + (3,), np.uint8)
    lib.or_generate_image(_p(v), _p(nm), v.size // 3, _p(np.asarray(light, F32)), nlights, _p(out))
    return out


def clean_tsdf_slice(vol, fmt, mn, mx, rb):
    lib.or_clean_tsdf_slice(_p(vol), fmt, _p(np.array(mn, np.int32)), _p(np.array(mx, np.int32)), C.byref(rb))


def integrate_colors(color, rgb, vmap, trunc, R_inv, t, intr, cell, rb, max_weight=255):
    """Colour integration in place on `color` (uint8 [n, 4] records r, g, b, w); returns the count of
    voxels updated."""
    n = np.zeros(1, np.uint64)
    lib.or_integrate_colors(_p(color), _p(np.ascontiguousarray(rgb, np.uint8)), _p(f32(vmap)), trunc, _p(f32(R_inv)),
                            _p(f32(t)), C.byref(intr), _p(f32(cell)), C.byref(rb), max_weight, _p(n))
    return int(n[0])


def clean_color_slice(color, mn, mx, rb):
    lib.or_clean_color_slice(_p(color), _p(np.array(mn, np.int32)), _p(np.array(mx, np.int32)), C.byref(rb))


def render_depth(scene, pose12, intr):
    out = np.empty((intr.rows, intr.cols), F32)
    sc = np.ascontiguousarray(scene, np.float64)
    lib.or_render_depth(_p(sc), sc.shape[0], _p(np.ascontiguousarray(pose12, np.float64)), C.byref(intr), _p(out))
    return out


def apply_noise(depth_m, seed, frame, max_range=4.0, dropout=0.02):
    H, W = depth_m.shape
    out = np.empty((H, W), np.uint16)
    lib.or_apply_noise(_p(f32(depth_m)), _p(out), W, H, seed & 0xFFFFFFFF, frame & 0xFFFFFFFF, max_range, dropout)
    return out


# ---------------------------------------------------------------------------
# The reference's kernels compiled as C (present only where the reference
# tree was available at build time).
# ---------------------------------------------------------------------------
def ref_available() -> bool:
    return (REF_DIR / "ref_raycast.so").exists()


_ref_cache = {}


def ref(name: str) -> C.CDLL:
    if name not in _ref_cache:
        _ref_cache[name] = C.CDLL(str(REF_DIR / f"ref_{name}.so"))
    return _ref_cache[name]


# ---------------------------------------------------------------------------
# full-FP64 model stages (precision study)
# ---------------------------------------------------------------------------
def f64(a):
    return np.ascontiguousarray(a, np.float64)


def scale_depth_f64(depth, intr):
    out = np.empty(depth.shape, np.float64)
    lib.or_scale_depth_f64(_p(np.ascontiguousarray(depth)), _p(out), C.byref(intr))
    return out


def integrate_f64(depth_scaled, tsdf, weight, trunc, R_inv, t, intr, cell, rb, max_weight):
    lib.or_integrate_f64(_p(f64(depth_scaled)), _p(tsdf), _p(weight), float(trunc), _p(f64(R_inv)), _p(f64(t)),
                         C.byref(intr), _p(f64(cell)), C.byref(rb), int(max_weight))


def raycast_f64(tsdf, rb, intr, R, t, trunc, cell):
    vm = np.empty((intr.rows, intr.cols, 3), np.float64)
    nm = np.empty_like(vm)
    lib.or_raycast_f64(_p(tsdf), _p(vm), _p(nm), _p(f64(t)), _p(f64(R)), float(trunc), C.byref(intr), C.byref(rb),
                       _p(f64(cell)))
    return vm, nm


def icp_terms_f64(vcur, ncur, vprev, nprev, R, t, R_prev_inv, t_prev, intr, dist_thresh, angle_thresh):
    sums = np.zeros(28, np.float64)
    lib.or_icp_terms_f64(_p(f32(vcur)), _p(f32(ncur)), _p(f64(vprev)), _p(f64(nprev)), _p(f64(R)), _p(f64(t)),
                         _p(f64(R_prev_inv)), _p(f64(t_prev)), C.byref(intr), float(dist_thresh), float(angle_thresh),
                         _p(sums))
    return sums


# ---------------------------------------------------------------------------
# dense RGB-D odometry (oracle_rgbd.c)
# ---------------------------------------------------------------------------
RGBD_MAX_DEPTH = 35.0        # scan_list_of_valid_correspondence.cl:9-15
RGBD_DEPTH_DIFF = 0.07       # DEFAULT_DEPTH_THRESHOLD_RGBD, common_defines.h:18


def render_rgb(scene, pose12, intr):
    out = np.zeros((intr.rows, intr.cols, 3), np.uint8)
    sc = np.ascontiguousarray(scene, np.float64)
    lib.or_render_rgb(_p(sc), sc.shape[0], _p(np.ascontiguousarray(pose12, np.float64)), C.byref(intr), _p(out))
    return out


def rgbd_prepare(depth_mm, rgb):
    H, W = depth_mm.shape
    I8 = np.zeros((H, W), np.uint8)
    D = np.zeros((H, W), F32)
    lib.or_rgbd_prepare(_p(np.ascontiguousarray(depth_mm, np.uint16)), _p(np.ascontiguousarray(rgb, np.uint8)), W, H,
                        _p(I8), _p(D))
    return I8, D


def rgbd_pyramid(I8, D):
    H, W = I8.shape
    I2 = np.zeros((H >> 1, W >> 1), np.uint8)
    D2 = np.zeros((H >> 1, W >> 1), F32)
    lib.or_rgbd_pyramid(_p(np.ascontiguousarray(I8)), _p(f32(D)), W, H, _p(I2), _p(D2))
    return I2, D2


def rgbd_sobel(I8):
    H, W = I8.shape
    dx = np.zeros((H, W), np.int16)
    dy = np.zeros((H, W), np.int16)
    lib.or_rgbd_sobel(_p(np.ascontiguousarray(I8)), W, H, _p(dx), _p(dy))
    return dx, dy


def rgbd_points(dx, dy, scale):
    H, W = dx.shape
    n = lib.or_rgbd_points(_p(np.ascontiguousarray(dx)), _p(np.ascontiguousarray(dy)), W, H, scale, None, 0)
    pts = np.zeros((max(n, 1), 2), np.int32)
    lib.or_rgbd_points(_p(np.ascontiguousarray(dx)), _p(np.ascontiguousarray(dy)), W, H, scale, _p(pts), n)
    return pts[:n]


def rgbd_levels(depth_mm, rgb, levels):
    """Per level (finest first): intensity, metric depth, Sobel dx, dy."""
    I8, D = rgbd_prepare(depth_mm, rgb)
    out = []
    for l in range(levels):
        if l:
            I8, D = rgbd_pyramid(I8, D)
        dx, dy = rgbd_sobel(I8)
        out.append((I8, D, dx, dy))
    return out


def rgbd_pairs(prev, curr, intr, pose12, min_gradient, max_depth_diff=RGBD_DEPTH_DIFF, max_depth=RGBD_MAX_DEPTH):
    """prev, curr: (I, D, dx, dy) of one level.  Returns (count, kept [H,W]
    (1 + index of the current pixel, 0 for none), residuals, sum r^2)."""
    H, W = prev[0].shape
    kept = np.zeros((H, W), np.int32)
    res = np.zeros((H, W), F32)
    s = np.zeros(1, np.float64)
    pose = np.ascontiguousarray(pose12, np.float64)
    n = lib.or_rgbd_pairs(_p(prev[0]), _p(f32(prev[1])), _p(curr[0]), _p(f32(curr[1])), _p(curr[2]), _p(curr[3]),
                          C.byref(intr), _p(pose[:9].copy()), _p(pose[9:].copy()), max_depth_diff, max_depth,
                          min_gradient, _p(kept), _p(res), _p(s))
    return n, kept, res, float(s[0])


def rgbd_lsm(prev, curr, intr, pose12, min_gradient, max_depth_diff=RGBD_DEPTH_DIFF, max_depth=RGBD_MAX_DEPTH):
    sums = np.zeros(28, np.float64)
    sigma = np.zeros(1, F32)
    pose = np.ascontiguousarray(pose12, np.float64)
    lib.or_rgbd_lsm(_p(prev[0]), _p(f32(prev[1])), _p(curr[0]), _p(f32(curr[1])), _p(curr[2]), _p(curr[3]),
                    C.byref(intr), _p(pose[:9].copy()), _p(pose[9:].copy()), max_depth_diff, max_depth, min_gradient,
                    _p(sums), _p(sigma))
    return sums, float(sigma[0])


def rgbd_row_single(u, v, z, Rt12, intr, dIdx, dIdy, r, sigma):
    row = np.zeros(7, F32)
    lib.or_rgbd_row_single(u, v, z, _p(f32(Rt12)), C.byref(intr), dIdx, dIdy, r, sigma, _p(row))
    return row


def rgbd_odometry(prev_levels, curr_levels, intr, iters, min_gradient, init_pose12=None,
                  max_depth_diff=RGBD_DEPTH_DIFF, max_depth=RGBD_MAX_DEPTH):
    """Pose (12 doubles) mapping previous-frame camera points to current ones, and the failed-solve count."""
    L = len(prev_levels)
    keep = []

    def arr(items, k, dtype):
        a = (C.c_void_p * L)()
        for l in range(L):
            x = np.ascontiguousarray(items[l][k], dtype)
            keep.append(x)
            a[l] = x.ctypes.data
        return a
    pose = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64) if init_pose12 is None else \
        np.ascontiguousarray(init_pose12, np.float64).copy()
    it = np.ascontiguousarray(iters, np.int32)
    mg = np.ascontiguousarray(min_gradient, F32)
    failed = lib.or_rgbd_odometry(arr(prev_levels, 0, np.uint8), arr(prev_levels, 1, F32), arr(curr_levels, 0, np.uint8),
                                  arr(curr_levels, 1, F32), arr(curr_levels, 2, np.int16), arr(curr_levels, 3, np.int16),
                                  C.byref(intr), L, _p(it), max_depth_diff, max_depth, _p(mg), _p(pose))
    return pose, failed
