"""3deye_gb300 -- GB300-native KinectFusion per-frame pipeline.

The product is ``lib3deye_gb300.so`` (hand-written sm_103a CUDA kernels
behind the C-ABI of ``include/tde_capi.h`` and the reference-compatible C++
API of ``include/3deye/``).  This Python package is a thin host-side mirror:
it binds the C-ABI with ctypes and passes torch CUDA tensors' device pointers
through it.  Every function raises when the CUDA library is missing or a
tensor is not on the GPU; nothing here computes on the CPU.

Names follow the reference's free functions (common/inc/opencl_wrappers.h).
"""
from __future__ import annotations

import ctypes as C

from ._capi import (TSDF_F16, TSDF_F32, TSDF_I16, Color, Intrinsics, LightSource, Matrix3f, Point3f, Point3i,
                    RoundBuffer, TdeError, check, last_error, lib, mat3, round_buffer, vec3)

__all__ = [
    "TSDF_I16", "TSDF_F16", "TSDF_F32", "Intrinsics", "RoundBuffer", "Point3f", "Point3i", "Matrix3f", "Color",
    "TdeError", "lib", "check", "last_error", "mat3", "vec3", "round_buffer", "ptr", "stream_ptr",
    "tsdf_volume_bytes", "tsdf_init", "bilateral_filter", "depth_pyramid_level", "vertex_map", "normal_map",
    "estimate_combined", "transform_estimation", "clean_buff", "scale_depth", "integrate_tsdf", "raycast",
    "resize_vertex_map", "resize_normal_map", "transform_maps", "extract_slice", "extract_tsdf_volume",
    "extract_color_volume", "extract_color_slice", "clean_tsdf_slice", "clean_color_slice", "generate_image", "LightSource",
]


def ptr(t) -> int:
    """Device pointer of a contiguous CUDA tensor (raises otherwise)."""
    if t is None:
        return None
    if not getattr(t, "is_cuda", False):
        raise TdeError(-1, "tensor is not on a CUDA device")
    if not t.is_contiguous():
        raise TdeError(-1, "tensor is not contiguous")
    return t.data_ptr()


def stream_ptr(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _torch():
    import torch
    return torch


def tsdf_volume_bytes(fmt: int, rb: RoundBuffer) -> int:
    return lib.tde_tsdf_volume_bytes(fmt, C.byref(rb))


def tsdf_init(volume, fmt: int, rb: RoundBuffer, stream=None):
    check(lib.tde_tsdf_init(ptr(volume), fmt, C.byref(rb), stream_ptr(stream)))
    return volume


def new_volume(fmt: int, rb: RoundBuffer, device="cuda"):
    torch = _torch()
    v = torch.empty(tsdf_volume_bytes(fmt, rb), dtype=torch.uint8, device=device)
    return tsdf_init(v, fmt, rb)


def bilateral_filter(depth, out=None, sigma_space=4.5, sigma_color=30.0, max_distance_mm=32767, stream=None):
    """Apply_Billateral_Filtration (opencl_wrappers.cpp:216-235)."""
    torch = _torch()
    H, W = depth.shape
    out = torch.empty_like(depth) if out is None else out
    check(lib.tde_bilateral_filter(ptr(depth), ptr(out), W, H, sigma_space, sigma_color, max_distance_mm,
                                   stream_ptr(stream)))
    return out


def depth_pyramid_level(src, sigma_color=30.0, stream=None):
    torch = _torch()
    H, W = src.shape
    dst = torch.empty((H >> 1, W >> 1), dtype=src.dtype, device=src.device)
    check(lib.tde_depth_pyramid_level(ptr(src), ptr(dst), W, H, sigma_color, stream_ptr(stream)))
    return dst


def vertex_map(depth, intr: Intrinsics, stream=None):
    torch = _torch()
    v = torch.empty((intr.rows, intr.cols, 3), dtype=torch.float32, device=depth.device)
    check(lib.tde_vertex_map(ptr(depth), ptr(v), C.byref(intr), stream_ptr(stream)))
    return v


def normal_map(vmap, stream=None):
    torch = _torch()
    H, W, _ = vmap.shape
    n = torch.empty_like(vmap)
    check(lib.tde_normal_map(ptr(vmap), ptr(n), W, H, stream_ptr(stream)))
    return n


def estimate_combined(vcur, ncur, vprev, nprev, R_cur, t_cur, R_prev_inv, t_prev, intr: Intrinsics,
                      dist_thresh=0.1, angle_thresh=0.34202014, stream=None):
    """Estimate_Combined (opencl_wrappers.cpp:364-438): returns the 27 sums."""
    torch = _torch()
    g = torch.empty(lib.tde_estimate_combined_gbuf_floats(intr.cols, intr.rows), dtype=torch.float32,
                    device=vcur.device)
    m = torch.empty(27, dtype=torch.float32, device=vcur.device)
    Rc, tc, Rp, tp = mat3(R_cur), vec3(t_cur), mat3(R_prev_inv), vec3(t_prev)
    check(lib.tde_estimate_combined(ptr(vcur), ptr(ncur), ptr(vprev), ptr(nprev), C.byref(Rc), C.byref(tc),
                                    C.byref(Rp), C.byref(tp), C.byref(intr), dist_thresh, angle_thresh, ptr(g),
                                    ptr(m), stream_ptr(stream)))
    return m


def transform_estimation(gbuf, buf_length: int, group_stride: int = 1200, stream=None):
    torch = _torch()
    out = torch.empty(27, dtype=torch.float32, device=gbuf.device)
    check(lib.tde_transform_estimation(ptr(gbuf), ptr(out), buf_length, group_stride, stream_ptr(stream)))
    return out


def clean_buff(gbuf, width: int, stream=None):
    check(lib.tde_clean_buff(ptr(gbuf), width, stream_ptr(stream)))
    return gbuf


def scale_depth(depth, intr: Intrinsics, stream=None):
    torch = _torch()
    out = torch.empty((intr.rows, intr.cols), dtype=torch.float32, device=depth.device)
    check(lib.tde_scale_depth(ptr(depth), ptr(out), C.byref(intr), stream_ptr(stream)))
    return out


def integrate_tsdf(depth_scaled, volume, fmt, trunc, R_inv, t, intr: Intrinsics, cell, rb: RoundBuffer,
                   max_weight=128, stream=None):
    """Integrate_Tsdf_Data (opencl_wrappers.cpp:21-64), integration stage."""
    Ri, tt, cs = mat3(R_inv), vec3(t), vec3(cell)
    check(lib.tde_integrate_tsdf(ptr(depth_scaled), ptr(volume), fmt, trunc, C.byref(Ri), C.byref(tt),
                                 C.byref(intr), C.byref(cs), C.byref(rb), max_weight, stream_ptr(stream)))
    return volume


def integrate_colors(color_volume, rgb, vertex_map, intr: Intrinsics, R_inv, t, trunc, cell, rb: RoundBuffer,
                     max_weight=255, stream=None):
    """Integrate_Colors (opencl_wrappers.cpp:181-214): color_volume uint8 [n, 4] (r, g, b, w) on the device,
    rgb uint8 [rows, cols, 3], vertex_map float32 [rows, cols, 3] (the model raycast from the same pose)."""
    Ri, tt, cs = mat3(R_inv), vec3(t), vec3(cell)
    check(lib.tde_integrate_colors(ptr(color_volume), ptr(rgb), ptr(vertex_map), C.byref(intr), C.byref(Ri),
                                   C.byref(tt), trunc, max_weight, C.byref(cs), C.byref(rb), stream_ptr(stream)))
    return color_volume


def raycast(volume, fmt, rb: RoundBuffer, intr: Intrinsics, R, t, trunc, cell, vmap=None, nmap=None, stream=None):
    """Raycast (opencl_wrappers.cpp:66-95)."""
    torch = _torch()
    shape = (intr.rows, intr.cols, 3)
    vmap = torch.empty(shape, dtype=torch.float32, device=volume.device) if vmap is None else vmap
    nmap = torch.empty(shape, dtype=torch.float32, device=volume.device) if nmap is None else nmap
    Rm, tt, cs = mat3(R), vec3(t), vec3(cell)
    check(lib.tde_raycast(ptr(volume), fmt, ptr(vmap), ptr(nmap), C.byref(tt), C.byref(Rm), trunc, C.byref(intr),
                          C.byref(rb), C.byref(cs), stream_ptr(stream)))
    return vmap, nmap


def _resize(fn, src, stream):
    torch = _torch()
    H, W, _ = src.shape
    dst = torch.empty((H >> 1, W >> 1, 3), dtype=torch.float32, device=src.device)
    check(fn(ptr(src), ptr(dst), W, H, stream_ptr(stream)))
    return dst


def resize_vertex_map(src, stream=None):
    return _resize(lib.tde_resize_vertex_map, src, stream)


def resize_normal_map(src, stream=None):
    return _resize(lib.tde_resize_normal_map, src, stream)


def transform_maps(vmap, nmap, R, t, stream=None):
    torch = _torch()
    H, W, _ = vmap.shape
    vd, nd = torch.empty_like(vmap), torch.empty_like(nmap)
    Rm, tt = mat3(R), vec3(t)
    check(lib.tde_transform_maps(ptr(vmap), ptr(nmap), ptr(vd), ptr(nd), C.byref(Rm), C.byref(tt), W, H,
                                 stream_ptr(stream)))
    return vd, nd


def extract_slice(volume, fmt, color, min_bounds, max_bounds, rb: RoundBuffer, capacity=None, weights=False,
                  stream=None):
    """Extract_Slice (opencl_wrappers.cpp:856-964).  Returns (points, colors,
    weights-or-None, total count); grows the output once if it was too small."""
    torch = _torch()
    dev = volume.device
    scratch = torch.empty(lib.tde_extract_slice_scratch_bytes(C.byref(rb)), dtype=torch.uint8, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    cap = 1 << 16 if capacity is None else int(capacity)
    for _ in range(2):
        pts = torch.empty((max(cap, 1), 4), dtype=torch.float32, device=dev)
        cols = torch.empty((max(cap, 1), 4), dtype=torch.uint8, device=dev)
        wts = torch.empty(max(cap, 1), dtype=torch.float32, device=dev) if weights else None
        check(lib.tde_extract_slice(ptr(volume), fmt, ptr(color) if color is not None else None,
                                    Point3i(*min_bounds), Point3i(*max_bounds), C.byref(rb), ptr(scratch),
                                    scratch.numel(), ptr(pts), ptr(cols), ptr(wts) if wts is not None else None,
                                    cap, ptr(count), stream_ptr(stream)))
        n = int(count.item())
        if n <= cap or capacity is not None:
            k = min(n, cap)
            return pts[:k], cols[:k], (wts[:k] if wts is not None else None), n
        cap = n
    raise TdeError(-5, "extract_slice: capacity retry failed")


def extract_color_slice(color, min_bounds, max_bounds, rb: RoundBuffer, capacity=None, stream=None):
    """Extract_Color_Slice (opencl_wrappers.cpp:687-782): the colours of the
    set voxels of the black zone in raster order.  Returns (colors, total
    count); grows the output once if it was too small."""
    torch = _torch()
    dev = color.device
    scratch = torch.empty(lib.tde_extract_slice_scratch_bytes(C.byref(rb)), dtype=torch.uint8, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    cap = 1 << 16 if capacity is None else int(capacity)
    for _ in range(2):
        cols = torch.empty((max(cap, 1), 4), dtype=torch.uint8, device=dev)
        check(lib.tde_extract_color_slice(ptr(color), Point3i(*min_bounds), Point3i(*max_bounds), C.byref(rb),
                                          ptr(scratch), scratch.numel(), ptr(cols), cap, ptr(count),
                                          stream_ptr(stream)))
        n = int(count.item())
        if n <= cap or capacity is not None:
            return cols[:min(n, cap)], n
        cap = n
    raise TdeError(-5, "extract_color_slice: capacity retry failed")


def generate_image(vmap, nmap, light_pos=(0.0, 0.0, 0.0), light_number=1, image=None, stream=None):
    """Generate_Image (opencl_wrappers.cpp:967-992): grey shading of [rows,
    cols, 3] vertex and normal maps into a uint8 [rows, cols, 3] image."""
    torch = _torch()
    rows, cols = vmap.shape[0], vmap.shape[1]
    if image is None:
        image = torch.empty((rows, cols, 3), dtype=torch.uint8, device=vmap.device)
    light = LightSource(Point3f(*light_pos), int(light_number))
    check(lib.tde_generate_image(ptr(vmap), ptr(nmap), cols, rows, C.byref(light), ptr(image), stream_ptr(stream)))
    return image


def extract_tsdf_volume(volume, fmt, rb: RoundBuffer, cell_size, capacity=None, weights=False, stream=None):
    """Extract_Tsdf_Volume (opencl_wrappers.cpp:440-543): every zero crossing
    of the volume as the metric centre {(i + 0.5) * cell, 1} of the voxel it
    names.  Returns (points [n, 4], weights-or-None, total count); grows the
    output once if it was too small."""
    torch = _torch()
    dev = volume.device
    scratch = torch.empty(lib.tde_extract_tsdf_volume_scratch_bytes(C.byref(rb)), dtype=torch.uint8, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    cap = 1 << 20 if capacity is None else int(capacity)
    for _ in range(2):
        pts = torch.empty((max(cap, 1), 4), dtype=torch.float32, device=dev)
        wts = torch.empty(max(cap, 1), dtype=torch.float32, device=dev) if weights else None
        check(lib.tde_extract_tsdf_volume(ptr(volume), fmt, C.byref(rb), Point3f(*cell_size), ptr(scratch),
                                          scratch.numel(), ptr(pts), ptr(wts) if wts is not None else None, cap,
                                          ptr(count), stream_ptr(stream)))
        n = int(count.item())
        if n <= cap or capacity is not None:
            k = min(n, cap)
            return pts[:k], (wts[:k] if wts is not None else None), n
        cap = n
    raise TdeError(-5, "extract_tsdf_volume: capacity retry failed")


def extract_color_volume(color, rb: RoundBuffer, points, cell_size, stream=None):
    """Extract_Color_Volume (opencl_wrappers.cpp:545-581): the colour of the
    voxel floor(p / cell) holding each point; uint8 [n, 4]."""
    torch = _torch()
    pts = points.contiguous()
    out = torch.zeros((pts.shape[0], 4), dtype=torch.uint8, device=pts.device)
    check(lib.tde_extract_color_volume(ptr(color), C.byref(rb), ptr(pts), pts.shape[0], Point3f(*cell_size),
                                       ptr(out), stream_ptr(stream)))
    return out


def clean_tsdf_slice(volume, fmt, min_bounds, max_bounds, rb: RoundBuffer, stream=None):
    check(lib.tde_clean_tsdf_slice(ptr(volume), fmt, Point3i(*min_bounds), Point3i(*max_bounds), C.byref(rb),
                                   stream_ptr(stream)))
    return volume


def clean_color_slice(color, min_bounds, max_bounds, rb: RoundBuffer, stream=None):
    check(lib.tde_clean_color_slice(ptr(color), Point3i(*min_bounds), Point3i(*max_bounds), C.byref(rb),
                                    stream_ptr(stream)))
    return color
