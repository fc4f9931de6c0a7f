"""ctypes bindings of ``include/tde_capi.h`` (the C-ABI of lib3deye_gb300.so).

The library is loaded from this package directory; importing this module
fails loudly when it has not been built -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib3deye_gb300.so"

TDE_OK = 0
TDE_ERR_INVALID_ARG = -1
TDE_ERR_OOM = -2
TDE_ERR_CUDA = -3
TDE_ERR_DEVICE_TIMEOUT = -4
TDE_ERR_CAPACITY = -5
TDE_ERR_NOT_FOUND = -6
TDE_ERR_UNSUPPORTED = -7

TSDF_I16, TSDF_F16, TSDF_F32 = 0, 1, 2


class Point3f(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Point3i(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class Matrix3f(C.Structure):
    _fields_ = [("row", Point3f * 3)]


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("cols", C.c_int), ("rows", C.c_int)]

    def level(self, l: int) -> "Intrinsics":
        """intrinsics::operator() -- common/src/intrinsics.cpp:7-18."""
        div = float(1 << l)
        return Intrinsics(self.fx / div, self.fy / div, self.cx / div, self.cy / div, self.cols >> l, self.rows >> l)


class RoundBuffer(C.Structure):
    _fields_ = [("start_index", C.c_int), ("end_index", C.c_int), ("buffer_length", C.c_int),
                ("origin_GRID", Point3i), ("origin_GRID_global", Point3f), ("origin_metric", Point3f),
                ("volume_size", Point3f), ("voxels_size", Point3i)]


class Color(C.Structure):
    _fields_ = [("r", C.c_uint8), ("g", C.c_uint8), ("b", C.c_uint8), ("w", C.c_uint8)]


class LightSource(C.Structure):
    """light_source {point_3f pos; int number;} (types/light_source.h:4-8)."""
    _fields_ = [("pos", Point3f), ("number", C.c_int)]


assert C.sizeof(RoundBuffer) == 72 and C.sizeof(Intrinsics) == 24 and C.sizeof(Matrix3f) == 36
assert C.sizeof(LightSource) == 16


class TdeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tde error {code}: {msg}")
        self.code = code


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                          " (the CUDA path has no fallback)")
    return C.CDLL(str(LIB_PATH))


lib = _load()

P = C.c_void_p
I = C.c_int
F = C.c_float
U32 = C.c_uint32
SZ = C.c_size_t
pI = C.POINTER(Intrinsics)
pRB = C.POINTER(RoundBuffer)
pM = C.POINTER(Matrix3f)
pV = C.POINTER(Point3f)

_SIGS = {
    "tde_last_error": (C.c_char_p, []),
    "tde_version": (C.c_char_p, []),
    "tde_tsdf_volume_bytes": (SZ, [I, pRB]),
    "tde_tsdf_init": (I, [P, I, pRB, P]),
    "tde_round_buffer_init": (I, [pRB, Point3i, Point3f]),
    "tde_determine_extract_step": (I, [C.c_uint, I, C.POINTER(C.c_uint), C.POINTER(C.c_uint)]),
    "tde_bilateral_filter": (I, [P, P, I, I, F, F, U32, P]),
    "tde_depth_pyramid_level": (I, [P, P, I, I, F, P]),
    "tde_bilateral_pyramid": (I, [P, C.POINTER(P), I, I, I, F, F, U32, P]),
    "tde_vertex_map": (I, [P, P, pI, P]),
    "tde_normal_map": (I, [P, P, I, I, P]),
    "tde_estimate_combined_gbuf_floats": (SZ, [I, I]),
    "tde_estimate_combined": (I, [P, P, P, P, pM, pV, pM, pV, pI, F, F, P, P, P]),
    "tde_transform_estimation": (I, [P, P, I, I, P]),
    "tde_clean_buff": (I, [P, I, P]),
    "tde_icp_solve_update_host": (I, [P, P, P, P]),
    "tde_icp_solve_device": (I, [P, I, P, P, P, P]),
    "tde_integrate_colors_scratch_bytes": (C.c_size_t, [I, I, C.POINTER(RoundBuffer)]),
    "tde_integrate_colors": (I, [P, P, P, C.POINTER(Intrinsics), C.POINTER(Matrix3f), C.POINTER(Point3f), C.c_float, I,
                                 C.POINTER(Point3f), C.POINTER(RoundBuffer), P]),
    "tde_integrate_colors_ex": (I, [P, P, P, C.POINTER(Intrinsics), C.POINTER(Matrix3f), C.POINTER(Point3f),
                                    C.c_float, I, C.POINTER(Point3f), C.POINTER(RoundBuffer), P, C.c_size_t, P, P]),
    "tde_scale_depth": (I, [P, P, pI, P]),
    "tde_integrate_tsdf": (I, [P, P, I, F, pM, pV, pI, pV, pRB, I, P]),
    "tde_raycast": (I, [P, I, P, P, pV, pM, F, pI, pRB, pV, P]),
    "tde_resize_vertex_map": (I, [P, P, I, I, P]),
    "tde_resize_normal_map": (I, [P, P, I, I, P]),
    "tde_transform_maps": (I, [P, P, P, P, pM, pV, I, I, P]),
    "tde_extract_slice_scratch_bytes": (SZ, [pRB]),
    "tde_extract_slice": (I, [P, I, P, Point3i, Point3i, pRB, P, SZ, P, P, P, U32, P, P]),
    "tde_extract_color_slice": (I, [P, Point3i, Point3i, pRB, P, SZ, P, U32, P, P]),
    "tde_extract_tsdf_volume_scratch_bytes": (SZ, [pRB]),
    "tde_extract_tsdf_volume": (I, [P, I, pRB, Point3f, P, SZ, P, P, U32, P, P]),
    "tde_extract_color_volume": (I, [P, pRB, P, U32, Point3f, P, P]),
    "tde_generate_image": (I, [P, P, I, I, C.POINTER(LightSource), P, P]),
    "tde_clean_tsdf_slice": (I, [P, I, Point3i, Point3i, pRB, P]),
    "tde_clean_color_slice": (I, [P, Point3i, Point3i, pRB, P]),
}


def _bind(name: str, sig) -> None:
    fn = getattr(lib, name, None)
    if fn is None:
        return
    fn.restype, fn.argtypes = sig[0], sig[1]


for _n, _s in _SIGS.items():
    _bind(_n, _s)


def declare(name: str, restype, argtypes) -> None:
    """Declare the signature of a further exported function."""
    fn = getattr(lib, name)
    fn.restype, fn.argtypes = restype, argtypes


def last_error() -> str:
    return lib.tde_last_error().decode()


def check(status: int) -> int:
    if status != TDE_OK:
        raise TdeError(status, last_error())
    return status


def mat3(R) -> Matrix3f:
    R = [float(v) for v in (R.ravel() if hasattr(R, "ravel") else R)]
    return Matrix3f((Point3f * 3)(Point3f(*R[0:3]), Point3f(*R[3:6]), Point3f(*R[6:9])))


def vec3(t) -> Point3f:
    t = [float(v) for v in (t.ravel() if hasattr(t, "ravel") else t)]
    return Point3f(*t[:3])


def round_buffer(voxels, metric, origin=(0, 0, 0)) -> RoundBuffer:
    rb = RoundBuffer()
    check(lib.tde_round_buffer_init(C.byref(rb), Point3i(*voxels), Point3f(*metric)))
    rb.origin_GRID = Point3i(*origin)
    return rb
