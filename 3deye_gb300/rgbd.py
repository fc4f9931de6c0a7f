"""Host side of the dense RGB-D (photometric) odometry: the reference's second
tracker, Estimate_Isometry_By_RGBD and its stages (common/src/
opencl_wrappers.cpp:345-362, 1008-1466), on the C-ABI of include/tde_capi.h.

Device buffers are torch CUDA tensors; poses are 12 doubles (R row-major,
then t) mapping previous-frame camera points to current-frame ones.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import Intrinsics, check, declare, lib

P, I, F, SZ, U32 = C.c_void_p, C.c_int, C.c_float, C.c_size_t, C.c_uint32

MAX_LEVELS = 4
SOBEL_SCALE = 0.125
IDENTITY = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)


class Point2i(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int)]


class RgbdFrameC(C.Structure):
    _fields_ = [("intensity", P * MAX_LEVELS), ("depth", P * MAX_LEVELS), ("dx", P * MAX_LEVELS),
                ("dy", P * MAX_LEVELS)]


class RgbdParams(C.Structure):
    _fields_ = [("levels", I), ("iters", I * MAX_LEVELS), ("min_gradient", F * MAX_LEVELS),
                ("max_depth_diff", F), ("max_depth", F)]


declare("tde_rgbd_prepare", I, [P, P, I, I, P, P, P])
declare("tde_rgbd_pyramid", I, [P, P, I, I, P, P, P])
declare("tde_rgbd_derivatives", I, [P, I, I, P, P, P])
declare("tde_rgbd_points_scratch_bytes", SZ, [I, I])
declare("tde_rgbd_points_of_interest", I, [P, P, I, I, F, P, SZ, P, U32, P, P])
declare("tde_rgbd_projective", I, [P, C.POINTER(Intrinsics), P])
declare("tde_rgbd_correspondences", I, [P, P, P, P, P, P, I, I, P, U32, P, F, F, F, P, P, P, P, P, P])
declare("tde_rgbd_lsm", I, [P, P, P, P, P, P, C.POINTER(Intrinsics), P, F, F, F, P, SZ, P, P, P])
declare("tde_rgbd_default_params", None, [C.POINTER(RgbdParams)])
declare("tde_rgbd_odometry_scratch_bytes", SZ, [I, I])
declare("tde_rgbd_odometry", I, [C.POINTER(RgbdFrameC), C.POINTER(RgbdFrameC), C.POINTER(Intrinsics),
                                 C.POINTER(RgbdParams), P, P, P, P, SZ, P])
declare("tde_synth_rgb", I, [P, I, P, C.POINTER(Intrinsics), P, P])

STATUS_SOLVE_FAILED, STATUS_SOLVED = 1, 2


def default_params(levels: int = MAX_LEVELS) -> RgbdParams:
    p = RgbdParams()
    lib.tde_rgbd_default_params(C.byref(p))
    p.levels = levels
    return p


def _stream(stream) -> int | None:
    if stream is None:
        return None
    return stream if isinstance(stream, int) else stream.cuda_stream


def projective(pose12, intr: Intrinsics) -> np.ndarray:
    """R' = K R K^-1, t' = K t (12 floats) of a pose at a level's camera."""
    out = np.zeros(12, np.float32)
    pose = np.ascontiguousarray(pose12, np.float64)
    check(lib.tde_rgbd_projective(pose.ctypes.data_as(P), C.byref(intr), out.ctypes.data_as(P)))
    return out


class RgbdFrame:
    """One frame's device pyramid: per level intensity (uint8), metric depth
    (float32) and, for frames that serve as the current one, Sobel dx, dy
    (int16)."""

    def __init__(self, cols: int, rows: int, levels: int = MAX_LEVELS, device="cuda"):
        import torch
        if not 1 <= levels <= MAX_LEVELS:
            raise ValueError(f"1 to {MAX_LEVELS} levels")
        self.cols, self.rows, self.levels = cols, rows, levels
        self.I, self.D, self.dx, self.dy = [], [], [], []
        for l in range(levels):
            h, w = rows >> l, cols >> l
            self.I.append(torch.empty((h, w), dtype=torch.uint8, device=device))
            self.D.append(torch.empty((h, w), dtype=torch.float32, device=device))
            self.dx.append(torch.empty((h, w), dtype=torch.int16, device=device))
            self.dy.append(torch.empty((h, w), dtype=torch.int16, device=device))

    def load(self, depth_mm, rgb, stream=None, derivatives: bool = True) -> "RgbdFrame":
        """Prepare_Data_For_RGBD, Generate_Intensity_And_Depth_Pyramid and
        Create_Intensity_Derivatives from device depth (uint16 mm, any 16-bit
        dtype) and RGB (uint8, rows x cols x 3)."""
        s = _stream(stream)
        if tuple(depth_mm.shape) != (self.rows, self.cols) or tuple(rgb.shape) != (self.rows, self.cols, 3):
            raise ValueError("depth must be rows x cols and rgb rows x cols x 3")
        if depth_mm.element_size() != 2 or rgb.element_size() != 1 or not (depth_mm.is_contiguous()
                                                                           and rgb.is_contiguous()):
            raise ValueError("contiguous 16-bit depth and 8-bit rgb expected")
        check(lib.tde_rgbd_prepare(depth_mm.data_ptr(), rgb.data_ptr(), self.cols, self.rows, self.I[0].data_ptr(),
                                   self.D[0].data_ptr(), s))
        for l in range(1, self.levels):
            check(lib.tde_rgbd_pyramid(self.I[l - 1].data_ptr(), self.D[l - 1].data_ptr(), self.cols >> (l - 1),
                                       self.rows >> (l - 1), self.I[l].data_ptr(), self.D[l].data_ptr(), s))
        if derivatives:
            for l in range(self.levels):
                check(lib.tde_rgbd_derivatives(self.I[l].data_ptr(), self.cols >> l, self.rows >> l,
                                               self.dx[l].data_ptr(), self.dy[l].data_ptr(), s))
        return self

    def c_struct(self) -> RgbdFrameC:
        f = RgbdFrameC()
        for l in range(self.levels):
            f.intensity[l] = self.I[l].data_ptr()
            f.depth[l] = self.D[l].data_ptr()
            f.dx[l] = self.dx[l].data_ptr()
            f.dy[l] = self.dy[l].data_ptr()
        return f


class RgbdOdometry:
    """Estimate_Isometry_By_RGBD: coarse-to-fine Gauss-Newton on the weighted
    photometric error.  Holds the scratch and the device pose and status."""

    def __init__(self, intr: Intrinsics, params: RgbdParams | None = None, device="cuda"):
        import torch
        self.intr = Intrinsics(intr.fx, intr.fy, intr.cx, intr.cy, intr.cols, intr.rows)
        self.params = params if params is not None else default_params()
        self.scratch_bytes = lib.tde_rgbd_odometry_scratch_bytes(intr.cols, intr.rows)
        self.scratch = torch.empty(self.scratch_bytes, dtype=torch.uint8, device=device)
        self.pose = torch.zeros(12, dtype=torch.float64, device=device)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)

    def enqueue(self, prev: RgbdFrame, curr: RgbdFrame, init_pose12=None, stream=None) -> None:
        """Launches only: the result is in self.pose / self.status when the
        stream reaches it."""
        if prev.levels < self.params.levels or curr.levels < self.params.levels:
            raise ValueError("frames have fewer levels than the parameters")
        init = None if init_pose12 is None else np.ascontiguousarray(init_pose12, np.float64)
        pc, cc = prev.c_struct(), curr.c_struct()
        check(lib.tde_rgbd_odometry(C.byref(pc), C.byref(cc), C.byref(self.intr), C.byref(self.params),
                                    None if init is None else init.ctypes.data_as(P), self.pose.data_ptr(),
                                    self.status.data_ptr(), self.scratch.data_ptr(), self.scratch_bytes,
                                    _stream(stream)))

    def estimate(self, prev: RgbdFrame, curr: RgbdFrame, init_pose12=None, stream=None):
        """(pose12 as numpy float64, status bits)."""
        import torch
        self.enqueue(prev, curr, init_pose12, stream)
        torch.cuda.synchronize()
        return self.pose.cpu().numpy(), int(self.status.item())


def points_of_interest(dx, dy, scale: float, stream=None):
    """Accumulate_Points_Of_Interest_For_RGBD: (N x 2 int32 tensor on the
    device, N) of pixels with dx^2 + dy^2 >= scale, raster order."""
    import torch
    h, w = dx.shape
    sb = lib.tde_rgbd_points_scratch_bytes(w, h)
    scratch = torch.empty(sb, dtype=torch.uint8, device=dx.device)
    pts = torch.empty((h * w, 2), dtype=torch.int32, device=dx.device)
    cnt = torch.zeros(1, dtype=torch.int32, device=dx.device)
    check(lib.tde_rgbd_points_of_interest(dx.data_ptr(), dy.data_ptr(), w, h, scale, scratch.data_ptr(), sb,
                                          pts.data_ptr(), h * w, cnt.data_ptr(), _stream(stream)))
    n = int(cnt.item())
    return pts[:n], n


def correspondences(prev: RgbdFrame, curr: RgbdFrame, level: int, pose12, intr0: Intrinsics, points=None,
                    min_gradient: float = 10.0, max_depth_diff: float = 0.07, max_depth: float = 35.0,
                    gradient_test: bool = True, stream=None):
    """Fill_List_Of_Valid_Correspondence_RGBD at one level: (corr_prev,
    corr_curr, diff, count, sum of squared differences).  points=None: every
    pixel of the level."""
    import torch
    intr = intr0.level(level)
    h, w = intr.rows, intr.cols
    npts = h * w if points is None else int(points.shape[0])
    dev = prev.I[level].device
    cp = torch.empty((max(npts, 1), 2), dtype=torch.int32, device=dev)
    cc = torch.empty_like(cp)
    diff = torch.empty(max(npts, 1), dtype=torch.float32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    s2 = torch.zeros(1, dtype=torch.float64, device=dev)
    proj = projective(pose12, intr)
    check(lib.tde_rgbd_correspondences(prev.I[level].data_ptr(), prev.D[level].data_ptr(), curr.I[level].data_ptr(),
                                       curr.D[level].data_ptr(),
                                       curr.dx[level].data_ptr() if gradient_test else None,
                                       curr.dy[level].data_ptr() if gradient_test else None, w, h,
                                       None if points is None else points.data_ptr(), npts, proj.ctypes.data_as(P),
                                       max_depth_diff, max_depth, min_gradient, cp.data_ptr(), cc.data_ptr(),
                                       diff.data_ptr(), cnt.data_ptr(), s2.data_ptr(), _stream(stream)))
    torch.cuda.synchronize()
    return cp[:npts], cc[:npts], diff[:npts], int(cnt.item()), float(s2.item())


def lsm(prev: RgbdFrame, curr: RgbdFrame, level: int, pose12, intr0: Intrinsics, min_gradient: float = 10.0,
        max_depth_diff: float = 0.07, max_depth: float = 35.0, stream=None):
    """Compute_Least_Squares_Equation at one level: (the 27 sums of [A | b]
    and the count as float64[28], sigma)."""
    import torch
    intr = intr0.level(level)
    dev = prev.I[level].device
    sb = lib.tde_rgbd_odometry_scratch_bytes(intr.cols, intr.rows)
    scratch = torch.empty(sb, dtype=torch.uint8, device=dev)
    sums = torch.zeros(28, dtype=torch.float64, device=dev)
    sigma = torch.zeros(1, dtype=torch.float32, device=dev)
    pose = np.ascontiguousarray(pose12, np.float64)
    check(lib.tde_rgbd_lsm(prev.I[level].data_ptr(), prev.D[level].data_ptr(), curr.I[level].data_ptr(),
                           curr.D[level].data_ptr(), curr.dx[level].data_ptr(), curr.dy[level].data_ptr(),
                           C.byref(intr), pose.ctypes.data_as(P), max_depth_diff, max_depth, min_gradient,
                           scratch.data_ptr(), sb, sums.data_ptr(), sigma.data_ptr(), _stream(stream)))
    torch.cuda.synchronize()
    return sums.cpu().numpy(), float(sigma.item())


def synth_rgb(d_scene, nprim: int, pose12, intr: Intrinsics, out, stream=None) -> None:
    """The synthetic colour camera: the scene's procedural texture (device
    scene, nprim x 8 doubles) from pose12 into out (rows x cols x 3 uint8)."""
    pose = np.ascontiguousarray(pose12, np.float64)
    check(lib.tde_synth_rgb(d_scene.data_ptr(), nprim, pose.ctypes.data_as(P), C.byref(intr), out.data_ptr(),
                            _stream(stream)))


class RgbdTracker:
    """Frame-to-frame RGB-D odometry over a stream of frames: each track()
    copies the frame into a fixed input slot, builds its pyramid and, from
    the second frame on, estimates the pose against the previous frame.  The
    per-frame launches (8 for the pyramid, 1 + 2 per Gauss-Newton step) are
    captured once per buffer parity in CUDA graphs and replayed.  Results:
    self.pose (device float64[12], previous -> current camera) and
    self.status (device int32[1]) after each frame."""

    def __init__(self, intr: Intrinsics, params: RgbdParams | None = None, device="cuda", graphs: bool = True):
        import torch
        self.torch = torch
        self.params = params if params is not None else default_params()
        L = self.params.levels
        self.bufs = [RgbdFrame(intr.cols, intr.rows, L, device) for _ in range(2)]
        self.od = RgbdOdometry(intr, self.params, device)
        self.depth_slot = torch.empty((intr.rows, intr.cols), dtype=torch.int16, device=device)
        self.rgb_slot = torch.empty((intr.rows, intr.cols, 3), dtype=torch.uint8, device=device)
        self.stream = torch.cuda.Stream(device)
        self.frames = 0
        self.graphs = None
        if graphs:
            self.graphs = []
            for p in (0, 1):
                g = torch.cuda.CUDAGraph()
                self.stream.synchronize()
                with torch.cuda.graph(g, stream=self.stream):
                    self._frame_step(p)
                self.graphs.append(g)
            torch.cuda.synchronize()

    @property
    def pose(self):
        return self.od.pose

    @property
    def status(self):
        return self.od.status

    def _frame_step(self, p: int) -> None:
        s = self.torch.cuda.current_stream()
        self.bufs[p].load(self.depth_slot, self.rgb_slot, s)
        self.od.enqueue(self.bufs[1 - p], self.bufs[p], None, s)

    def track(self, depth_mm, rgb) -> None:
        """Enqueue one frame (device uint16 mm and rows x cols x 3 RGB) on
        self.stream.  The first frame only fills the pyramid."""
        torch = self.torch
        p = self.frames & 1
        with torch.cuda.stream(self.stream):
            self.depth_slot.copy_(depth_mm.view(torch.int16), non_blocking=True)
            self.rgb_slot.copy_(rgb, non_blocking=True)
            if self.frames == 0:
                self.bufs[p].load(self.depth_slot, self.rgb_slot, self.stream)
            elif self.graphs is not None:
                self.graphs[p].replay()
            else:
                self._frame_step(p)
        self.frames += 1
