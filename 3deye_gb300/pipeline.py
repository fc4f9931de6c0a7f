"""Host-side handle of the per-frame pipeline (include/tde_pipeline.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import Intrinsics, LightSource, Point3f, Point3i, RoundBuffer, check, declare, lib

P, I, F = C.c_void_p, C.c_int, C.c_float


class PipelineConfig(C.Structure):
    _fields_ = [("intr", Intrinsics), ("voxels", Point3i), ("volume_size", Point3f), ("tsdf_format", I),
                ("trunc", F), ("max_weight", I), ("sigma_space", F), ("sigma_color", F),
                ("max_depth_mm", C.c_uint32), ("icp_levels", I), ("icp_iters", I * 3), ("dist_thresh", F),
                ("angle_thresh", F), ("use_graphs", I), ("integrate_stats", I)]


declare("tde_pipeline_create", I, [C.POINTER(PipelineConfig), P, C.POINTER(P)])
declare("tde_pipeline_destroy", I, [P])
declare("tde_pipeline_stream", P, [P])
declare("tde_pipeline_enqueue", I, [P, P, I, P, P])
declare("tde_pipeline_sync", I, [P])
declare("tde_pipeline_process", I, [P, P, I, P, P])
declare("tde_pipeline_pose", I, [P, P])
declare("tde_pipeline_volume", I, [P, C.POINTER(P), C.POINTER(RoundBuffer)])
declare("tde_pipeline_model_maps", I, [P, I, C.POINTER(P), C.POINTER(P)])
declare("tde_pipeline_frame_maps", I, [P, I, C.POINTER(P), C.POINTER(P), C.POINTER(P)])
declare("tde_pipeline_frame_count", I, [P])
declare("tde_pipeline_enable_timing", I, [P, I])
declare("tde_pipeline_timings", I, [P, P, P, I])
declare("tde_pipeline_integrate_stats", I, [P, P, I])
declare("tde_pipeline_stage_timings", I, [P, P, I])
declare("tde_pipeline_launches_per_frame", I, [P])
declare("tde_pipeline_set_round_buffer", I, [P, C.POINTER(RoundBuffer)])
declare("tde_pipeline_set_pose", I, [P, P])
declare("tde_pipeline_set_refiner", I, [P, P])
declare("tde_pipeline_model_depth", I, [P, P])
declare("tde_pipeline_raycast_records", I, [P, I, C.POINTER(C.c_uint64)])
declare("tde_pipeline_shift_needed", I, [P, F, F, P])
declare("tde_pipeline_shift", I, [P, P, P, P, C.c_uint32, C.POINTER(C.c_uint32)])
declare("tde_pipeline_shift_ex", I, [P, P, P, P, P, C.c_uint32, C.POINTER(C.c_uint32)])
declare("tde_pipeline_extract_volume", I, [P, P, P, P, C.c_uint32, C.POINTER(C.c_uint32)])
declare("tde_pipeline_render", I, [P, P, P])
declare("tde_pipeline_shift_needed_pose", I, [P, P, C.c_float, C.c_float, P])
declare("tde_pipeline_checkpoint_bytes", C.c_size_t, [P])
declare("tde_pipeline_checkpoint", I, [P, P, C.c_size_t])
declare("tde_pipeline_restore", I, [P, P, C.c_size_t])
declare("tde_pipeline_enqueue_rgbd", I, [P, P, P, I, P, P])
declare("tde_pipeline_enable_color", I, [P, I])
declare("tde_pipeline_color_volume", I, [P, C.POINTER(P)])


def config_from(cfg, use_graphs=True, integrate_stats=False, levels=3) -> PipelineConfig:
    c = PipelineConfig()
    c.intr = Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    c.voxels = Point3i(cfg.voxels, cfg.voxels, cfg.voxels)
    c.volume_size = Point3f(cfg.volume_m, cfg.volume_m, cfg.volume_m)
    c.tsdf_format = cfg.tsdf_format
    c.trunc = cfg.trunc_m
    c.max_weight = cfg.max_weight
    c.sigma_space = cfg.sigma_space
    c.sigma_color = cfg.sigma_color
    c.max_depth_mm = cfg.max_depth_mm
    c.icp_levels = levels
    for l in range(3):
        c.icp_iters[l] = cfg.icp_iters[l] if l < len(cfg.icp_iters) else 0
    c.dist_thresh = cfg.dist_thresh
    c.angle_thresh = cfg.angle_thresh
    c.use_graphs = int(use_graphs)
    c.integrate_stats = int(integrate_stats)
    return c


class Pipeline:
    """One KinectFusion reconstruction on the current CUDA device."""

    def __init__(self, cfg, pose12, use_graphs=True, integrate_stats=False):
        self.cfg = cfg
        self._c = config_from(cfg, use_graphs, integrate_stats)
        self._h = P()
        pose = np.ascontiguousarray(pose12, np.float64)
        check(lib.tde_pipeline_create(C.byref(self._c), pose.ctypes.data_as(P), C.byref(self._h)))

    def close(self):
        if self._h:
            lib.tde_pipeline_destroy(self._h)
            self._h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib.tde_pipeline_stream(self._h)

    def enqueue(self, depth_ptr: int, on_device: bool, pose_out_ptr=None, status_out_ptr=None):
        check(lib.tde_pipeline_enqueue(self._h, depth_ptr, int(on_device), pose_out_ptr, status_out_ptr))

    def process(self, depth) -> tuple[np.ndarray, int]:
        """Blocking: depth is a numpy uint16 array or a CUDA tensor."""
        pose = np.zeros(12, np.float64)
        st = C.c_int()
        if isinstance(depth, np.ndarray):
            d = np.ascontiguousarray(depth, np.uint16)
            check(lib.tde_pipeline_process(self._h, d.ctypes.data_as(P), 0, pose.ctypes.data_as(P), C.byref(st)))
        else:
            check(lib.tde_pipeline_process(self._h, depth.data_ptr(), 1, pose.ctypes.data_as(P), C.byref(st)))
        return pose, st.value

    def enable_color(self, max_weight: int = 255):
        """Adds a colour volume; every frame then needs an RGB image (enqueue_rgbd / process_rgbd)."""
        check(lib.tde_pipeline_enable_color(self._h, max_weight))

    def enqueue_rgbd(self, depth_ptr: int, rgb_ptr: int, on_device: bool, pose_out_ptr=None, status_out_ptr=None):
        check(lib.tde_pipeline_enqueue_rgbd(self._h, depth_ptr, rgb_ptr, int(on_device), pose_out_ptr, status_out_ptr))

    def process_rgbd(self, depth: np.ndarray, rgb: np.ndarray) -> tuple[np.ndarray, int]:
        """Blocking RGB-D frame from host arrays: depth uint16 [rows, cols], rgb uint8 [rows, cols, 3]."""
        d = np.ascontiguousarray(depth, np.uint16)
        c = np.ascontiguousarray(rgb, np.uint8)
        pose = np.zeros(12, np.float64)
        st = np.zeros(1, np.int32)
        check(lib.tde_pipeline_enqueue_rgbd(self._h, d.ctypes.data_as(P), c.ctypes.data_as(P), 0,
                                            pose.ctypes.data_as(P), st.ctypes.data_as(P)))
        self.sync()
        return pose, int(st[0])

    def color_volume(self) -> int:
        v = P()
        check(lib.tde_pipeline_color_volume(self._h, C.byref(v)))
        return v.value

    def sync(self):
        check(lib.tde_pipeline_sync(self._h))

    def pose(self) -> np.ndarray:
        out = np.zeros(12, np.float64)
        check(lib.tde_pipeline_pose(self._h, out.ctypes.data_as(P)))
        return out

    def volume(self):
        v, rb = P(), RoundBuffer()
        check(lib.tde_pipeline_volume(self._h, C.byref(v), C.byref(rb)))
        return v.value, rb

    def model_maps(self, level=0):
        v, n = P(), P()
        check(lib.tde_pipeline_model_maps(self._h, level, C.byref(v), C.byref(n)))
        return v.value, n.value

    def frame_maps(self, level=0):
        d, v, n = P(), P(), P()
        check(lib.tde_pipeline_frame_maps(self._h, level, C.byref(d), C.byref(v), C.byref(n)))
        return d.value, v.value, n.value

    def enable_timing(self, capacity: int):
        check(lib.tde_pipeline_enable_timing(self._h, capacity))

    def timings(self, capacity: int):
        a = np.zeros(capacity, np.float32)
        b = np.zeros(capacity, np.float32)
        n = lib.tde_pipeline_timings(self._h, a.ctypes.data_as(P), b.ctypes.data_as(P), capacity)
        if n < 0:
            check(n)
        return a[:n], b[:n]

    STAGES = ("preprocess", "icp", "integrate", "raycast", "model_pyramid")

    def stage_timings(self, capacity: int) -> dict:
        """Milliseconds per timed frame of each stage (STAGES), as arrays."""
        a = np.zeros((capacity, len(self.STAGES)), np.float32)
        n = lib.tde_pipeline_stage_timings(self._h, a.ctypes.data_as(P), capacity)
        if n < 0:
            check(n)
        return {k: a[:n, i] for i, k in enumerate(self.STAGES)}

    def integrate_stats(self, reset=False, bricks=False):
        out = np.zeros(3, np.uint64)
        check(lib.tde_pipeline_integrate_stats(self._h, out.ctypes.data_as(P), int(reset)))
        if bricks:
            return int(out[0]), int(out[1]), int(out[2])
        return int(out[0]), int(out[1])

    def launches_per_frame(self) -> int:
        return lib.tde_pipeline_launches_per_frame(self._h)

    def set_round_buffer(self, rb: RoundBuffer):
        check(lib.tde_pipeline_set_round_buffer(self._h, C.byref(rb)))

    def set_pose(self, pose12):
        p = np.ascontiguousarray(pose12, np.float64)
        check(lib.tde_pipeline_set_pose(self._h, p.ctypes.data_as(P)))

    def set_refiner(self, refiner):
        """Learned refinement instead of the bilateral filter (None restores it)."""
        self._refiner = refiner  # keeps it alive while the pipeline uses it
        check(lib.tde_pipeline_set_refiner(self._h, refiner.handle if refiner is not None else None))

    def shift_needed(self, radius_m: float, ahead_m: float | None = None) -> np.ndarray:
        """Voxel shift re-centring the volume on the point ahead_m (default: half
        the volume) in front of the camera; zeros while it is within radius_m."""
        if ahead_m is None:
            ahead_m = 0.5 * self.cfg.volume_m
        d = np.zeros(3, np.int32)
        check(lib.tde_pipeline_shift_needed(self._h, ahead_m, radius_m, d.ctypes.data_as(P)))
        return d

    def shift_needed_for(self, pose12, radius_m: float, ahead_m: float | None = None) -> np.ndarray:
        """shift_needed for a given pose (current volume frame), without waiting for the GPU."""
        if ahead_m is None:
            ahead_m = 0.5 * self.cfg.volume_m
        pose = np.ascontiguousarray(pose12, np.float64)
        d = np.zeros(3, np.int32)
        check(lib.tde_pipeline_shift_needed_pose(self._h, pose.ctypes.data_as(P), ahead_m, radius_m,
                                                 d.ctypes.data_as(P)))
        return d

    def shift(self, delta, capacity: int = 1 << 22):
        """Shift the volume by delta voxels; returns the outgoing slab's points
        [n,4] (logical voxel units before the shift) and their weights."""
        pts, w, _, n = self.shift_colors(delta, capacity)
        return pts, w, n

    def shift_colors(self, delta, capacity: int = 1 << 22):
        """As shift, and the points' colours uint8 [n, 4] (zeros without a colour volume)."""
        d = np.ascontiguousarray(delta, np.int32)
        pts = np.zeros((capacity, 4), np.float32)
        w = np.zeros(capacity, np.float32)
        col = np.zeros((capacity, 4), np.uint8)
        n = C.c_uint32()
        check(lib.tde_pipeline_shift_ex(self._h, d.ctypes.data_as(P), pts.ctypes.data_as(P), w.ctypes.data_as(P),
                                        col.ctypes.data_as(P), capacity, C.byref(n)))
        k = min(n.value, capacity)
        return pts[:k], w[:k], col[:k], n.value

    def extract_volume(self, capacity: int | None = None):
        """The whole model as zero-crossing points (Extract_Tsdf_Volume):
        metric voxel centres [n, 4] in the volume frame, their weights and,
        with a colour volume, colours uint8 [n, 4] (zeros without one).
        Without `capacity` the buffers are sized from a count pass."""
        n = C.c_uint32()
        if capacity is None:
            check(lib.tde_pipeline_extract_volume(self._h, None, None, None, 0, C.byref(n)))
            capacity = n.value
        pts = np.zeros((max(capacity, 1), 4), np.float32)
        w = np.zeros(max(capacity, 1), np.float32)
        col = np.zeros((max(capacity, 1), 4), np.uint8)
        check(lib.tde_pipeline_extract_volume(self._h, pts.ctypes.data_as(P), w.ctypes.data_as(P),
                                              col.ctypes.data_as(P), capacity, C.byref(n)))
        k = min(n.value, capacity)
        return pts[:k], w[:k], col[:k], n.value

    def render(self, image_ptr: int, light_pos=None):
        """Enqueue Generate_Image of the current model into a device buffer
        of cols*rows*3 bytes; light at the camera centre unless light_pos."""
        light = None if light_pos is None else C.byref(LightSource(Point3f(*light_pos), 1))
        check(lib.tde_pipeline_render(self._h, light, image_ptr))

    def checkpoint(self) -> np.ndarray:
        """The state the next frame depends on, as bytes (see tde_pipeline_checkpoint)."""
        n = lib.tde_pipeline_checkpoint_bytes(self._h)
        buf = np.empty(n, np.uint8)
        check(lib.tde_pipeline_checkpoint(self._h, buf.ctypes.data_as(P), n))
        return buf

    def restore(self, buf) -> None:
        """Continue from a checkpoint of a pipeline with the same configuration."""
        b = np.ascontiguousarray(buf, np.uint8)
        check(lib.tde_pipeline_restore(self._h, b.ctypes.data_as(P), b.size))

    def save(self, path) -> None:
        self.checkpoint().tofile(path)

    def load(self, path) -> None:
        self.restore(np.fromfile(path, np.uint8))

    def world_cloud(self, points):
        """Volume-frame points (as extract_volume returns them) in the world
        frame: plus the round buffer's origin_metric."""
        _, rb = self.volume()
        out = np.array(points, np.float32, copy=True)
        out[:, :3] += np.array([rb.origin_metric.x, rb.origin_metric.y, rb.origin_metric.z], np.float32)
        return out

    def raycast_records(self, skip_empty: bool = True) -> int:
        """Distinct voxel records a raycast of the current model reads."""
        n = C.c_uint64()
        check(lib.tde_pipeline_raycast_records(self._h, int(skip_empty), C.byref(n)))
        return n.value

    def model_depth(self, out_ptr: int):
        """Enqueue: the last frame's model surface as depth in mm (device uint16)."""
        check(lib.tde_pipeline_model_depth(self._h, out_ptr))


def ate_rmse(est: np.ndarray, gt: np.ndarray, align: bool = False) -> float:
    """Absolute trajectory error (Sturm et al. 2012): RMS of camera-centre
    differences, optionally after a least-squares rigid alignment (Horn)."""
    a = np.asarray(est)[:, 9:12]
    b = np.asarray(gt)[:, 9:12]
    if align:
        ma, mb = a.mean(0), b.mean(0)
        H = (a - ma).T @ (b - mb)
        U, _, Vt = np.linalg.svd(H)
        D = np.diag([1, 1, np.sign(np.linalg.det(Vt.T @ U.T))])
        R = Vt.T @ D @ U.T
        a = (R @ (a - ma).T).T + mb
    return float(np.sqrt(np.mean(np.sum((a - b) ** 2, axis=1))))
