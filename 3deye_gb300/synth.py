"""Seeded synthetic sequences standing in for the Kinect sensor.

No public dataset is named for this pipeline; the workloads are procedural:
a ground plane with random spheres and axis-aligned boxes, seen from a smooth
random orbit (scene seed 1000+k, trajectory seed 2000+k, noise seed 3000+k),
with the Kinect axial noise model sigma = 0.0012 + 0.0019 (z - 0.4)^2 m, 1 mm
quantisation, 2 % dropout and no depth beyond 4 m.

Frame conventions: the world frame is the TSDF volume frame, spanning
[0, V]^3; y points down (the ground plane is y = const); a camera looks along
its +z axis with image v growing along its +y axis.  Poses are (R, t) with R
mapping camera to world and t the camera centre.

Scene encoding (8 doubles per primitive) is the one of oracle_scene.c and the
GPU sensor (k_synth.cu): [type, a0..a6], type 0 plane (n, d), 1 sphere (c, r),
2 box (min, max).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass(frozen=True)
class Config:
    name: str
    frames: int
    cols: int
    rows: int
    fx: float
    fy: float
    cx: float
    cy: float
    voxels: int
    volume_m: float
    tsdf_format: int            # 0 int16, 1 fp16, 2 fp32
    trunc_m: float
    sigma_space: float
    sigma_color: float
    icp_iters: tuple = (10, 5, 4)
    max_weight: int = 128
    dist_thresh: float = 0.1
    angle_thresh: float = math.sin(math.radians(20.0))
    scene_cube_m: float = 2.0
    max_depth_mm: int = 4000

    @property
    def cell(self) -> float:
        return self.volume_m / self.voxels


# Workloads of the benchmark definition (frames x resolution, volume, storage).
CONFIGS = {
    # 100 x 320x240, 128^3 FP32 over 2 m, truncation 3 voxels, sigma_s 4 px
    "c1": Config("c1-320x240-128^3-fp32", 100, 320, 240, 262.5, 262.5, 159.5, 119.5, 128, 2.0, 2,
                 3 * 2.0 / 128, 4.0, 30.0, scene_cube_m=2.0),
    # 600 x 640x480, 512^3 FP16+u16 over 3 m
    "c2": Config("c2-640x480-512^3-fp16", 600, 640, 480, 525.0, 525.0, 319.5, 239.5, 512, 3.0, 1,
                 0.03, 4.5, 30.0, scene_cube_m=3.0),
    # 600 x 640x480 along a 12 m corridor, 512^3 FP16+u16 over 3 m following the camera
    "c3": Config("c3-640x480-512^3-corridor", 600, 640, 480, 525.0, 525.0, 319.5, 239.5, 512, 3.0, 1,
                 0.03, 4.5, 30.0, scene_cube_m=3.0),
    # 300 x 640x480 of the c1 scene, 1024^3 over 4 m (precision study)
    "c4": Config("c4-640x480-1024^3", 300, 640, 480, 525.0, 525.0, 319.5, 239.5, 1024, 4.0, 1,
                 3 * 4.0 / 1024, 4.5, 30.0, scene_cube_m=2.0),
}


def small_config(base: str = "c1", frames: int = 20, cols: int = 160, rows: int = 120, voxels: int = 64,
                 fmt: int | None = None) -> Config:
    """A reduced copy of a workload for tests (same scene and noise model)."""
    c = CONFIGS[base]
    s = cols / c.cols
    return dataclasses.replace(c, name=f"{c.name}-small", frames=frames, cols=cols, rows=rows, fx=c.fx * s,
                               fy=c.fy * s, cx=(cols - 1) / 2.0, cy=(rows - 1) / 2.0, voxels=voxels,
                               tsdf_format=c.tsdf_format if fmt is None else fmt,
                               trunc_m=max(c.trunc_m, 3 * c.volume_m / voxels))


def make_scene(cfg: Config, seed: int) -> np.ndarray:
    """Ground plane + 20 spheres (r 0.1-0.4 m) + 10 boxes (0.2-0.6 m) in a
    cube of cfg.scene_cube_m centred in the volume."""
    rng = np.random.default_rng(seed)
    V = cfg.volume_m
    c = V / 2.0
    half = cfg.scene_cube_m / 2.0
    y_ground = c + 0.5 * half
    prims = [[0, 0.0, 1.0, 0.0, -y_ground, 0, 0, 0]]  # plane y = y_ground
    reach = 0.7 * half
    for _ in range(20):
        r = rng.uniform(0.1, 0.4) * cfg.scene_cube_m / 2.0
        ang, rad = rng.uniform(0, 2 * np.pi), reach * np.sqrt(rng.uniform(0, 1))
        x, z = c + rad * np.cos(ang), c + rad * np.sin(ang)
        y = y_ground - r - rng.uniform(0.0, 0.6) * half
        prims.append([1, x, y, z, r, 0, 0, 0])
    for _ in range(10):
        sz = rng.uniform(0.2, 0.6, size=3) * cfg.scene_cube_m / 2.0
        ang, rad = rng.uniform(0, 2 * np.pi), reach * np.sqrt(rng.uniform(0, 1))
        x, z = c + rad * np.cos(ang), c + rad * np.sin(ang)
        ymax = y_ground
        prims.append([2, x - sz[0] / 2, ymax - sz[1], z - sz[2] / 2, x + sz[0] / 2, ymax, z + sz[2] / 2, 0])
    return np.asarray(prims, dtype=np.float64)


def look_at(eye: np.ndarray, target: np.ndarray, down=np.array([0.0, 1.0, 0.0])) -> np.ndarray:
    """Camera->world rotation for a camera at `eye` looking at `target`."""
    zc = target - eye
    zc = zc / np.linalg.norm(zc)
    xc = np.cross(down, zc)
    xc = xc / np.linalg.norm(xc)
    yc = np.cross(zc, xc)
    return np.stack([xc, yc, zc], axis=1)


def make_trajectory(cfg: Config, seed: int, frames: int | None = None) -> np.ndarray:
    """Smooth random orbit at 1.2-1.8 m (scaled by the cube), <= 2 cm and
    <= 1 degree per frame.  Returns (frames, 12) float64: R row-major, t."""
    n = cfg.frames if frames is None else frames
    rng = np.random.default_rng(seed)
    V = cfg.volume_m
    c = V / 2.0
    half = cfg.scene_cube_m / 2.0
    s = cfg.scene_cube_m / 2.0
    y_ground = c + 0.5 * half
    k = np.arange(n, dtype=np.float64)
    ph = rng.uniform(0, 2 * np.pi, size=8)
    fr = rng.uniform(0.005, 0.02, size=8)
    radius = s * (1.5 + 0.25 * np.sin(fr[0] * k + ph[0]) + 0.05 * np.sin(fr[1] * k + ph[1]))
    height = s * (0.65 + 0.15 * np.sin(fr[2] * k + ph[2]))
    dtheta = math.radians(0.3) * (1.0 + 0.3 * np.sin(fr[3] * k + ph[3]))
    theta = ph[4] + np.cumsum(dtheta) - dtheta[0]
    eye = np.stack([c + radius * np.cos(theta), y_ground - height, c + radius * np.sin(theta)], axis=1)
    tgt = np.stack([c + 0.15 * s * np.sin(fr[5] * k + ph[5]), y_ground - 0.35 * s + 0.05 * s * np.sin(fr[6] * k),
                    c + 0.15 * s * np.cos(fr[7] * k + ph[7])], axis=1)
    out = np.empty((n, 12), np.float64)
    for i in range(n):
        R = look_at(eye[i], tgt[i])
        out[i, :9] = R.ravel()
        out[i, 9:] = eye[i]
    return out


# ---------------------------------------------------------------------------
# Corridor (cyclic-volume workload): the camera travels `length` metres along
# +z through a tiled corridor while the volume follows it.
# ---------------------------------------------------------------------------
CORRIDOR_HALF_WIDTH = 1.1   # walls at x = V/2 +- this
CORRIDOR_FLOOR = 1.2        # floor this far below the camera line (y down)
CORRIDOR_CEILING = 1.0      # ceiling this far above it


def make_corridor_scene(cfg: Config, seed: int, length: float = 12.0) -> np.ndarray:
    """Floor, ceiling and two walls (planes) plus a random box every 0.5 m,
    alternating walls, from the start of the walk (the volume's rear face,
    z = 0) to beyond its end."""
    rng = np.random.default_rng(seed)
    c = cfg.volume_m / 2.0
    y_floor, y_ceil = c + CORRIDOR_FLOOR, c - CORRIDOR_CEILING
    xl, xr = c - CORRIDOR_HALF_WIDTH, c + CORRIDOR_HALF_WIDTH
    prims = [[0, 0.0, 1.0, 0.0, -y_floor, 0, 0, 0], [0, 0.0, 1.0, 0.0, -y_ceil, 0, 0, 0],
             [0, 1.0, 0.0, 0.0, -xl, 0, 0, 0], [0, 1.0, 0.0, 0.0, -xr, 0, 0, 0]]
    z = 0.5
    side = 1
    while z < length + cfg.volume_m + 4.5:
        w, h, d = rng.uniform(0.2, 0.5, size=3)
        zz = z + rng.uniform(-0.1, 0.1)
        if side > 0:
            x0, x1 = xr - w, xr
        else:
            x0, x1 = xl, xl + w
        if rng.uniform() < 0.6:      # on the floor
            y0, y1 = y_floor - h, y_floor
        else:                        # on the wall, at some height
            ym = rng.uniform(y_ceil + 0.3, y_floor - 0.3)
            y0, y1 = ym - h / 2, ym + h / 2
        prims.append([2, x0, y0, zz - d / 2, x1, y1, zz + d / 2, 0])
        side = -side
        z += 0.5
    return np.asarray(prims, dtype=np.float64)


def make_corridor_trajectory(cfg: Config, seed: int, frames: int | None = None, length: float = 12.0) -> np.ndarray:
    """Walk along +z from the volume's rear face (z = 0, the volume ahead of
    the camera) over `length` metres (2 cm per frame for 600 frames), with
    slow lateral / vertical sway and a gently wandering gaze ahead.  Returns
    (frames, 12) float64: R row-major, t."""
    n = cfg.frames if frames is None else frames
    rng = np.random.default_rng(seed)
    c = cfg.volume_m / 2.0
    k = np.arange(n, dtype=np.float64)
    ph = rng.uniform(0, 2 * np.pi, size=6)
    fr = rng.uniform(0.01, 0.03, size=6)
    zc = length * k / max(n - 1, 1)
    eye = np.stack([c + 0.15 * np.sin(fr[0] * k + ph[0]), c + 0.08 * np.sin(fr[1] * k + ph[1]), zc], axis=1)
    tgt = np.stack([c + 0.4 * np.sin(fr[2] * k + ph[2]), c + 0.3 + 0.15 * np.sin(fr[3] * k + ph[3]), zc + 2.0], axis=1)
    out = np.empty((n, 12), np.float64)
    for i in range(n):
        out[i, :9] = look_at(eye[i], tgt[i]).ravel()
        out[i, 9:] = eye[i]
    return out


def intrinsics_tuple(cfg: Config):
    return (cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)


def seeds(k: int = 0):
    return 1000 + k, 2000 + k, 3000 + k
