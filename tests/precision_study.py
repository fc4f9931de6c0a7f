"""TSDF storage precision study: the GPU pipeline with FP32, FP16 and int16
TSDF storage against a full-FP64 oracle run of the same frames (FP64 TSDF,
integration, raycast, ICP terms and solve; oracle/pipeline.py).

Reported per storage format: the TSDF field on voxels both runs observed
(mean / max |f - f64|, and the same in millimetres, f being the TSDF
normalised to the truncation; sign disagreements), the model raycast from the
oracle's final pose (depth along the optical axis, normal angle), the
per-frame camera positions against the oracle's, and ATE against the ground
truth and against the oracle.

    python tests/precision_study.py --config c4 --frames 300 --out precision_c4.json

The workload defaults to the 1024^3 / 4 m volume, 640x480, with the config-1
scene.  TEST INFRASTRUCTURE: it runs the CPU oracle as the reference.
"""
from __future__ import annotations

import argparse
import ctypes as C
import dataclasses
import importlib
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402
from oracle.pipeline import OraclePipelineF64  # noqa: E402

tde = importlib.import_module("3deye_gb300")
syn = importlib.import_module("3deye_gb300.synth")
pl = importlib.import_module("3deye_gb300.pipeline")
learned = importlib.import_module("3deye_gb300.learned")

FORMAT_NAMES = {0: "int16", 1: "fp16", 2: "fp32"}


def decode(raw: np.ndarray, fmt: int, n: int):
    """Volume bytes -> (f float64 [n], weight int [n])."""
    if fmt == 0:
        rec = raw[: 4 * n].view(np.int16).reshape(n, 2)
        return rec[:, 0].astype(np.float64) / 32767.0, rec[:, 1].astype(np.int64)
    if fmt == 1:
        rec = raw[: 4 * n].view(np.uint16).reshape(n, 2)
        return rec[:, 0].copy().view(np.float16).astype(np.float64), rec[:, 1].astype(np.int64)
    f = raw[: 4 * n].view(np.float32).astype(np.float64)
    w = raw[4 * n: 6 * n].view(np.uint16).astype(np.int64)
    return f, w


def download(ptr: int, nbytes: int) -> np.ndarray:
    out = np.empty(nbytes, np.uint8)
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    tde.check(tde.lib.tde_memcpy(out.ctypes.data_as(C.c_void_p), ptr, nbytes, 1))
    return out


def model_depth(vmap, R, t):
    """Depth along the optical axis of a vertex map (NaN where no hit)."""
    return (vmap - t) @ R[:, 2]


def study(cfg, seed_k: int = 0, formats=(2, 1, 0), log=print) -> dict:
    import torch
    frames, traj, _, _ = learned.render_sequence(cfg, seed_k, cfg.frames)
    host = frames.cpu().numpy().view(np.uint16)
    t0 = time.time()
    ref = OraclePipelineF64(cfg, traj[0])
    ref_poses = np.array([ref.process(host[i]) for i in range(cfg.frames)])
    log(f"FP64 oracle: {cfg.frames} frames in {time.time() - t0:.1f} s")
    n = cfg.voxels ** 3
    Rf, tf = ref.R, ref.t
    zf = model_depth(ref.vmod[0], Rf, tf)
    nf = ref.nmod[0]
    out = {"workload": f"{cfg.cols}x{cfg.rows}, {cfg.voxels}^3 over {cfg.volume_m} m, {cfg.frames} frames, seed {seed_k}",
           "oracle": {"ate_vs_gt_m": pl.ate_rmse(ref_poses, traj), "frames_lost": int(sum(ref.lost))}}
    intr = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    c = float(cfg.volume_m / cfg.voxels)
    cell = tde.vec3([c, c, c])
    for fmt in formats:
        fc = dataclasses.replace(cfg, tsdf_format=fmt)
        p = pl.Pipeline(fc, traj[0])
        poses = []
        base, fb = frames.data_ptr(), cfg.rows * cfg.cols * 2
        for i in range(cfg.frames):
            p.enqueue(base + i * fb, True)
            poses.append(p.pose())
        poses = np.array(poses)
        vol, rb = p.volume()
        f, w = decode(download(vol, int(tde.lib.tde_tsdf_volume_bytes(fmt, C.byref(rb)))), fmt, n)
        both = (w > 0) & (ref.weight > 0)
        d = np.abs(f[both] - ref.tsdf[both])
        sign = np.mean(np.sign(f[both]) != np.sign(ref.tsdf[both])) if both.any() else 0.0
        # raycast of this volume from the oracle's final pose
        vm = torch.empty((cfg.rows, cfg.cols, 3), dtype=torch.float32, device="cuda")
        nm = torch.empty_like(vm)
        tde.check(tde.lib.tde_raycast(C.c_void_p(vol), fmt, C.c_void_p(vm.data_ptr()), C.c_void_p(nm.data_ptr()),
                                      C.byref(tde.vec3(tf)), C.byref(tde.mat3(Rf)), C.c_float(cfg.trunc_m),
                                      C.byref(intr), C.byref(rb), C.byref(cell), None))
        torch.cuda.synchronize()
        vmh, nmh = vm.cpu().numpy().astype(np.float64), nm.cpu().numpy().astype(np.float64)
        zg = model_depth(vmh, Rf, tf)
        hit = np.isfinite(zg) & np.isfinite(zf)
        dz = np.abs(zg[hit] - zf[hit])
        nh = hit & np.isfinite(nmh[..., 0]) & np.isfinite(nf[..., 0])
        cosang = np.clip(np.sum(nmh[nh] * nf[nh], axis=-1), -1.0, 1.0)
        ang = np.degrees(np.arccos(cosang))
        dp = np.linalg.norm(poses[:, 9:] - ref_poses[:, 9:], axis=1)
        out[FORMAT_NAMES[fmt]] = {
            "tsdf_voxels_compared": int(both.sum()),
            "tsdf_abs_err_mean": float(d.mean()), "tsdf_abs_err_max": float(d.max()),
            "tsdf_abs_err_mean_mm": float(d.mean() * cfg.trunc_m * 1e3),
            "tsdf_sign_disagreement": float(sign),
            "raycast_pixels_compared": int(hit.sum()),
            "raycast_hit_agreement": float(np.mean(np.isfinite(zg) == np.isfinite(zf))),
            "raycast_depth_err_mean_mm": float(dz.mean() * 1e3), "raycast_depth_err_p99_mm": float(np.percentile(dz, 99) * 1e3),
            "normal_err_mean_deg": float(ang.mean()), "normal_err_p99_deg": float(np.percentile(ang, 99)),
            "pose_err_mean_mm": float(dp.mean() * 1e3), "pose_err_max_mm": float(dp.max() * 1e3),
            "ate_vs_oracle_m": pl.ate_rmse(poses, ref_poses), "ate_vs_gt_m": pl.ate_rmse(poses, traj),
        }
        log(f"{FORMAT_NAMES[fmt]}: " + json.dumps(out[FORMAT_NAMES[fmt]]))
        p.close()
        del f, w
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--config", default="c4")
    ap.add_argument("--frames", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    cfg = syn.CONFIGS[a.config]
    if a.frames:
        cfg = dataclasses.replace(cfg, frames=a.frames)
    orc.set_threads(a.threads or os.cpu_count() or 1)
    res = study(cfg, a.seed)
    if a.out:
        Path(a.out).write_text(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
