"""The learned refiner end to end: training pairs generated by the pipeline
itself, training with the library's own kernels, and evaluation against the
plain bilateral pipeline on held-out sequences.

Pairs: every frame of a sequence run through the pipeline gives (raw noisy
depth, model depth) -- the raycast of the fused volume (tde_pipeline_model_depth).
Fusion and raycast run at the ground-truth poses of the synthetic sequence
(tracking off), so the targets carry no tracking error.  Evaluation: the same
held-out sequences through the plain and the learned pipeline; ATE against the
ground-truth trajectory, and surface error of the final volume raycast at
ground-truth poses against the noise-free rendered depth.

    python -m 3deye_gb300.learned --scenes 40 --frames 500 --steps 6000 \\
        --eval-seqs 5 --eval-frames 600 --out weights.f32 --report report.json
"""
from __future__ import annotations

import argparse
import ctypes as C
import dataclasses
import importlib
import json
import time

import numpy as np

tde = importlib.import_module("3deye_gb300")
syn = importlib.import_module("3deye_gb300.synth")
pl = importlib.import_module("3deye_gb300.pipeline")
rf = importlib.import_module("3deye_gb300.refiner")

TRAIN_SEED0 = 100   # training sequences k = 100, 101, ...
EVAL_SEED0 = 200    # held-out sequences k = 200, 201, ...


def _synth_fn():
    f = tde.lib.tde_synth_depth
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(tde.Intrinsics), C.c_uint32, C.c_uint32, C.c_float,
                  C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def render_sequence(cfg, k, nframes, noise_free=False):
    """Seeded scene k: (device uint16 frames [n,H,W], ground-truth poses, device scene, noise-free depth or None)."""
    import torch
    s_scene, s_traj, s_noise = syn.seeds(k)
    scene = syn.make_scene(cfg, s_scene)
    traj = syn.make_trajectory(cfg, s_traj, nframes)
    d_scene = torch.from_numpy(scene).cuda()
    intr = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    frames = torch.empty((nframes, cfg.rows, cfg.cols), dtype=torch.uint16, device="cuda")
    clean = torch.empty((nframes, cfg.rows, cfg.cols), dtype=torch.float32, device="cuda") if noise_free else None
    fn = _synth_fn()
    stream = torch.cuda.current_stream().cuda_stream
    for i in range(nframes):
        pose = np.ascontiguousarray(traj[i])
        tde.check(fn(d_scene.data_ptr(), scene.shape[0], pose.ctypes.data_as(C.c_void_p), C.byref(intr), s_noise, i,
                     cfg.max_depth_mm / 1000.0, 0.02, frames[i].data_ptr(),
                     clean[i].data_ptr() if clean is not None else None, stream))
    torch.cuda.synchronize()
    return frames, traj, d_scene, clean


SKIP_FRAMES = 50        # the model of a sequence's first frames is still thin: no pairs from them
OUTLIER_MM = 30         # target pixels this far from the raw depth become the raw depth (edges, disocclusions)


def generate_pairs(cfg, scenes, frames_per_scene, seed0=TRAIN_SEED0, log=print):
    """Training pairs (raw, model depth) in mm as device int16 tensors [N,H,W].
    Each scene runs SKIP_FRAMES + frames_per_scene frames; target pixels with
    no model surface or more than OUTLIER_MM from the raw depth take the raw
    depth."""
    import torch
    n = scenes * frames_per_scene
    # int16 storage (values <= 32767): the same bits, and every torch op on it
    raw = torch.empty((n, cfg.rows, cfg.cols), dtype=torch.int16, device="cuda")
    tgt = torch.empty_like(raw)
    t0 = time.time()
    total = SKIP_FRAMES + frames_per_scene
    scratch = torch.empty((cfg.rows, cfg.cols), dtype=torch.int16, device="cuda")
    # fusion and raycast at the ground-truth poses (tracking off: 0 ICP
    # iterations), so that tracking error does not leak into the targets
    fuse_cfg = dataclasses.replace(cfg, icp_iters=(0, 0, 0))
    for s in range(scenes):
        frames, traj, _, _ = render_sequence(cfg, seed0 + s, total)
        p = pl.Pipeline(fuse_cfg, traj[0], use_graphs=True)
        base = frames.data_ptr()
        fb = cfg.rows * cfg.cols * 2
        for i in range(total):
            p.set_pose(traj[i])
            p.enqueue(base + i * fb, True)
            j = s * frames_per_scene + i - SKIP_FRAMES
            p.model_depth(tgt[j].data_ptr() if j >= s * frames_per_scene else scratch.data_ptr())
        p.sync()
        raw[s * frames_per_scene:(s + 1) * frames_per_scene].copy_(frames[SKIP_FRAMES:].view(torch.int16))
        p.close()
        del frames
        if log and (s + 1) % 10 == 0:
            log(f"pairs: {s + 1}/{scenes} scenes, {time.time() - t0:.1f} s")
    # where the model has no surface, or one far from the raw depth (depth
    # edges, disocclusions), the target is the raw depth itself: the refiner
    # learns to leave such pixels alone
    r32, t32 = raw.to(torch.int32), tgt.to(torch.int32)
    keep = (r32 > 0) & ((t32 == 0) | ((t32 - r32).abs() > OUTLIER_MM))
    tgt.copy_(torch.where(keep, raw, tgt))
    del r32, t32, keep
    torch.cuda.synchronize()
    return raw, tgt


def lr_at(step, steps, lr, warmup=100, floor=0.01):
    """Linear warm-up, then cosine decay to floor * lr."""
    if step < warmup:
        return lr * (step + 1) / warmup
    u = (step - warmup) / max(1, steps - warmup)
    return lr * (floor + (1.0 - floor) * 0.5 * (1.0 + np.cos(np.pi * u)))


def train(refiner, raw, tgt, steps, batch, lr, seed=0, log=print, log_every=250):
    """AdamW on random batches of the pairs; returns the per-step mean L1 (m) over valid pixels."""
    import torch
    n = raw.shape[0]
    rng = np.random.default_rng(seed)
    braw = torch.empty((batch,) + tuple(raw.shape[1:]), dtype=raw.dtype, device=raw.device)
    btgt = torch.empty_like(braw)
    losses = []
    t0 = time.time()
    for it in range(steps):
        idx = torch.from_numpy(rng.integers(0, n, batch)).cuda()
        torch.index_select(raw, 0, idx, out=braw)
        torch.index_select(tgt, 0, idx, out=btgt)
        refiner.train_step_ptr(braw.data_ptr(), btgt.data_ptr(), batch, lr_at(it, steps, lr),
                               torch.cuda.current_stream().cuda_stream)
        if (it + 1) % 50 == 0 or it == 0:
            loss, cnt = refiner.last_loss()
            losses.append((it + 1, loss * batch * raw.shape[1] * raw.shape[2] / max(cnt, 1.0)))
            if log and ((it + 1) % log_every == 0 or it == 0):
                log(f"step {it + 1}: mean L1 {losses[-1][1] * 1000:.3f} mm ({time.time() - t0:.1f} s)")
    refiner.check_status()
    return losses


def run_sequence(cfg, frames, traj, refiner=None):
    """(estimated poses [n,12], frames tracking lost, ms per frame, pipeline)."""
    import torch
    n = frames.shape[0]
    p = pl.Pipeline(cfg, traj[0], use_graphs=True)
    if refiner is not None:
        p.set_refiner(refiner)
    poses = torch.zeros((n, 12), dtype=torch.float64, pin_memory=True)
    status = torch.zeros(n, dtype=torch.int32, pin_memory=True)
    base, fb = frames.data_ptr(), cfg.rows * cfg.cols * 2
    warm = min(10, n)
    for i in range(warm):
        p.enqueue(base + i * fb, True, poses.data_ptr() + 96 * i, status.data_ptr() + 4 * i)
    p.sync()
    stream = torch.cuda.ExternalStream(p.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(warm, n):
        p.enqueue(base + i * fb, True, poses.data_ptr() + 96 * i, status.data_ptr() + 4 * i)
    e1.record(stream)
    p.sync()
    ms = e0.elapsed_time(e1) / max(n - warm, 1)
    return poses.numpy().copy(), int((status.numpy() != 0).sum()), ms, p


def surface_error(p, cfg, traj, clean, frame_ids):
    """Mean |model depth - noise-free depth| (m) of the final volume raycast at
    ground-truth poses, over pixels where both have a surface within 4 cm, and
    the fraction of noise-free pixels the model covers."""
    import torch
    vol, rb = p.volume()
    intr = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    c = float(cfg.volume_m / cfg.voxels)
    cell = tde.vec3([c, c, c])
    vmap = torch.empty((cfg.rows, cfg.cols, 3), dtype=torch.float32, device="cuda")
    nmap = torch.empty_like(vmap)
    errs, cover = [], []
    for k in frame_ids:
        R = traj[k][:9].reshape(3, 3)
        t = traj[k][9:12]
        tde.check(tde.lib.tde_raycast(C.c_void_p(vol), cfg.tsdf_format, C.c_void_p(vmap.data_ptr()),
                                      C.c_void_p(nmap.data_ptr()), C.byref(tde.vec3(t)), C.byref(tde.mat3(R)),
                                      C.c_float(cfg.trunc_m), C.byref(intr), C.byref(rb), C.byref(cell), None))
        torch.cuda.synchronize()
        Rt = torch.from_numpy(R.astype(np.float32)).cuda()
        z = (vmap - torch.from_numpy(t.astype(np.float32)).cuda()) @ Rt[:, 2]
        g = clean[k]
        hit = torch.isfinite(z) & (z > 0)
        have = g > 0
        both = hit & have & ((z - g).abs() < 0.04)
        errs.append(float((z - g).abs()[both].mean().item()) if bool(both.any()) else float("nan"))
        cover.append(float(both.sum().item()) / max(float(have.sum().item()), 1.0))
    return float(np.nanmean(errs)), float(np.mean(cover))


def evaluate(cfg, refiner, seqs, nframes, seed0=EVAL_SEED0, log=print):
    rows = []
    for s in range(seqs):
        k = seed0 + s
        frames, traj, _, clean = render_sequence(cfg, k, nframes, noise_free=True)
        ids = list(range(nframes - 1, 0, -max(1, nframes // 6)))[:6]
        row = {"seed_k": k}
        for name, r in (("plain", None), ("learned", refiner)):
            est, lost, ms, p = run_sequence(cfg, frames, traj, r)
            surf, cover = surface_error(p, cfg, traj, clean, ids)
            p.close()
            row[name] = {"ate_m": pl.ate_rmse(est, traj), "lost": lost, "ms_per_frame": ms, "fps": 1e3 / ms,
                         "surface_err_m": surf, "surface_cover": cover}
        rows.append(row)
        if log:
            log(json.dumps(row))
        del frames, clean
    mean = {name: {key: float(np.mean([r[name][key] for r in rows])) for key in rows[0][name]}
            for name in ("plain", "learned")}
    return {"sequences": rows, "mean": mean}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--config", default="c2")
    ap.add_argument("--scenes", type=int, default=40)
    ap.add_argument("--frames", type=int, default=500)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval-seqs", type=int, default=5)
    ap.add_argument("--eval-frames", type=int, default=600)
    ap.add_argument("--init", default=None, help="start from these weights (raw float32)")
    ap.add_argument("--out", default=None, help="write trained weights (raw float32)")
    ap.add_argument("--report", default=None, help="write the evaluation as JSON")
    a = ap.parse_args(argv)
    cfg = syn.CONFIGS[a.config]
    R = rf.Refiner(a.batch, cfg.rows, cfg.cols, seed=a.seed)
    R.set_adamw(0.9, 0.999, 1e-8, 0.01)
    report = {"config": a.config, "scenes": a.scenes, "frames_per_scene": a.frames, "steps": a.steps,
              "batch": a.batch, "lr": a.lr}
    if a.init:
        R.set_params(np.fromfile(a.init, dtype=np.float32))
    if a.steps > 0:
        t0 = time.time()
        raw, tgt = generate_pairs(cfg, a.scenes, a.frames)
        report["pairs_s"] = time.time() - t0
        t0 = time.time()
        losses = train(R, raw, tgt, a.steps, a.batch, a.lr, a.seed)
        report["train_s"] = time.time() - t0
        report["loss_curve_m"] = losses
        del raw, tgt
        if a.out:
            R.get_params().tofile(a.out)
    if a.eval_seqs > 0:
        E = rf.Refiner(1, cfg.rows, cfg.cols, seed=0)
        E.set_params(R.get_params())
        report["eval"] = evaluate(cfg, E, a.eval_seqs, a.eval_frames)
        print(json.dumps(report["eval"]["mean"]))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(report, f, indent=1)


if __name__ == "__main__":
    main()
