"""Command-line fusion of a depth sequence: the per-frame loop the reference
leaves to its (absent) application, with runtime configuration in place of
its compile-time constants.

    python -m 3deye_gb300.fuse --config c2 --frames 600 --out run/
    python -m 3deye_gb300.fuse --depth-dir frames/ --fx 525 --fy 525 --cx 319.5 --cy 239.5 --out run/

Input: a synthetic configuration rendered on the GPU sensor (the seeded
scenes of synth.py; --corridor follows the camera with the cyclic volume), or
a directory of 16-bit depth frames in millimetres (binary PGM, maxval 65535,
or .npy uint16), taken in name order.  Output, in --out:

* trajectory.txt -- the camera poses, write_isometry_to_file's format;
* model_points.txt -- the fused surface (Extract_Tsdf_Volume, world frame),
  matrix<Point_XYZI>::Save_To_File's format;
* model.ppm -- the model shaded from the last camera (Generate_Image);
* metrics.jsonl -- one line per frame (status, world pose) and a summary
  line (frames/s, shifts, points, and the ATE for synthetic input).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import time
from pathlib import Path

import numpy as np

from . import formats, synth
from .pipeline import Pipeline

FORMATS = {"int16": 0, "fp16": 1, "fp32": 2}


def read_depth(path: Path) -> np.ndarray:
    """A 16-bit depth frame: binary PGM (P5, maxval > 255, big-endian samples) or .npy uint16."""
    if path.suffix == ".npy":
        return np.ascontiguousarray(np.load(path), np.uint16)
    raw = path.read_bytes()
    fields, pos = [], 0
    while len(fields) < 4:  # magic, width, height, maxval, skipping comments
        while pos < len(raw) and raw[pos:pos + 1].isspace():
            pos += 1
        if raw[pos:pos + 1] == b"#":
            nl = raw.find(b"\n", pos)
            if nl < 0:
                break
            pos = nl + 1
            continue
        end = pos
        while end < len(raw) and not raw[end:end + 1].isspace():
            end += 1
        if end == pos or end >= len(raw):
            break  # the header ends early
        fields.append(raw[pos:end])
        pos = end
    if len(fields) < 4 or fields[0] != b"P5" or not fields[3].isdigit() or int(fields[3]) <= 255:
        raise ValueError(f"{path}: not a 16-bit binary PGM")
    w, h = int(fields[1]), int(fields[2])
    if len(raw) < pos + 1 + 2 * w * h:
        raise ValueError(f"{path}: {w}x{h} samples do not fit in the file")
    data = np.frombuffer(raw, ">u2", w * h, pos + 1)
    return data.reshape(h, w).astype(np.uint16)


def write_depth_pgm(path, depth: np.ndarray) -> None:
    """Inverse of read_depth for PGM."""
    d = np.ascontiguousarray(depth, np.uint16)
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n65535\n" % (d.shape[1], d.shape[0]))
        f.write(d.astype(">u2").tobytes())


def parse(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    src = ap.add_mutually_exclusive_group(required=True)
    src.add_argument("--config", choices=sorted(synth.CONFIGS), help="synthetic configuration")
    src.add_argument("--depth-dir", type=Path, help="directory of 16-bit depth frames (mm)")
    ap.add_argument("--out", type=Path, required=True)
    ap.add_argument("--frames", type=int, default=None, help="frames to fuse (default: all)")
    ap.add_argument("--seed", type=int, default=0, help="synthetic sequence seed index")
    ap.add_argument("--corridor", action="store_true",
                    help="synthetic corridor walk (the cyclic-volume workload; implied by --config c3)")
    ap.add_argument("--fx", type=float), ap.add_argument("--fy", type=float)
    ap.add_argument("--cx", type=float), ap.add_argument("--cy", type=float)
    # volume settings of --depth-dir input; a --config fixes its own
    ap.add_argument("--voxels", type=int, default=None, help="voxels per axis (default 512)")
    ap.add_argument("--volume", type=float, default=None, help="volume edge in m (default 3.0)")
    ap.add_argument("--format", choices=sorted(FORMATS), default=None, help="TSDF storage (default fp16)")
    ap.add_argument("--trunc", type=float, default=None, help="truncation distance in m (default 0.03)")
    ap.add_argument("--shift-radius", type=float, default=0.4,
                    help="re-centre the volume when the point half a volume ahead leaves this radius (m); "
                         "0 disables shifts")
    args = ap.parse_args(argv)
    fixed = [f"--{k}" for k in ("voxels", "volume", "format", "trunc", "fx", "fy", "cx", "cy")
             if getattr(args, k) is not None]
    if args.config and fixed:
        ap.error(f"{', '.join(fixed)} cannot be combined with --config (the configuration fixes them)")
    args.voxels = 512 if args.voxels is None else args.voxels
    args.volume = 3.0 if args.volume is None else args.volume
    args.format = "fp16" if args.format is None else args.format
    args.trunc = 0.03 if args.trunc is None else args.trunc
    return args


def run(args) -> dict:
    import torch
    tde = __import__("3deye_gb300", fromlist=["lib"])
    dev = torch.device("cuda", 0)
    if args.config:
        cfg = synth.CONFIGS[args.config]
        n = cfg.frames if args.frames is None else args.frames
        s_scene, s_traj, s_noise = synth.seeds(args.seed)
        if args.corridor or args.config == "c3":  # c3 is the corridor workload
            scene, gt = synth.make_corridor_scene(cfg, s_scene), synth.make_corridor_trajectory(cfg, s_traj, n)
        else:
            scene, gt = synth.make_scene(cfg, s_scene), synth.make_trajectory(cfg, s_traj, n)
        frames = synth_frames(tde, cfg, scene, gt, s_noise, dev)
        start = gt[0]
    else:
        files = sorted(p for p in args.depth_dir.iterdir() if p.suffix in (".pgm", ".npy"))
        if args.frames is not None:
            files = files[:args.frames]
        if not files:
            raise SystemExit(f"no .pgm or .npy frames in {args.depth_dir}")
        if None in (args.fx, args.fy, args.cx, args.cy):
            raise SystemExit("--depth-dir needs --fx --fy --cx --cy")
        first = read_depth(files[0])
        base = synth.CONFIGS["c2"]
        cfg = dataclasses.replace(base, name="depth-dir", frames=len(files), cols=first.shape[1], rows=first.shape[0],
                                  fx=args.fx, fy=args.fy, cx=args.cx, cy=args.cy, voxels=args.voxels,
                                  volume_m=args.volume, tsdf_format=FORMATS[args.format], trunc_m=args.trunc)
        n = len(files)
        frames = torch.from_numpy(np.stack([read_depth(f) for f in files])).to(dev)
        gt = None
        # the camera at the centre of the volume's rear face, looking along +z
        start = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, cfg.volume_m / 2, cfg.volume_m / 2, 0.0])
    args.out.mkdir(parents=True, exist_ok=True)
    p = Pipeline(cfg, start)
    cell = cfg.volume_m / cfg.voxels
    offset = np.zeros(3)
    poses, shifts, points = [], 0, 0
    t0 = time.perf_counter()
    with open(args.out / "metrics.jsonl", "w") as log:
        for i in range(n):
            pose, st = p.process(frames[i])
            world = pose.copy()
            world[9:] += offset
            poses.append(world)
            log.write(json.dumps({"frame": i, "status": int(st), "pose": [round(float(v), 7) for v in world]}) + "\n")
            if args.shift_radius > 0:
                delta = p.shift_needed(args.shift_radius)
                if delta.any():
                    _, _, k = p.shift(delta)
                    offset = offset + delta * cell
                    shifts += 1
                    points += k
        elapsed = time.perf_counter() - t0
        pts, _, _, m = p.extract_volume()
        world_pts = p.world_cloud(pts) if m else pts
        formats.write_trajectory(args.out / "trajectory.txt", np.array(poses))
        formats.write_cloud(args.out / "model_points.txt", points=world_pts)
        img = torch.empty((cfg.rows, cfg.cols, 3), dtype=torch.uint8, device=dev)
        p.render(img.data_ptr())
        p.sync()
        formats.write_ppm(args.out / "model.ppm", img.cpu().numpy())
        summary = {"summary": True, "frames": n, "frames_per_s": round(n / elapsed, 2), "shifts": shifts,
                   "slab_points": int(points), "model_points": int(m),
                   "volume_offset_m": [float(v) for v in offset]}
        if gt is not None:
            from .pipeline import ate_rmse
            summary["ate_m"] = round(ate_rmse(np.array(poses), gt), 6)
        log.write(json.dumps(summary) + "\n")
    p.close()
    return summary


def synth_frames(tde, cfg, scene, traj, seed, dev):
    """Depth frames rendered on the GPU sensor (device uint16 [n, H, W])."""
    import ctypes as C
    import torch
    tde.lib.tde_synth_depth.restype = C.c_int
    tde.lib.tde_synth_depth.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(tde.Intrinsics), C.c_uint32,
                                        C.c_uint32, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    d_scene = torch.from_numpy(scene).to(dev)
    intr = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    frames = torch.empty((len(traj), cfg.rows, cfg.cols), dtype=torch.uint16, device=dev)
    for i in range(len(traj)):
        pose = np.ascontiguousarray(traj[i])
        tde.check(tde.lib.tde_synth_depth(d_scene.data_ptr(), scene.shape[0], pose.ctypes.data_as(C.c_void_p),
                                          C.byref(intr), seed, i, cfg.max_depth_mm / 1000.0, 0.02,
                                          frames[i].data_ptr(), None, None))
    torch.cuda.synchronize()
    return frames


def main(argv=None):
    print(json.dumps(run(parse(argv))))


if __name__ == "__main__":
    main()
