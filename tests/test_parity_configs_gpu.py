"""Parity at the benchmark's own configurations, not reduced copies.

* Config 1 (100 frames of 320x240, 128^3 FP32 over 2 m, ICP 10/5/4): the
  GPU trajectory against the CPU oracle pipeline (the same FP32 stages with
  FP64 ICP sums) and against the full-FP64 oracle pipeline (FP64 TSDF,
  integration, raycast, ICP terms and solve), ATE <= 1e-3 m for both.
* Config 2 (640x480, 512^3 FP16+u16 over 3 m): five frames fused by the
  pipeline (depth-tile pyramid, brick culling and the saturated-brick skip at
  full size) give the volume a full sweep of the oracle's integration gives
  at the pipeline's own poses, bit for bit; and 60 tracked frames stay within
  1e-3 m ATE of both oracle pipelines.
* The GPU sensor renders the CPU sensor's frames bit for bit, so the
  benchmark's CPU arm times the GPU arm's own sequence.

Frames come from the seeded CPU sensor with the benchmark's sequence seeds
(synth.seeds(0)).
"""
import ctypes as C
import os
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

syn = importlib.import_module("3deye_gb300.synth")
ATE_BOUND_M = 1e-3


def sequence(orc, name, n):
    cfg = syn.CONFIGS[name]
    s_scene, s_traj, s_noise = syn.seeds(0)
    scene = syn.make_scene(cfg, s_scene)
    traj = syn.make_trajectory(cfg, s_traj, n)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    depths = [orc.apply_noise(orc.render_depth(scene, traj[i], intr), s_noise, i) for i in range(n)]
    return cfg, scene, traj, depths


def gpu_poses(cfg, traj, depths):
    pl = importlib.import_module("3deye_gb300.pipeline")
    p = pl.Pipeline(cfg, traj[0], use_graphs=True)
    poses, st = [], []
    for d in depths:
        pose, s = p.process(d)
        poses.append(pose)
        st.append(s)
    p.close()
    return np.array(poses), st


def oracle_poses(cfg, traj, depths, f64):
    from oracle.pipeline import OraclePipeline, OraclePipelineF64
    op = (OraclePipelineF64 if f64 else OraclePipeline)(cfg, traj[0])
    poses = np.array([op.process(d) for d in depths])
    return poses, op.lost


@pytest.mark.parametrize("name,frames", [("c1", 100), ("c2", 60)])
def test_trajectory_at_config_size_matches_oracles(cuda, orc, name, frames):
    pl = importlib.import_module("3deye_gb300.pipeline")
    orc.set_threads(os.cpu_count() or 1)
    cfg, _, traj, depths = sequence(orc, name, frames)
    gpu, st = gpu_poses(cfg, traj, depths)
    assert not any(st), "GPU tracking lost"
    for f64 in (False, True):
        ref, lost = oracle_poses(cfg, traj, depths, f64)
        assert not any(lost), "oracle tracking lost"
        ate = pl.ate_rmse(gpu, ref)
        assert ate <= ATE_BOUND_M, (name, "FP64" if f64 else "FP32-storage", ate)
    # and the trajectory follows the ground truth
    assert pl.ate_rmse(gpu, traj) < 0.01, pl.ate_rmse(gpu, traj)


def test_config2_volume_equals_full_sweep_oracle(cuda, orc, tde):
    """Five frames at 640x480 into 512^3 FP16+u16 through the pipeline; the
    oracle integrates the same raw frames at the pipeline's poses with a full
    sweep of every voxel, and the volumes agree bit for bit."""
    pl = importlib.import_module("3deye_gb300.pipeline")
    orc.set_threads(os.cpu_count() or 1)
    cfg, _, traj, depths = sequence(orc, "c2", 5)
    p = pl.Pipeline(cfg, traj[0], use_graphs=True)
    poses = []
    for d in depths:
        pose, s = p.process(d)
        assert s == 0
        poses.append(pose)
    vptr, rb = p.volume()
    vol = np.zeros(tde.lib.tde_tsdf_volume_bytes(cfg.tsdf_format, C.byref(rb)), np.uint8)
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    tde.check(tde.lib.tde_memcpy(vol.ctypes.data_as(C.c_void_p), C.c_void_p(vptr), vol.nbytes, 1))
    p.close()

    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    orb = orc.make_rb((cfg.voxels,) * 3, (cfg.volume_m,) * 3)
    ref = np.zeros(orc.volume_bytes(cfg.tsdf_format, orb), np.uint8)
    cell = np.full(3, cfg.cell, np.float32)
    for d, pose in zip(depths, poses):
        Rf = pose[:9].reshape(3, 3).astype(np.float32)
        tf = pose[9:].astype(np.float32)
        sd = orc.scale_depth(d, intr)
        orc.integrate(sd, ref, cfg.tsdf_format, cfg.trunc_m, np.ascontiguousarray(Rf.T), tf, intr, cell, orb,
                      cfg.max_weight)
    w = ref.view(np.uint16)[1::2]
    assert (w > 0).sum() > 1_000_000 and (w == 5).sum() > 100_000  # a real surface, seen by every frame
    diff = np.flatnonzero(vol.view(np.uint32) != ref.view(np.uint32))
    assert diff.size == 0, f"{diff.size} voxel records differ, first at {diff[:5]}"


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_gpu_sensor_renders_the_cpu_sensor_frames(cuda, orc, tde, name):
    import torch
    cfg = syn.CONFIGS[name]
    s_scene, s_traj, s_noise = syn.seeds(0)
    scene = syn.make_scene(cfg, s_scene)
    traj = syn.make_trajectory(cfg, s_traj, 4)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    ti = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    L = tde.lib
    L.tde_synth_depth.restype = C.c_int
    L.tde_synth_depth.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(tde.Intrinsics), C.c_uint32, C.c_uint32,
                                  C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    d_scene = torch.from_numpy(scene).to(cuda)
    out = torch.empty((cfg.rows, cfg.cols), dtype=torch.uint16, device=cuda)
    for i in range(4):
        pose = np.ascontiguousarray(traj[i])
        tde.check(L.tde_synth_depth(d_scene.data_ptr(), scene.shape[0], pose.ctypes.data_as(C.c_void_p), C.byref(ti),
                                    s_noise, i, cfg.max_depth_mm / 1000.0, 0.02, out.data_ptr(), None,
                                    tde.stream_ptr()))
        torch.cuda.synchronize()
        ref = orc.apply_noise(orc.render_depth(scene, traj[i], intr), s_noise, i)
        got = out.cpu().numpy()
        assert np.array_equal(got, ref), f"frame {i}: {(got != ref).sum()} pixels differ"
        assert (ref > 0).mean() > 0.5
