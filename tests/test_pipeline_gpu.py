"""The per-frame pipeline (include/tde_pipeline.h) on the GPU against the CPU
oracle pipeline (FP64 ICP sums and solve) and against itself (graph replay
vs eager launches, asynchronous vs blocking API)."""
import ctypes as C
import dataclasses
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

syn = importlib.import_module("3deye_gb300.synth")


@pytest.fixture(scope="module")
def seq(orc):
    cfg = syn.small_config("c1", frames=14, cols=160, rows=120, voxels=96, fmt=2)
    scene = syn.make_scene(cfg, 1000)
    traj = syn.make_trajectory(cfg, 2000)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    depths = [orc.apply_noise(orc.render_depth(scene, traj[i], intr), 3000, i) for i in range(cfg.frames)]
    return cfg, traj, depths


def run_gpu(cfg, traj, depths, use_graphs=True):
    pl = importlib.import_module("3deye_gb300.pipeline")
    p = pl.Pipeline(cfg, traj[0], use_graphs=use_graphs)
    poses, stats = [], []
    for d in depths:
        pose, st = p.process(d)
        poses.append(pose)
        stats.append(st)
    p.close()
    return np.array(poses), stats


def test_graph_replay_equals_eager_launches(cuda, seq):
    cfg, traj, depths = seq
    a, sa = run_gpu(cfg, traj, depths, True)
    b, sb = run_gpu(cfg, traj, depths, False)
    assert np.array_equal(a, b) and sa == sb


def test_trajectory_matches_fp64_oracle(cuda, orc, seq):
    from oracle.pipeline import OraclePipeline
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    gpu, st = run_gpu(cfg, traj, depths)
    op = OraclePipeline(cfg, traj[0])
    ref = np.array([op.process(d) for d in depths])
    assert not any(st) and not any(op.lost)
    # ATE of the GPU trajectory against the FP64 oracle run: <= 1e-3 m
    assert pl.ate_rmse(gpu, ref) <= 1e-3, pl.ate_rmse(gpu, ref)
    # and both track the ground truth
    assert pl.ate_rmse(gpu, traj) < 0.02, pl.ate_rmse(gpu, traj)
    Rg = gpu[-1, :9].reshape(3, 3)
    np.testing.assert_allclose(Rg @ Rg.T, np.eye(3), atol=1e-9)


def test_async_enqueue_matches_blocking(cuda, seq):
    import torch
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    ref, _ = run_gpu(cfg, traj, depths)
    host = torch.from_numpy(np.stack(depths)).pin_memory()
    poses = torch.zeros((len(depths), 12), dtype=torch.float64).pin_memory()
    status = torch.zeros(len(depths), dtype=torch.int32).pin_memory()
    p = pl.Pipeline(cfg, traj[0], integrate_stats=True)
    p.enable_timing(len(depths))
    fb = cfg.rows * cfg.cols * 2
    for i in range(len(depths)):
        p.enqueue(host.data_ptr() + i * fb, False, poses.data_ptr() + 96 * i, status.data_ptr() + 4 * i)
    p.sync()
    assert np.array_equal(poses.numpy(), ref)
    assert not status.numpy().any()
    ti, tr = p.timings(len(depths))
    assert len(ti) == len(depths) and (ti > 0).all() and (tr > 0).all()
    r, w = p.integrate_stats()
    assert r > 0 and 0 < w <= r
    assert p.launches_per_frame() == 31
    p.close()


@pytest.mark.parametrize("use_graphs", [True, False])
def test_overlapped_preprocessing_matches_blocking(cuda, tde, seq, use_graphs):
    """Frames enqueued back to back: each frame's upload and preprocessing run
    on the second stream into alternating input sets while the previous frame
    is tracked; the poses equal the one-frame-at-a-time run bit for bit, and
    the last frame's maps are those of the last frame."""
    import torch
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    ref, _ = run_gpu(cfg, traj, depths)
    host = torch.from_numpy(np.stack(depths)).pin_memory()
    poses = torch.zeros((len(depths), 12), dtype=torch.float64).pin_memory()
    status = torch.zeros(len(depths), dtype=torch.int32).pin_memory()
    p = pl.Pipeline(cfg, traj[0], use_graphs=use_graphs)
    fb = cfg.rows * cfg.cols * 2
    for i in range(len(depths)):
        p.enqueue(host.data_ptr() + i * fb, False, poses.data_ptr() + 96 * i, status.data_ptr() + 4 * i)
    p.sync()
    assert np.array_equal(poses.numpy(), ref)
    assert not status.numpy().any()
    nbytes = cfg.rows * cfg.cols * 2
    q = pl.Pipeline(cfg, traj[0], use_graphs=use_graphs)
    q.process(depths[-1])
    last = [np.zeros(nbytes, np.uint8) for _ in range(2)]
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    for buf, pipe in zip(last, (p, q)):
        ptr = pipe.frame_maps(0)[0]
        tde.check(tde.lib.tde_memcpy(buf.ctypes.data_as(C.c_void_p), C.c_void_p(ptr), nbytes, 1))
    assert np.array_equal(last[0], last[1]) and last[0].any()
    q.close()
    p.close()


def test_tracking_loss_keeps_previous_pose(cuda, seq):
    """A frame with no valid depth cannot be registered: the pipeline reports
    it and keeps the previous pose (failure made on the host, no GPU fault)."""
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    p = pl.Pipeline(cfg, traj[0])
    for d in depths[:3]:
        pose, st = p.process(d)
        assert st == 0
    blank = np.zeros_like(depths[3])
    pose2, st2 = p.process(blank)
    assert st2 & 1
    assert np.array_equal(pose2, pose)
    pose3, st3 = p.process(depths[4])
    assert st3 == 0
    p.close()


def test_raycast_record_count_matches_oracle(cuda, orc, tde, seq):
    """The raycast's distinct voxel records (the numerator of its roofline):
    the reference march counted on the GPU equals the oracle's count on the
    same volume and pose; skipping empty bricks reads fewer."""
    import ctypes as C
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    p = pl.Pipeline(cfg, traj[0])
    for d in depths[:6]:
        p.process(d)
    full = p.raycast_records(skip_empty=False)
    skipped = p.raycast_records(skip_empty=True)
    vptr, rb = p.volume()
    nbytes = int(tde.lib.tde_tsdf_volume_bytes(cfg.tsdf_format, C.byref(rb)))
    vol = np.zeros(nbytes, np.uint8)
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    tde.check(tde.lib.tde_memcpy(vol.ctypes.data_as(C.c_void_p), vptr, nbytes, 1))
    pose = p.pose()
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    orb = orc.RB.from_buffer_copy(bytes(rb))
    cnt, _, _ = orc.raycast_records(vol, cfg.tsdf_format, orb, intr, pose[:9].astype(np.float32).reshape(3, 3),
                                    pose[9:].astype(np.float32), cfg.trunc_m, np.full(3, cfg.cell, np.float32))
    assert cnt == full > 0
    assert 0 < skipped <= full
    p.close()


def test_model_pyramid_matches_oracle_resize(cuda, orc, tde, seq):
    """The fused model-map pyramid (levels 1 and 2 in one launch) equals the
    oracle's 2x2 resize applied level by level, bit for bit."""
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    p = pl.Pipeline(cfg, traj[0])
    for d in depths[:5]:
        p.process(d)
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]

    def maps(level):
        out = []
        for ptr in p.model_maps(level):
            a = np.zeros(((cfg.rows >> level), (cfg.cols >> level), 3), np.float32)
            tde.check(tde.lib.tde_memcpy(a.ctypes.data_as(C.c_void_p), C.c_void_p(ptr), a.nbytes, 1))
            out.append(a)
        return out

    v0, n0 = maps(0)
    assert np.isfinite(v0).any()
    v1, n1 = maps(1)
    v2, n2 = maps(2)

    def same(a, b):
        na, nb = np.isnan(a[..., 0]), np.isnan(b[..., 0])
        return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))

    rv1, rn1 = orc.resize_map(v0, False), orc.resize_map(n0, True)
    assert same(v1, rv1) and same(n1, rn1)
    assert same(v2, orc.resize_map(rv1, False)) and same(n2, orc.resize_map(rn1, True))
    p.close()


def test_saturated_brick_skip_is_exact(cuda, tde, seq):
    """Bricks whose voxels all hold f = 1 at the maximum weight and lie more
    than the truncation distance in front of the observed surface are not
    swept.  With max_weight 4 many bricks saturate within a few frames; the
    pipeline's volume still equals, bit for bit, a replay of the same frames
    and poses through the C-ABI integration (which sweeps every brick), and
    the pipeline swept fewer bricks than with a weight that never saturates."""
    import torch
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg0, traj, depths = seq
    swept = {}
    for mw in (4, 128):
        cfg = dataclasses.replace(cfg0, max_weight=mw)
        p = pl.Pipeline(cfg, traj[0], integrate_stats=True)
        poses = [p.process(d)[0] for d in depths]
        swept[mw] = p.integrate_stats(bricks=True)[2]
        if mw != 4:
            p.close()
            continue
        vptr, rb = p.volume()
        nbytes = int(tde.lib.tde_tsdf_volume_bytes(cfg.tsdf_format, C.byref(rb)))
        got = np.zeros(nbytes, np.uint8)
        tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        tde.check(tde.lib.tde_memcpy(got.ctypes.data_as(C.c_void_p), C.c_void_p(vptr), nbytes, 1))
        p.close()
        intr = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
        cell = float(np.float32(np.float32(cfg.volume_m) / np.float32(cfg.voxels)))
        vol = tde.new_volume(cfg.tsdf_format, rb)
        for d, pose in zip(depths, poses):
            R = pose[:9].reshape(3, 3)
            scaled = tde.scale_depth(torch.from_numpy(np.ascontiguousarray(d)).to(cuda), intr)
            tde.integrate_tsdf(scaled, vol, cfg.tsdf_format, cfg.trunc_m, np.ascontiguousarray(R.T), pose[9:], intr,
                               [cell] * 3, rb, max_weight=mw)
        torch.cuda.synchronize()
        ref = vol.cpu().numpy()
        assert np.array_equal(got, ref)
    assert swept[4] < swept[128], swept


def test_color_pipeline_matches_c_abi_replay(cuda, tde, seq):
    """RGB-D frames: the pipeline updates its colour volume right after each
    frame's raycast; replaying each frame's model map, pose and RGB image
    through the C-ABI colour integration gives the same volume, byte for byte.
    Plain enqueue is refused once colour is on."""
    import torch
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    p = pl.Pipeline(cfg, traj[0])
    p.enable_color(max_weight=4)
    with pytest.raises(RuntimeError):
        p.process(depths[0])
    rng = np.random.default_rng(3)
    n = cfg.voxels ** 3
    ref = torch.zeros((n, 4), dtype=torch.uint8, device=cuda)
    intr = tde.Intrinsics(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    cell = float(np.float32(np.float32(cfg.volume_m) / np.float32(cfg.voxels)))
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    for d in depths:
        rgb = rng.integers(0, 256, (cfg.rows, cfg.cols, 3), dtype=np.uint8)
        pose, st = p.process_rgbd(d, rgb)
        assert st == 0
        vptr, _ = p.model_maps(0)
        vm = torch.empty((cfg.rows, cfg.cols, 3), dtype=torch.float32, device=cuda)
        tde.check(tde.lib.tde_memcpy(C.c_void_p(vm.data_ptr()), C.c_void_p(vptr), vm.numel() * 4, 2))
        _, rb = p.volume()
        R = pose[:9].reshape(3, 3)
        tde.integrate_colors(ref, torch.from_numpy(rgb).to(cuda), vm, intr, np.ascontiguousarray(R.T), pose[9:],
                             cfg.trunc_m, [cell] * 3, rb, max_weight=4)
    torch.cuda.synchronize()
    got = np.zeros((n, 4), np.uint8)
    tde.check(tde.lib.tde_memcpy(got.ctypes.data_as(C.c_void_p), C.c_void_p(p.color_volume()), got.nbytes, 1))
    assert np.array_equal(got, ref.cpu().numpy())
    assert (got[:, 3] > 0).sum() > 1000 and got[:, 3].max() == 4
    p.close()


def test_color_update_overlapped_equals_serial(cuda, tde, seq):
    """The colour update runs on its own stream beside the next frame's
    tracking, reading per-set snapshots of the model map and pose: frames
    enqueued back to back (device-resident inputs, one sync at the end) give
    the same colour volume, TSDF and pose as frames synchronised one by one."""
    import torch
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    rng = np.random.default_rng(8)
    rgbs = [rng.integers(0, 256, (cfg.rows, cfg.cols, 3), dtype=np.uint8) for _ in depths]
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]

    def volumes(p):
        vptr, rb = p.volume()
        vol = np.zeros(tde.lib.tde_tsdf_volume_bytes(cfg.tsdf_format, C.byref(rb)), np.uint8)
        tde.check(tde.lib.tde_memcpy(vol.ctypes.data_as(C.c_void_p), C.c_void_p(vptr), vol.nbytes, 1))
        col = np.zeros((cfg.voxels ** 3, 4), np.uint8)
        tde.check(tde.lib.tde_memcpy(col.ctypes.data_as(C.c_void_p), C.c_void_p(p.color_volume()), col.nbytes, 1))
        return vol, col, p.pose()

    serial = pl.Pipeline(cfg, traj[0])
    serial.enable_color(max_weight=16)
    for d, c in zip(depths, rgbs):
        assert serial.process_rgbd(d, c)[1] == 0
    ref = volumes(serial)
    serial.close()
    over = pl.Pipeline(cfg, traj[0])
    over.enable_color(max_weight=16)
    dd = torch.from_numpy(np.stack(depths)).to(cuda)
    cc = torch.from_numpy(np.stack(rgbs)).to(cuda)
    for i in range(len(depths)):
        over.enqueue_rgbd(dd[i].data_ptr(), cc[i].data_ptr(), True)
    over.sync()
    got = volumes(over)
    over.close()
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    assert (ref[1][:, 3] > 0).sum() > 1000


def test_pipeline_extract_volume_matches_oracle(cuda, tde, orc, seq, tmp_path):
    """Whole-model export after tracking: the pipeline's points, weights and
    colours equal the oracle's Extract_Tsdf_Volume / Extract_Color_Volume on
    the downloaded volumes, and survive the on-disk cloud format."""
    pl = importlib.import_module("3deye_gb300.pipeline")
    fmt = importlib.import_module("3deye_gb300.formats")
    cfg, traj, depths = seq
    p = pl.Pipeline(cfg, traj[0])
    p.enable_color(max_weight=8)
    rng = np.random.default_rng(4)
    for d in depths:
        pose, st = p.process_rgbd(d, rng.integers(0, 256, (cfg.rows, cfg.cols, 3), dtype=np.uint8))
        assert st == 0
    pts, w, col, n = p.extract_volume()
    assert n > 1000 and len(pts) == n
    vptr, rb = p.volume()
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    vol = np.zeros(tde.lib.tde_tsdf_volume_bytes(cfg.tsdf_format, C.byref(rb)), np.uint8)
    tde.check(tde.lib.tde_memcpy(vol.ctypes.data_as(C.c_void_p), C.c_void_p(vptr), vol.nbytes, 1))
    colv = np.zeros((cfg.voxels ** 3, 4), np.uint8)
    tde.check(tde.lib.tde_memcpy(colv.ctypes.data_as(C.c_void_p), C.c_void_p(p.color_volume()), colv.nbytes, 1))
    orb = orc.RB.from_buffer_copy(bytes(rb))
    cell = np.full(3, np.float32(np.float32(cfg.volume_m) / np.float32(cfg.voxels)), np.float32)
    po, wo, no = orc.extract_tsdf_volume(vol, cfg.tsdf_format, orb, cell, weights=True)
    assert n == no and np.array_equal(pts.view(np.uint32), po.view(np.uint32)) and np.array_equal(w, wo)
    assert np.array_equal(col, orc.extract_color_volume(colv, orb, pts, cell))
    assert (col[:, 3] > 0).mean() > 0.5  # the surface was coloured
    # a short buffer: the prefix, and the total
    p2, _, _, n2 = p.extract_volume(capacity=10)
    assert n2 == n and np.array_equal(p2, pts[:10])
    # the cloud file round trip (6 significant digits)
    path = tmp_path / "model.txt"
    fmt.write_cloud(path, points=p.world_cloud(pts))
    back = fmt.read_cloud(path)
    np.testing.assert_allclose(back, p.world_cloud(pts), rtol=1e-5, atol=1e-6)
    p.close()


def test_pipeline_render_matches_oracle(cuda, tde, orc, seq, tmp_path):
    """Generate_Image of the tracked model: light at the camera by default or
    given; equal to the oracle's shading of the downloaded model maps."""
    import torch
    pl = importlib.import_module("3deye_gb300.pipeline")
    fmt = importlib.import_module("3deye_gb300.formats")
    cfg, traj, depths = seq
    p = pl.Pipeline(cfg, traj[0])
    for d in depths:
        pose, st = p.process(d)
        assert st == 0
    img = torch.empty((cfg.rows, cfg.cols, 3), dtype=torch.uint8, device=cuda)
    p.render(img.data_ptr())
    p.sync()
    vptr, nptr = p.model_maps(0)
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    vm = np.zeros((cfg.rows, cfg.cols, 3), np.float32)
    nm = np.zeros_like(vm)
    tde.check(tde.lib.tde_memcpy(vm.ctypes.data_as(C.c_void_p), C.c_void_p(vptr), vm.nbytes, 1))
    tde.check(tde.lib.tde_memcpy(nm.ctypes.data_as(C.c_void_p), C.c_void_p(nptr), nm.nbytes, 1))
    ref = orc.generate_image(vm, nm, pose[9:].astype(np.float32))
    got = img.cpu().numpy()
    assert np.array_equal(got, ref)
    assert (got[..., 0] > 0).mean() > 0.3
    p.render(img.data_ptr(), light_pos=(0.0, 0.0, 0.0))
    p.sync()
    assert np.array_equal(img.cpu().numpy(), orc.generate_image(vm, nm, (0.0, 0.0, 0.0)))
    fmt.write_ppm(tmp_path / "model.ppm", got)
    assert np.array_equal(fmt.read_ppm(tmp_path / "model.ppm"), got)
    p.close()


@pytest.mark.parametrize("color", [False, True])
def test_checkpoint_resume_bit_identical(cuda, tde, seq, tmp_path, color):
    """A pipeline restored from a checkpoint (here one that started from
    another pose) continues exactly as the checkpointed one: the same poses,
    TSDF and colour volume, bit for bit.  Checkpoints of another
    configuration are refused."""
    pl = importlib.import_module("3deye_gb300.pipeline")
    cfg, traj, depths = seq
    rng = np.random.default_rng(12)
    rgbs = [rng.integers(0, 256, (cfg.rows, cfg.cols, 3), dtype=np.uint8) for _ in depths]
    tde.lib.tde_memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]

    def make(pose):
        p = pl.Pipeline(cfg, pose)
        if color:
            p.enable_color(max_weight=16)
        return p

    def step(p, i):
        return p.process_rgbd(depths[i], rgbs[i]) if color else p.process(depths[i])

    def state(p):
        vptr, rb = p.volume()
        vol = np.zeros(tde.lib.tde_tsdf_volume_bytes(cfg.tsdf_format, C.byref(rb)), np.uint8)
        tde.check(tde.lib.tde_memcpy(vol.ctypes.data_as(C.c_void_p), C.c_void_p(vptr), vol.nbytes, 1))
        col = None
        if color:
            col = np.zeros((cfg.voxels ** 3, 4), np.uint8)
            tde.check(tde.lib.tde_memcpy(col.ctypes.data_as(C.c_void_p), C.c_void_p(p.color_volume()), col.nbytes, 1))
        return vol, col

    k = 6
    a = make(traj[0])
    for i in range(k):
        assert step(a, i)[1] == 0
    ck = a.checkpoint()
    a.save(tmp_path / "ck.bin")
    ref = [step(a, i)[0] for i in range(k, len(depths))]
    ref_vol, ref_col = state(a)
    a.close()
    for via_file in (False, True):
        b = make(traj[3])
        if via_file:
            b.load(tmp_path / "ck.bin")
        else:
            b.restore(ck)
        got = [step(b, i)[0] for i in range(k, len(depths))]
        vol, col = state(b)
        b.close()
        assert all(np.array_equal(x, y) for x, y in zip(got, ref))
        assert np.array_equal(vol, ref_vol)
        if color:
            assert np.array_equal(col, ref_col) and (col[:, 3] > 0).sum() > 1000
    # another storage format, volume edge (same voxel count), truncation or
    # camera, or colour on one side only, is refused and changes nothing
    for change in (dict(tsdf_format=1), dict(volume_m=cfg.volume_m * 1.25), dict(trunc_m=cfg.trunc_m * 1.5),
                   dict(fx=cfg.fx * 1.01)):
        other = pl.Pipeline(dataclasses.replace(cfg, **change), traj[0])
        if color:
            other.enable_color(max_weight=16)
        with pytest.raises(tde.TdeError):
            other.restore(ck)
        assert step(other, 0)[1] == 0  # still usable
        other.close()
    if color:
        other = make(traj[0])
        other.enable_color(max_weight=17)
        with pytest.raises(tde.TdeError):
            other.restore(ck)
        other.close()
    if color:
        plain = pl.Pipeline(cfg, traj[0])
        with pytest.raises(tde.TdeError):
            plain.restore(ck)
        plain.close()
