"""The command-line runner (3deye_gb300/fuse.py): depth-frame reading on the
CPU, and a short fusion on the GPU whose outputs read back in the
reference's text formats."""
import importlib
import json

import numpy as np
import pytest

fuse = importlib.import_module("3deye_gb300.fuse")
fmt = importlib.import_module("3deye_gb300.formats")


def test_pgm_depth_round_trip(tmp_path):
    d = np.random.default_rng(2).integers(0, 65536, (7, 11), dtype=np.uint16)
    fuse.write_depth_pgm(tmp_path / "a.pgm", d)
    np.testing.assert_array_equal(fuse.read_depth(tmp_path / "a.pgm"), d)
    # a comment line in the header, and an .npy frame
    raw = (tmp_path / "a.pgm").read_bytes().replace(b"P5\n", b"P5\n# depth in mm\n", 1)
    (tmp_path / "b.pgm").write_bytes(raw)
    np.testing.assert_array_equal(fuse.read_depth(tmp_path / "b.pgm"), d)
    np.save(tmp_path / "c.npy", d)
    np.testing.assert_array_equal(fuse.read_depth(tmp_path / "c.npy"), d)
    (tmp_path / "d.pgm").write_bytes(b"P5\n3 2\n255\n" + bytes(6))
    with pytest.raises(ValueError):
        fuse.read_depth(tmp_path / "d.pgm")
    # headers cut short, and too few samples, are refused (not read past the end)
    for bad in (b"P5\n3 2", b"P5\n3", b"P5\n# comment without end", b"P5\n3 2\n65535\n" + bytes(5)):
        (tmp_path / "e.pgm").write_bytes(bad)
        with pytest.raises(ValueError):
            fuse.read_depth(tmp_path / "e.pgm")


@pytest.mark.gpu
def test_fuse_synthetic_and_depth_dir(tmp_path, cuda, orc):
    out = tmp_path / "synthetic"
    s = fuse.run(fuse.parse(["--config", "c1", "--frames", "12", "--out", str(out), "--shift-radius", "0"]))
    assert s["frames"] == 12 and s["model_points"] > 1000 and s["ate_m"] < 0.01
    lines = [json.loads(x) for x in (out / "metrics.jsonl").read_text().splitlines()]
    assert len(lines) == 13 and lines[-1]["summary"] and all(x["status"] == 0 for x in lines[:-1])
    traj = fmt.read_trajectory(out / "trajectory.txt")
    pose = np.array([x["pose"] for x in lines[:-1]])
    np.testing.assert_allclose(traj[:, :3, 3], pose[:, 9:], atol=1e-5)
    assert len(fmt.read_cloud(out / "model_points.txt")) == s["model_points"]
    img = fmt.read_ppm(out / "model.ppm")
    assert img.shape == (240, 320, 3) and (img[..., 0] > 0).mean() > 0.3
    # the same scene as 16-bit PGM frames from a directory
    syn = importlib.import_module("3deye_gb300.synth")
    cfg = syn.small_config("c1", frames=6, cols=160, rows=120, voxels=64)
    scene = syn.make_scene(cfg, 1000)
    traj = syn.make_trajectory(cfg, 2000)
    intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
    frames_dir = tmp_path / "frames"
    frames_dir.mkdir()
    for i in range(cfg.frames):
        fuse.write_depth_pgm(frames_dir / f"{i:04d}.pgm", orc.apply_noise(orc.render_depth(scene, traj[i], intr), 3000, i))
    out2 = tmp_path / "dir"
    s2 = fuse.run(fuse.parse(["--depth-dir", str(frames_dir), "--fx", str(cfg.fx), "--fy", str(cfg.fy), "--cx",
                              str(cfg.cx), "--cy", str(cfg.cy), "--voxels", "128", "--volume", "3.0",
                              "--format", "int16", "--out", str(out2), "--shift-radius", "0"]))
    assert s2["frames"] == 6 and s2["model_points"] > 100
    assert len(fmt.read_trajectory(out2 / "trajectory.txt")) == 6


def test_config_refuses_volume_overrides(capsys):
    """A synthetic --config fixes its own volume and camera: explicit volume or
    camera options beside it are an error, not silently ignored."""
    for extra in (["--voxels", "256"], ["--volume", "4"], ["--format", "int16"], ["--trunc", "0.05"],
                  ["--fx", "500"]):
        with pytest.raises(SystemExit):
            fuse.parse(["--config", "c2", "--out", "x", *extra])
        assert "cannot be combined with --config" in capsys.readouterr().err
    a = fuse.parse(["--config", "c2", "--out", "x"])
    assert (a.voxels, a.volume, a.format, a.trunc) == (512, 3.0, "fp16", 0.03)
