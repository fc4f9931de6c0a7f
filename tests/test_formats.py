"""On-disk trajectory and cloud formats (string_utils.cpp:26-74,
impl/matrix.hpp:413-540, base_points.cpp:279-282,571-574): known answers
worked out from the reference's stream operators, byte equality between the
Python writers and the header-only C++ writers of include/3deye/, and round
trips through both readers.  CPU only."""
import importlib
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

fmt = importlib.import_module("3deye_gb300.formats")


def test_trajectory_known_answer(tmp_path):
    # identity rotation, t = (0.5, -1, 2.25); second pose a quarter turn about z
    poses = np.zeros((2, 12))
    poses[0, :9] = np.eye(3).ravel()
    poses[0, 9:] = (0.5, -1.0, 2.25)
    poses[1, :9] = [0, -1, 0, 1, 0, 0, 0, 0, 1]
    poses[1, 9:] = (1e-7, 123456.7, -0.0)
    expect = ("0\n1x0x0 \n0x1x0 \n0x0x1  \n0.5x-1x2.25 \n"
              "1\n0x-1x0 \n1x0x0 \n0x0x1  \n1e-07x123457x-0 \n")
    assert fmt.format_trajectory(poses) == expect
    p = tmp_path / "t.txt"
    fmt.write_trajectory(p, poses)
    assert p.read_text() == expect
    back = fmt.read_trajectory(p)
    assert back.shape == (2, 4, 4)
    np.testing.assert_array_equal(back[0, :3, :3], np.eye(3))
    np.testing.assert_allclose(back[1, :3, 3], (1e-7, 123457.0, 0.0))


def test_cloud_known_answer():
    pts = np.array([[1, 2, 3, 1], [0.25, -7.5, 1e-3, 1]], np.float32)
    assert fmt.format_cloud(points=pts) == "2 1 1 P5PointI4XYZIE\n1x2x3x1 0.25x-7.5x0.001x1 \n"
    cols = np.array([[255, 0, 7, 128]], np.uint8)
    assert fmt.format_cloud(colors=cols) == "1 1 1 P5PointI5ColorE\n255.0.7.128  \n"
    assert fmt.format_cloud(points=np.zeros((0, 4), np.float32)) == "0 1 1 P5PointI4XYZIE\n\n"


def test_pose_layouts_agree():
    rng = np.random.default_rng(5)
    m = np.tile(np.eye(4), (3, 1, 1))
    m[:, :3, :] = rng.normal(size=(3, 3, 4))
    p12 = np.concatenate([m[:, :3, :3].reshape(3, 9), m[:, :3, 3]], axis=1)
    assert fmt.format_trajectory(m) == fmt.format_trajectory(m[:, :3]) == fmt.format_trajectory(p12)
    with pytest.raises(ValueError):
        fmt.format_trajectory(np.zeros((2, 5)))


@pytest.mark.parametrize("n_pts", [0, 1, 257])
def test_cxx_writers_match_python_and_round_trip(tmp_path, n_pts):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "formats_roundtrip"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include" / "3deye"), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cxx" / "formats_roundtrip.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(11 + n_pts)
    n_poses = 4
    R = rng.normal(size=(n_poses, 3, 3)).astype(np.float32)
    t = (rng.normal(size=(n_poses, 3)) * 10.0 ** rng.integers(-6, 6, size=(n_poses, 3))).astype(np.float32)
    t[0, 0] = -0.0
    pts = (rng.normal(size=(n_pts, 4)) * 100).astype(np.float32)
    pts[:, 3] = 1.0
    if n_pts > 2:
        pts[1, :3] = np.round(pts[1, :3])  # integral values print without a point
        pts[2, 0] = 3.0e-12
    cols = rng.integers(0, 256, size=(n_pts, 4), dtype=np.uint8)
    with open(tmp_path / "input.bin", "wb") as f:
        np.array([n_poses, n_pts], np.int32).tofile(f)
        R.tofile(f)
        t.tofile(f)
        pts.tofile(f)
        cols.tofile(f)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    m = np.tile(np.eye(4), (n_poses, 1, 1))
    m[:, :3, :3], m[:, :3, 3] = R, t
    assert (tmp_path / "trajectory.txt").read_text() == fmt.format_trajectory(m)
    assert (tmp_path / "cloud.txt").read_text() == fmt.format_cloud(points=pts)
    assert (tmp_path / "colors.txt").read_text() == fmt.format_cloud(colors=cols)
    # readers: C++ Fill_From_File and Python read_cloud agree (6 digits)
    raw = (tmp_path / "readback.bin").read_bytes()
    st = np.frombuffer(raw, np.int32, 4)
    assert st[0] == 0 and st[1] == 0 and st[2] == n_pts and st[3] == n_pts
    back_pts = np.frombuffer(raw, np.float32, 4 * n_pts, 16).reshape(-1, 4)
    back_cols = np.frombuffer(raw, np.uint8, 4 * n_pts, 16 + 16 * n_pts).reshape(-1, 4)
    py_pts = fmt.read_cloud(tmp_path / "cloud.txt")
    np.testing.assert_array_equal(back_pts, py_pts.reshape(-1, 4))
    np.testing.assert_allclose(py_pts, pts, rtol=5e-6, atol=0)
    np.testing.assert_array_equal(back_cols, cols)
    if n_pts:
        np.testing.assert_array_equal(fmt.read_cloud(tmp_path / "colors.txt"), cols)
    np.testing.assert_allclose(fmt.read_trajectory(tmp_path / "trajectory.txt"), m, rtol=5e-6, atol=0)


def test_ppm_known_answer_and_round_trip(tmp_path):
    img = np.zeros((2, 3, 3), np.uint8)
    img[0, 1] = (50, 50, 50)
    img[1, 2] = (255, 255, 255)
    p = tmp_path / "a.ppm"
    fmt.write_ppm(p, img)
    raw = p.read_bytes()
    assert raw[:11] == b"P6\n3 2\n255\n" and len(raw) == 11 + 18
    assert raw[11 + 3:11 + 6] == b"\x32\x32\x32"
    np.testing.assert_array_equal(fmt.read_ppm(p), img)
    with pytest.raises(ValueError):
        fmt.write_ppm(p, np.zeros((2, 3), np.uint8))
    for bad in (b"P6\n3 2\n", b"P6\n3 2\n255\n" + bytes(5), b"P5\n3 2\n255\n" + bytes(18)):
        (tmp_path / "bad.ppm").write_bytes(bad)
        with pytest.raises(ValueError):
            fmt.read_ppm(tmp_path / "bad.ppm")


def test_golden_slab_clouds_in_reference_text_format():
    """tests/golden/slices_c*_{points,colors}.txt hold the reference kernels'
    slab clouds as matrix<T>::Save_To_File writes them; read back they equal
    the binary fixtures exactly (voxel-unit points print without rounding)."""
    golden = ROOT / "tests" / "golden"
    g = np.load(golden / "slices.npz")
    for ci in range(int(g["ncases"])):
        pts = fmt.read_cloud(golden / f"slices_c{ci}_points.txt")
        np.testing.assert_array_equal(pts.reshape(-1, 4), g[f"c{ci}_points"])
        cols = fmt.read_cloud(golden / f"slices_c{ci}_colors.txt")
        if len(cols):
            np.testing.assert_array_equal(cols, g[f"c{ci}_colors"])
        text = (golden / f"slices_c{ci}_points.txt").read_text()
        assert text == fmt.format_cloud(points=g[f"c{ci}_points"])


def test_golden_text_clouds_read_by_cxx_fill_from_file(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "formats_roundtrip"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include" / "3deye"), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cxx" / "formats_roundtrip.cpp"), "-o", str(exe)], check=True)
    with open(tmp_path / "input.bin", "wb") as f:
        np.array([0, 0], np.int32).tofile(f)
    golden = ROOT / "tests" / "golden"
    g = np.load(golden / "slices.npz")
    ci = 1
    r = subprocess.run([str(exe), str(tmp_path), str(golden / f"slices_c{ci}_points.txt"),
                        str(golden / f"slices_c{ci}_colors.txt")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = (tmp_path / "golden.bin").read_bytes()
    st = np.frombuffer(raw, np.int32, 4)
    n = len(g[f"c{ci}_points"])
    assert st[0] == 0 and st[1] == 0 and st[2] == n and st[3] == n
    np.testing.assert_array_equal(np.frombuffer(raw, np.float32, 4 * n, 16).reshape(-1, 4), g[f"c{ci}_points"])
    np.testing.assert_array_equal(np.frombuffer(raw, np.uint8, 4 * n, 16 + 16 * n).reshape(-1, 4), g[f"c{ci}_colors"])


def test_round_buffer_text_record(tmp_path):
    """C++ operator<< writes round_buffer.cpp's record byte for byte as the
    Python formatter does, and operator>> reads every field back."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "formats_roundtrip"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include" / "3deye"), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cxx" / "formats_roundtrip.cpp"), "-o", str(exe)], check=True)
    with open(tmp_path / "input.bin", "wb") as f:
        np.array([0, 0], np.int32).tofile(f)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    f32 = np.float32
    expect = fmt.format_round_buffer((3, 500, 7), (f32(3), f32(-12), f32(7)),
                                     (f32(0.0175781), f32(-0.0703125), f32(0.0410156)), (f32(3),) * 3, (512,) * 3,
                                     0, 512 ** 3)
    assert (tmp_path / "rb.txt").read_text() == expect
    assert expect.startswith("3x500x7 r3x-12x7 r0.0175781x-0.0703125x0.0410156 r3x3x3 r512x512x512 r0r134217728r")
    raw = (tmp_path / "rb.bin").read_bytes()
    assert np.frombuffer(raw, np.int32, 1)[0] == 1
    ints = np.frombuffer(raw, np.int32, 18, 4)
    floats = np.frombuffer(raw, np.float32, 18, 4)
    assert list(ints[0:3]) == [0, 0, 512 ** 3]          # start_index, end_index (unset), buffer_length
    assert list(ints[3:6]) == [3, 500, 7] and list(ints[15:18]) == [512, 512, 512]
    np.testing.assert_array_equal(floats[6:9], [3, -12, 7])
    np.testing.assert_allclose(floats[9:12], [0.0175781, -0.0703125, 0.0410156], rtol=1e-6)
