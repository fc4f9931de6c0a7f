"""On-disk text formats of 3deye's host code: trajectories and point clouds.

* Trajectory -- write_isometry_to_file (common/src/string_utils.cpp:26-74):
  per pose, its index on one line, then the rotation as matrix_3f and the
  translation as vector_3f, both cast to float.  A matrix_3f prints its three
  rows separated by newlines and then one space
  (common/inc/types/elementary_matrix_template.h:61-73); a point prints its
  components joined by "x" and then one space
  (common/inc/types/elementary_point_template.h:182-194).

* Image -- binary PPM (P6) of an RGB8 image, the headless output of
  Generate_Image (the reference draws it in a window).

* Cloud -- matrix<T>::Save_To_File (common/inc/impl/matrix.hpp:413-476): a
  header line "width height depth typename", then one line per row of
  elements, each element followed by a space.  A cloud is one row
  (matrix(n) is n x 1 x 1).  XYZI prints "x"-joined floats
  (common/src/base_points.cpp:571-574); Color prints "."-joined unsigned
  bytes and a space (base_points.cpp:279-282).  The typename is
  typeid(T *).name() as GCC spells it; the reader ignores it, as
  matrix<T>::Fill_From_File does (impl/matrix.hpp:491-540).

Floats print as std::ostream prints them by default: 6 significant digits,
"%g".  The C++ twins of these writers are in include/3deye/string_utils.h and
include/3deye/matrix.h; the two produce identical bytes.
"""
from __future__ import annotations

import numpy as np

XYZI_TYPENAME = "P5PointI4XYZIE"
COLOR_TYPENAME = "P5PointI5ColorE"


def _g(v) -> str:
    return "%g" % float(v)


def format_point(p) -> str:
    """point_3f / vector_3f: "axbxc " (elementary_point_template.h:182-194)."""
    return "x".join(_g(v) for v in p) + " "


def format_matrix3(R) -> str:
    """matrix_3f: rows joined by newlines, then a space."""
    return "\n".join(format_point(r) for r in R) + " "


def _poses_rt(poses):
    a = np.asarray(poses, np.float64)
    if a.ndim == 2 and a.shape[1] == 12:  # pipeline pose: R row-major, then t
        return a[:, :9].reshape(-1, 3, 3), a[:, 9:]
    if a.ndim == 3 and a.shape[1:] in ((4, 4), (3, 4)):
        return a[:, :3, :3], a[:, :3, 3]
    raise ValueError(f"poses must be [n, 12], [n, 3, 4] or [n, 4, 4], got {a.shape}")


def format_trajectory(poses) -> str:
    R, t = _poses_rt(poses)
    R, t = R.astype(np.float32), t.astype(np.float32)  # rotation().cast<float>()
    return "".join(f"{i}\n{format_matrix3(R[i])}\n{format_point(t[i])}\n" for i in range(len(R)))


def write_trajectory(path, poses) -> None:
    """write_isometry_to_file: poses as [n, 12] (R row-major, t), [n, 3, 4] or [n, 4, 4]."""
    with open(path, "w", newline="\n") as f:
        f.write(format_trajectory(poses))


def read_trajectory(path) -> np.ndarray:
    """Inverse of write_trajectory: [n, 4, 4] float64 poses (float precision)."""
    lines = open(path).read().split("\n")
    out = []
    i = 0
    while i + 4 < len(lines) and lines[i].strip():
        idx = int(lines[i])
        if idx != len(out):
            raise ValueError(f"trajectory: pose index {idx} out of order")
        rows = [[float(v) for v in lines[i + 1 + r].split()[0].split("x")] for r in range(3)]
        t = [float(v) for v in lines[i + 4].split()[0].split("x")]
        m = np.eye(4)
        m[:3, :3], m[:3, 3] = rows, t
        out.append(m)
        i += 5
    return np.array(out).reshape(-1, 4, 4)


def format_xyzi(p) -> str:
    return "x".join(_g(v) for v in p)


def format_color(c) -> str:
    return ".".join(str(int(v)) for v in c) + " "


def format_cloud(points=None, colors=None) -> str:
    """matrix<Point_XYZI> (points [n, 4] float) or matrix<Point_Color>
    (colors [n, 4] uint8) as Save_To_File writes it."""
    if (points is None) == (colors is None):
        raise ValueError("give points or colors")
    if points is not None:
        a = np.asarray(points, np.float32).reshape(-1, 4)
        body = "".join(format_xyzi(p) + " " for p in a)
        name = XYZI_TYPENAME
    else:
        a = np.asarray(colors, np.uint8).reshape(-1, 4)
        body = "".join(format_color(c) + " " for c in a)
        name = COLOR_TYPENAME
    return f"{len(a)} 1 1 {name}\n{body}\n"


def write_cloud(path, points=None, colors=None) -> None:
    with open(path, "w", newline="\n") as f:
        f.write(format_cloud(points, colors))


def read_cloud(path):
    """Fill_From_File for a cloud written by write_cloud: float32 [n, 4] for
    XYZI elements, uint8 [n, 4] for Color elements."""
    with open(path) as f:
        head = f.readline().split()
        width, height, depth = int(head[0]), int(head[1]), int(head[2])
        if height * depth != 1:
            raise ValueError("read_cloud: a cloud is one row")
        toks = f.read().split()
    if len(toks) != width:
        raise ValueError(f"read_cloud: {len(toks)} elements, header says {width}")
    if not toks:
        return np.zeros((0, 4), np.float32)
    if "." in toks[0] and "x" not in toks[0]:
        return np.array([[int(v) for v in t.split(".")] for t in toks], np.uint8).reshape(-1, 4)
    return np.array([[float(v) for v in t.split("x")] for t in toks], np.float32).reshape(-1, 4)


def write_ppm(path, image) -> None:
    """RGB8 image uint8 [rows, cols, 3] as binary PPM (P6, maxval 255)."""
    a = np.ascontiguousarray(image, np.uint8)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError(f"image must be [rows, cols, 3], got {a.shape}")
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
        f.write(a.tobytes())


def read_ppm(path) -> np.ndarray:
    """Inverse of write_ppm."""
    raw = open(path, "rb").read()
    parts = raw.split(b"\n", 3)
    if len(parts) < 4 or parts[0] != b"P6" or parts[2] != b"255" or len(parts[1].split()) != 2:
        raise ValueError("read_ppm: not a binary 8-bit PPM as write_ppm writes it")
    cols, rows = (int(v) for v in parts[1].split())
    if len(parts[3]) < rows * cols * 3:
        raise ValueError(f"read_ppm: {cols}x{rows} pixels do not fit in the file")
    return np.frombuffer(parts[3], np.uint8, rows * cols * 3).reshape(rows, cols, 3)


def format_round_buffer(origin_grid, origin_grid_global, origin_metric, volume_size, voxels_size, start_index,
                        buffer_length) -> str:
    """round_buffer's text record (common/src/round_buffer.cpp:99-113): the five
    points "axbxc " each followed by "r", then start_index and buffer_length
    each followed by "r", then a space."""
    pts = (origin_grid, origin_grid_global, origin_metric, volume_size, voxels_size)
    return "".join(format_point(p) + "r" for p in pts) + f"{int(start_index)}r{int(buffer_length)}r "
