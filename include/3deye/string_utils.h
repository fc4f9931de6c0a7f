/*
 * string_utils.h -- the reference's text output of points, 3x3 matrices,
 * point records and trajectories, header-only:
 *   point_3f / point_3i   "axbxc "   common/inc/types/elementary_point_template.h:182-194
 *   matrix_3f             rows joined by newlines, then " "
 *                                    common/inc/types/elementary_matrix_template.h:61-73
 *   XYZI                  "xxyxzxw"  common/src/base_points.cpp:571-574 (reader :550-568)
 *   Color                 "r.g.b.w " common/src/base_points.cpp:279-282 (reader :251-276)
 *   Point<T>              as T       common/inc/types/base_point_interface.hpp:46-62
 *   round_buffer          "<p>r" x5, "start r length r "  common/src/round_buffer.cpp:99-113
 *   write_isometry_to_file           common/src/string_utils.cpp:26-74
 * Floats print with the stream's defaults (6 significant digits).  The
 * Python twin (3deye_gb300/formats.py) writes the same bytes.
 */
#ifndef TDE_3DEYE_STRING_UTILS_H
#define TDE_3DEYE_STRING_UTILS_H

#include <algorithm>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "tde_types.h"

inline void replaceAll(std::string &str, const std::string &from, const std::string &to) {
    if (from.empty()) return;
    for (size_t pos = str.find(from); pos != std::string::npos; pos = str.find(from, pos + to.size()))
        str.replace(pos, from.size(), to);
}

inline std::ostream &operator<<(std::ostream &out, const point_3f &p) {
    return out << p.x << 'x' << p.y << 'x' << p.z << ' ';
}
inline std::ostream &operator<<(std::ostream &out, const point_3i &p) {
    return out << p.x << 'x' << p.y << 'x' << p.z << ' ';
}
inline std::ostream &operator<<(std::ostream &out, const matrix_3f &m) {
    return out << m.data[0] << std::endl << m.data[1] << std::endl << m.data[2] << ' ';
}
inline std::ostream &operator<<(std::ostream &out, const XYZI &v) {
    return out << v.x << 'x' << v.y << 'x' << v.z << 'x' << v.w;
}
inline std::ostream &operator<<(std::ostream &out, const Color &c) {
    return out << (unsigned)c.r << '.' << (unsigned)c.g << '.' << (unsigned)c.b << '.' << (unsigned)c.w << ' ';
}
template <class T> std::ostream &operator<<(std::ostream &out, const Point<T> &p) { return out << p.data; }

inline std::istream &operator>>(std::istream &in, XYZI &v) {
    std::string s;
    in >> s;
    replaceAll(s, "x", " ");
    std::istringstream t(s);
    t >> v.x >> v.y >> v.z >> v.w;
    return in;
}
inline std::istream &operator>>(std::istream &in, Color &c) {
    std::string s;
    in >> s;
    replaceAll(s, ".", " ");
    std::istringstream t(s);
    unsigned short r = 0, g = 0, b = 0, w = 0;
    t >> r >> g >> b >> w;
    c.r = (unsigned char)r; c.g = (unsigned char)g; c.b = (unsigned char)b; c.w = (unsigned char)w;
    return in;
}
template <class T> std::istream &operator>>(std::istream &in, Point<T> &p) { return in >> p.data; }

/* round_buffer as common/src/round_buffer.cpp:99-113 writes it: origin_GRID,
 * origin_GRID_global, origin_metric, volume_size and voxels_size (points,
 * "axbxc "), start_index and buffer_length, each followed by "r", then a
 * space. */
inline std::ostream &operator<<(std::ostream &out, const round_buffer &rb) {
    return out << rb.origin_GRID << 'r' << rb.origin_GRID_global << 'r' << rb.origin_metric << 'r' << rb.volume_size
               << 'r' << rb.voxels_size << 'r' << rb.start_index << 'r' << rb.buffer_length << 'r' << ' ';
}
/* Reads the whole record back (six whitespace-separated tokens; the
 * reference's reader, round_buffer.cpp:76-97, takes one token, which ends
 * after the first point). */
inline std::istream &operator>>(std::istream &in, round_buffer &rb) {
    std::string rec, tok;
    for (int k = 0; k < 6 && in >> tok; ++k) rec += tok + " ";
    replaceAll(rec, "x", " ");
    replaceAll(rec, "r", " ");
    std::istringstream t(rec);
    t >> rb.origin_GRID.x >> rb.origin_GRID.y >> rb.origin_GRID.z >> rb.origin_GRID_global.x >>
        rb.origin_GRID_global.y >> rb.origin_GRID_global.z >> rb.origin_metric.x >> rb.origin_metric.y >>
        rb.origin_metric.z >> rb.volume_size.x >> rb.volume_size.y >> rb.volume_size.z >> rb.voxels_size.x >>
        rb.voxels_size.y >> rb.voxels_size.z >> rb.start_index >> rb.buffer_length;
    if (!t) in.setstate(std::ios::failbit);
    return in;
}

/* write_isometry_to_file: per pose its index, R (matrix_3f) and t
 * (vector_3f), each followed by a newline.  A null name throws (the
 * reference rethrows with no active exception, which terminates). */
inline void write_isometry_to_file(const char *file_name, const matrix_3f *R, const vector_3f *t, size_t n) {
    if (!file_name) throw std::invalid_argument("write_isometry_to_file: bad file name");
    std::ofstream out(file_name);
    if (!out.is_open()) return;
    for (size_t i = 0; i < n; ++i) out << i << std::endl << R[i] << std::endl << t[i] << std::endl;
}

/* The reference's overloads take std::vector<Eigen::Affine3d> /
 * std::vector<Eigen::Isometry3d>; any type with rotation() and translation()
 * indexable as (r, c) / (r) binds here, cast to float as there. */
template <class Iso> void write_isometry_to_file(const char *file_name, std::vector<Iso> &data) {
    std::vector<matrix_3f> R(data.size());
    std::vector<vector_3f> t(data.size());
    for (size_t i = 0; i < data.size(); ++i) {
        const auto rot = data[i].rotation();
        const auto tr = data[i].translation();
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) R[i].data[r].data[c] = (float)rot(r, c);
            t[i].data[r] = (float)tr(r);
        }
    }
    write_isometry_to_file(file_name, R.data(), t.data(), data.size());
}

#endif
