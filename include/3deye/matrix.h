/*
 * matrix.h -- the host container matrix<T> of the reference
 * (common/inc/matrix.h:13-79, impl/matrix.hpp), reduced to what the pipeline
 * API uses: sized construction, element access, extend_from (concatenation,
 * used to gather slab points), the size queries, and the text file format
 * (operator<<, Save_To_File, Fill_From_File: impl/matrix.hpp:400-540).
 */
#ifndef TDE_3DEYE_MATRIX_H
#define TDE_3DEYE_MATRIX_H

#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <typeinfo>
#include <vector>

#include "string_utils.h"
#include "tde_types.h"

template <class T> class matrix {
  public:
    T *data = nullptr;
    matrix() : sz(0, 1, 1) {}
    explicit matrix(unsigned int n) : sz(n, 1, 1), buf(n) { data = buf.empty() ? nullptr : buf.data(); }
    explicit matrix(dim3 s) : sz(s), buf(s.x * s.y * s.z) { data = buf.empty() ? nullptr : buf.data(); }
    matrix(const matrix &o) : sz(o.sz), buf(o.buf) { data = buf.empty() ? nullptr : buf.data(); }
    matrix &operator=(const matrix &o) {
        sz = o.sz; buf = o.buf; data = buf.empty() ? nullptr : buf.data();
        return *this;
    }
    T &operator[](size_t i) {
        if (i >= buf.size()) throw std::out_of_range("matrix index");
        return buf[i];
    }
    const T &operator[](size_t i) const {
        if (i >= buf.size()) throw std::out_of_range("matrix index");
        return buf[i];
    }
    dim3 Get_Size() const { return sz; }
    size_t Get_Width() const { return sz.x; }
    size_t Get_Height() const { return sz.y; }
    size_t Get_Depth() const { return sz.z; }
    /* typeid(data).name(), as the reference prints in the file header */
    std::string Get_Matrix_Type() const { return typeid(data).name(); }
    void Set_Dimensions(size_t w, size_t h, size_t d) {
        sz = dim3(w, h, d);
        buf.assign(w * h * d, T());
        data = buf.empty() ? nullptr : buf.data();
    }
    /* Save_To_File: "W H D type" then one line per row, each element
     * followed by a space; an empty name makes "WxHxD-type.tst". */
    void Save_To_File(const std::string &custom_file_name) const {
        std::string name = custom_file_name;
        if (name.empty()) {
            std::ostringstream g;
            g << sz.x << "x" << sz.y << "x" << sz.z << "-" << Get_Matrix_Type() << ".tst";
            name = g.str();
        }
        std::ofstream f(name.c_str());
        if (f.is_open()) f << *this;
    }
    /* Fill_From_File: 0 on success, -1 on a missing file or a row whose
     * element count differs from the width (the type name is not checked,
     * as there); rows beyond height * depth are refused instead of written
     * past the end. */
    int Fill_From_File(const std::string &file_name) {
        if (file_name.empty()) return -1;
        std::ifstream f(file_name.c_str());
        if (!f.is_open()) return -1;
        std::string line, type;
        std::getline(f, line);
        std::istringstream head(line);
        size_t w = 0, h = 0, d = 0;
        if (!(head >> w >> h >> d)) return -1;
        Set_Dimensions(w, h, d);
        size_t row = 0;
        while (std::getline(f, line)) {
            if (row >= h * d) return line.find_first_not_of(" \t\r") == std::string::npos ? 0 : -1;
            std::istringstream in(line);
            size_t col = 0;
            T v;
            while (col <= w && in >> v) {
                if (col < w) buf[row * w + col] = v;
                ++col;
            }
            if (col != w) return -1;
            ++row;
        }
        return 0;
    }
    friend std::ostream &operator<<(std::ostream &out, const matrix &m) {
        out << m.sz.x << " " << m.sz.y << " " << m.sz.z << " " << m.Get_Matrix_Type() << std::endl;
        for (size_t r = 0; r < m.sz.y * m.sz.z; ++r) {
            for (size_t c = 0; c < m.sz.x; ++c) out << m.buf[r * m.sz.x + c] << " ";
            out << std::endl;
        }
        return out;
    }
    unsigned int Get_Num_Of_Elem() const { return (unsigned)buf.size(); }
    void extend_from(const matrix &o) {
        buf.insert(buf.end(), o.buf.begin(), o.buf.end());
        sz = dim3(buf.size(), 1, 1);
        data = buf.empty() ? nullptr : buf.data();
    }

  private:
    dim3 sz;
    std::vector<T> buf;
};

#endif
