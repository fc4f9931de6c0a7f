/*
 * matrix.h -- the host container matrix<T> of the reference
 * (common/inc/matrix.h:13-79, impl/matrix.hpp), reduced to what the pipeline
 * API uses: sized construction, element access, extend_from (concatenation,
 * used to gather slab points) and the size queries.
 */
#ifndef TDE_3DEYE_MATRIX_H
#define TDE_3DEYE_MATRIX_H

#include <cstring>
#include <stdexcept>
#include <vector>

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
