// tde_common.cuh -- types, cyclic addressing and TSDF storage shared by every
// kernel of the GB300 KinectFusion pipeline.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stddef.h>
#include <type_traits>

#include "../../include/tde_capi.h"

// ---------------------------------------------------------------------------
// Layouts must be byte-identical to the reference's shared host/device types.
// ---------------------------------------------------------------------------
static_assert(sizeof(tde_point3f) == 12, "point_3f");
static_assert(sizeof(tde_point3i) == 12, "point_3i");
static_assert(sizeof(tde_matrix3f) == 36, "matrix_3f");
static_assert(sizeof(tde_intrinsics) == 24, "intrinsics");
static_assert(sizeof(tde_round_buffer) == 72, "round_buffer");
static_assert(offsetof(tde_round_buffer, origin_GRID) == 12, "round_buffer.origin_GRID");
static_assert(offsetof(tde_round_buffer, volume_size) == 48, "round_buffer.volume_size");
static_assert(offsetof(tde_round_buffer, voxels_size) == 60, "round_buffer.voxels_size");
static_assert(sizeof(tde_tsdf_i16) == 4, "Tsdf");
static_assert(sizeof(tde_color) == 4, "Color");
static_assert(sizeof(tde_xyzi) == 16, "XYZI");

#define TDE_MAX_DEPTH_VALUE 32767  // common/inc/common_defines.h:6
#define TDE_MAX_TSDF_WEIGHT 128    // common/inc/common_defines.h:10

namespace tde {

// Reports a failure to the thread-local error slot and returns its code.
int set_error(int code, const char *fmt, ...);
// Maps the last CUDA launch error to a status code.
int check_launch(const char *what);
inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }
inline int cuda_fail(cudaError_t e, const char *what) {
    return set_error(e == cudaErrorMemoryAllocation ? TDE_ERR_OOM : TDE_ERR_CUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

#define TDE_CUDA(call, what)                                    \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return ::tde::cuda_fail(e_, what); \
    } while (0)
#define TDE_TRY(call)                \
    do {                             \
        int s_ = (call);             \
        if (s_ != TDE_OK) return s_; \
    } while (0)

// ---------------------------------------------------------------------------
// OpenCL min/max for floats: max(x, y) = x < y ? y : x.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float cl_fmax(float a, float b) { return a < b ? b : a; }
__host__ __device__ __forceinline__ float cl_fmin(float a, float b) { return b < a ? b : a; }

// ---------------------------------------------------------------------------
// Cyclic address of logical voxel (x,y,z): GPU/opencl/raycast.cl:29-47.
// Same int arithmetic; v % n is replaced by a conditional subtract on the
// range [0, 2n) where the two agree.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int wrap_mod(int v, int n) {
    if (v >= 0 && v < 2 * n) return v >= n ? v - n : v;
    return v % n;
}

__host__ __device__ __forceinline__ size_t voxel_address(int x, int y, int z, const tde_round_buffer &rb) {
    int px = wrap_mod(x + rb.origin_GRID.x, rb.voxels_size.x);
    int py = wrap_mod(y + rb.origin_GRID.y, rb.voxels_size.y);
    int pz = wrap_mod(z + rb.origin_GRID.z, rb.voxels_size.z);
    size_t a = (size_t)(long)(rb.voxels_size.x * rb.voxels_size.y * pz + rb.voxels_size.x * py + px);
    a += (size_t)(long)rb.start_index;
    if (a > (size_t)(long)rb.buffer_length) a %= (size_t)(long)rb.buffer_length;
    return a;
}

// "black zone" membership: scan_slice_of_both_volumes.cl:63-74 (OR over axes).
__host__ __device__ __forceinline__ bool in_black_zone(int x, int y, int z, const tde_point3i &mn,
                                                      const tde_point3i &mx, const tde_round_buffer &rb) {
    int ix = x + rb.origin_GRID.x, iy = y + rb.origin_GRID.y, iz = z + rb.origin_GRID.z;
    return (ix >= mn.x && ix <= mx.x) || (iy >= mn.y && iy <= mx.y) || (iz >= mn.z && iz <= mx.z);
}

// ---------------------------------------------------------------------------
// TSDF storage.  `n` is the voxel count (the F32 weight plane follows the
// value plane).
// ---------------------------------------------------------------------------
template <int FMT> struct TsdfStore;

// Packed 32-bit records: I16 {int16 v, int16 w} and F16 {half f, uint16 w}.
template <> struct TsdfStore<TDE_TSDF_I16> {
    static constexpr int bytes_per_voxel = 4;
    typedef uint32_t Raw;
    __device__ __forceinline__ static float value(const void *base, size_t i, size_t) {
        int v = reinterpret_cast<const tde_tsdf_i16 *>(base)[i].value;
        return (float)v / (float)TDE_MAX_DEPTH_VALUE;
    }
    // value() through the read-only path (the volume must not change during the kernel)
    __device__ __forceinline__ static float value_ro(const void *base, size_t i, size_t) {
        int v = __ldg(reinterpret_cast<const short *>(base) + 2 * i);
        return (float)v / (float)TDE_MAX_DEPTH_VALUE;
    }
    __device__ __forceinline__ static Raw load_raw(const void *base, size_t i, size_t) {
        return __ldg(reinterpret_cast<const uint32_t *>(base) + i);
    }
    __device__ __forceinline__ static void decode(Raw raw, float &f, int &w) {
        int v = (int)(int16_t)(raw & 0xffffu);
        w = (int)(int16_t)(raw >> 16);
        f = (float)v / (float)TDE_MAX_DEPTH_VALUE;
    }
    // set_tsdf: raycast.cl:18-27 (convert_int_rtz, clamp to +-32767)
    __device__ __forceinline__ static Raw encode(float f, int w) {
        int q = __float2int_rz(f * (float)TDE_MAX_DEPTH_VALUE);
        q = max(-TDE_MAX_DEPTH_VALUE, min(TDE_MAX_DEPTH_VALUE, q));
        return (uint32_t)(uint16_t)(int16_t)q | ((uint32_t)(uint16_t)(int16_t)w << 16);
    }
    __device__ __forceinline__ static bool same(Raw a, Raw b) { return a == b; }
    __device__ __forceinline__ static void store_raw(void *base, size_t i, size_t, Raw r) {
        reinterpret_cast<uint32_t *>(base)[i] = r;
    }
    __device__ __forceinline__ static void clear(void *base, size_t i, size_t) {
        reinterpret_cast<uint32_t *>(base)[i] = 0u;
    }
};

template <> struct TsdfStore<TDE_TSDF_F16> {
    static constexpr int bytes_per_voxel = 4;
    typedef uint32_t Raw;
    __device__ __forceinline__ static float value(const void *base, size_t i, size_t) {
        return __half2float(reinterpret_cast<const __half *>(base)[2 * i]);
    }
    __device__ __forceinline__ static float value_ro(const void *base, size_t i, size_t) {
        return __half2float(__ushort_as_half(__ldg(reinterpret_cast<const unsigned short *>(base) + 2 * i)));
    }
    __device__ __forceinline__ static Raw load_raw(const void *base, size_t i, size_t) {
        return __ldg(reinterpret_cast<const uint32_t *>(base) + i);
    }
    __device__ __forceinline__ static void decode(Raw raw, float &f, int &w) {
        f = __half2float(__ushort_as_half((unsigned short)(raw & 0xffffu)));
        w = (int)(raw >> 16);
    }
    __device__ __forceinline__ static Raw encode(float f, int w) {
        return (uint32_t)__half_as_ushort(__float2half_rn(f)) | ((uint32_t)(uint16_t)w << 16);
    }
    __device__ __forceinline__ static bool same(Raw a, Raw b) { return a == b; }
    __device__ __forceinline__ static void store_raw(void *base, size_t i, size_t, Raw r) {
        reinterpret_cast<uint32_t *>(base)[i] = r;
    }
    __device__ __forceinline__ static void clear(void *base, size_t i, size_t) {
        reinterpret_cast<uint32_t *>(base)[i] = 0u;
    }
};

// Planar: float f[n] followed by uint16 w[n].
struct TsdfRawF32 { float f; int w; };
template <> struct TsdfStore<TDE_TSDF_F32> {
    static constexpr int bytes_per_voxel = 6;
    typedef TsdfRawF32 Raw;
    __device__ __forceinline__ static float value(const void *base, size_t i, size_t) {
        return reinterpret_cast<const float *>(base)[i];
    }
    __device__ __forceinline__ static float value_ro(const void *base, size_t i, size_t) {
        return __ldg(reinterpret_cast<const float *>(base) + i);
    }
    __device__ __forceinline__ static const unsigned short *wplane(const void *base, size_t n) {
        return reinterpret_cast<const unsigned short *>(reinterpret_cast<const float *>(base) + n);
    }
    __device__ __forceinline__ static Raw load_raw(const void *base, size_t i, size_t n) {
        return Raw{__ldg(reinterpret_cast<const float *>(base) + i), (int)__ldg(wplane(base, n) + i)};
    }
    __device__ __forceinline__ static void decode(Raw raw, float &f, int &w) { f = raw.f; w = raw.w; }
    __device__ __forceinline__ static Raw encode(float f, int w) { return Raw{f, w}; }
    __device__ __forceinline__ static bool same(Raw a, Raw b) {
        return __float_as_uint(a.f) == __float_as_uint(b.f) && a.w == b.w;
    }
    __device__ __forceinline__ static void store_raw(void *base, size_t i, size_t n, Raw r) {
        reinterpret_cast<float *>(base)[i] = r.f;
        const_cast<unsigned short *>(wplane(base, n))[i] = (unsigned short)r.w;
    }
    __device__ __forceinline__ static void clear(void *base, size_t i, size_t n) { store_raw(base, i, n, Raw{0.f, 0}); }
};

inline size_t voxel_count(const tde_round_buffer &rb) {
    return (size_t)rb.voxels_size.x * (size_t)rb.voxels_size.y * (size_t)rb.voxels_size.z;
}

bool valid_round_buffer(const tde_round_buffer *rb);
inline bool valid_format(int f) { return f == TDE_TSDF_I16 || f == TDE_TSDF_F16 || f == TDE_TSDF_F32; }

// Dispatch a functor templated on the TSDF format.
template <class F> int dispatch_format(int fmt, F &&f) {
    switch (fmt) {
    case TDE_TSDF_I16: return f(std::integral_constant<int, TDE_TSDF_I16>());
    case TDE_TSDF_F16: return f(std::integral_constant<int, TDE_TSDF_F16>());
    case TDE_TSDF_F32: return f(std::integral_constant<int, TDE_TSDF_F32>());
    default: return set_error(TDE_ERR_INVALID_ARG, "unknown TSDF format %d", fmt);
    }
}

inline unsigned div_up(unsigned a, unsigned b) { return (a + b - 1) / b; }

}  // namespace tde
