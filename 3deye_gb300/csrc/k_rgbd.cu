// k_rgbd.cu -- dense RGB-D (photometric) odometry: the reference's second
// tracker (Estimate_Isometry_By_RGBD and its stages, common/src/
// opencl_wrappers.cpp:345-362, 1008-1466) after the RGB-D odometry of
// OpenCV's contrib rgbd module (Steinbruecker, Sturm, Cremers 2011).
//
// Per frame: 8-bit intensity and metric depth, a pyramid, 3x3 Sobel
// derivatives of the current frame.  Per Gauss-Newton step, two passes over
// the previous frame's pixels of the level: the first finds each pixel's
// correspondence in the current frame (projective transform R' = K R K^-1,
// t' = K t, depth and gradient tests) and sums the squared intensity
// differences -- integers, so the sum is exact in any order; the second
// forms sigma from those sums, each kept pair's weighted Jacobian row and the
// 27 terms of [A | b], reduced per block in float in a fixed order; the last
// block of that pass sums the blocks in float-float, solves (the ICP path's
// solve) and moves the FP64 pose (T <- exp(xi) T).  Every step is two
// launches: the pose lives on the device, nothing waits on the host.
//
// Built with -fmad=false: the pair tests and row values are the same IEEE
// operations as the CPU oracle (oracle/oracle_rgbd.c), explicit fused
// multiply-adds written out on both sides.
#include <cmath>
#include <utility>

#include "tde_common.cuh"
#include "tde_icp.cuh"
#include "tde_solve.cuh"

namespace tde {
namespace {

constexpr int kThreads = 256;
// The odometry passes: 512 threads x 4 pixels, 150 blocks at 640x480 (one per
// SM).  Measured per 640x480 frame (graphs): 0.504 ms against 0.579 with
// 256 x 8 -- the same pixels per SM with twice the warps to cover the
// gathers' and reductions' latencies.
constexpr int kOdoThreads = 512;  // threads a block in the odometry passes
constexpr int kPix = 4;           // pixels per thread in the odometry passes
constexpr float kSobelScale = 0.125f;  // SOBEL_SCALE, compute_least_squares_equation.cl:8

inline unsigned odo_blocks(int W, int H) { return div_up((unsigned)(W * H), (unsigned)(kOdoThreads * kPix)); }

__global__ void prepare_kernel(const uint16_t *__restrict__ depth, const uint8_t *__restrict__ rgb, int n,
                               uint8_t *__restrict__ I, float *__restrict__ D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    I[i] = (uint8_t)((r * 4899u + g * 9617u + b * 1868u + 8192u) >> 14);  // BT.601 luma, 14-bit fixed point
    D[i] = __fmul_rn((float)depth[i], 0.001f);
}

__global__ void pyramid_kernel(const uint8_t *__restrict__ I, const float *__restrict__ D, int W, int H,
                               uint8_t *__restrict__ I2, float *__restrict__ D2) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W2 = W >> 1, H2 = H >> 1;
    if (x >= W2 || y >= H2) return;
    const size_t s = (size_t)(2 * y) * W + 2 * x;
    I2[(size_t)y * W2 + x] = (uint8_t)((I[s] + I[s + 1] + I[s + W] + I[s + W + 1] + 2u) >> 2);
    D2[(size_t)y * W2 + x] = D[s];
}

__global__ void sobel_kernel(const uint8_t *__restrict__ I, int W, int H, int16_t *__restrict__ dx,
                             int16_t *__restrict__ dy) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t o = (size_t)y * W + x;
    if (x == 0 || y == 0 || x == W - 1 || y == H - 1) {
        dx[o] = 0;
        dy[o] = 0;
        return;
    }
    const int a = I[o - W - 1], b = I[o - W], c = I[o - W + 1];
    const int d = I[o - 1], f = I[o + 1];
    const int g = I[o + W - 1], h = I[o + W], k = I[o + W + 1];
    dx[o] = (int16_t)((c + 2 * f + k) - (a + 2 * d + g));
    dy[o] = (int16_t)((g + 2 * h + k) - (a + 2 * b + c));
}

// ---- points of interest: per-row counts, one scan over rows, per-row scatter ----
__device__ __forceinline__ bool textured(const int16_t *dx, const int16_t *dy, size_t i, float scale) {
    const int g = dx[i] * dx[i] + dy[i] * dy[i];
    return (float)g >= scale;
}

__global__ void points_count_kernel(const int16_t *__restrict__ dx, const int16_t *__restrict__ dy, int W,
                                    float scale, uint32_t *__restrict__ counts) {
    __shared__ unsigned s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    const size_t row = (size_t)blockIdx.x * W;
    unsigned c = 0;
    for (int x = threadIdx.x; x < W; x += blockDim.x) c += textured(dx, dy, row + x, scale);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0) counts[blockIdx.x] = s;
}

// Exclusive scan of n counts in place by one block; total to *total.
__global__ void scan_counts_kernel(uint32_t *__restrict__ a, int n, uint32_t *__restrict__ total) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + tid;
        const uint32_t v = i < n ? a[i] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            const int nw = blockDim.x >> 5;
            uint32_t w = lane < nw ? warp_sums[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < nw) warp_sums[lane] = w;
        }
        __syncthreads();
        const uint32_t before = carry + (warp ? warp_sums[warp - 1] : 0u) + x - v;
        if (i < n) a[i] = before;
        __syncthreads();
        if (tid == blockDim.x - 1) carry = before + v;
        __syncthreads();
    }
    if (tid == 0) *total = carry;
}

__global__ void points_scatter_kernel(const int16_t *__restrict__ dx, const int16_t *__restrict__ dy, int W,
                                      float scale, const uint32_t *__restrict__ offs, tde_point2i *__restrict__ pts,
                                      uint32_t capacity) {
    __shared__ unsigned s_warp[kThreads / 32];
    __shared__ unsigned s_base;
    const int y = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_base = offs[y];
    __syncthreads();
    const size_t row = (size_t)y * W;
    for (int x0 = 0; x0 < W; x0 += kThreads) {
        const int x = x0 + threadIdx.x;
        const bool set = x < W && textured(dx, dy, row + x, scale);
        const unsigned m = __ballot_sync(0xffffffffu, set);
        if (lane == 0) s_warp[warp] = __popc(m);
        __syncthreads();
        if (set) {
            unsigned before = 0;
            for (int w = 0; w < warp; ++w) before += s_warp[w];
            const uint32_t slot = s_base + before + __popc(m & ((1u << lane) - 1u));
            if (slot < capacity) pts[slot] = tde_point2i{x, y};
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (int w = 0; w < kThreads / 32; ++w) t += s_warp[w];
            s_base += t;
        }
        __syncthreads();
    }
}

// ---- correspondences and rows: the oracle's operations, in its order ----
struct Level {
    const uint8_t *Ip, *Ic;
    const float *Dp, *Dc;
    const int16_t *dx, *dy;
    int W, H;
    float fx, fy, cx, cy;
    float mdd, maxd, grad2;
    double ifx, ify;  // 1 / fx, 1 / fy in FP64 (host-computed)
};

// One piece of R' = K R K^-1, t' = K t (FP64, explicit fused operations,
// then float) and of the float pose M: row t of R' for t < 3, t' for t = 3;
// threads 4..15 convert pose entry t - 4.  Threads 0..15 of a block run it
// side by side (the FP64 pipe is narrow: one thread doing everything
// serialises several microseconds of dependent FP64 work).
__device__ __forceinline__ void projective_part(int t, const double *pose, const Level &L, float *proj, float *M) {
    const double fx = L.fx, fy = L.fy, cx = L.cx, cy = L.cy;
    const double *R = pose, *tv = pose + 9;
    if (t < 3) {
        const int i = t;  // R'[i][.] = (K R)[i][.] K^-1
        double m0, m1, m2;
        if (i == 0) {
            m0 = __fma_rn(fx, R[0], __dmul_rn(cx, R[6]));
            m1 = __fma_rn(fx, R[1], __dmul_rn(cx, R[7]));
            m2 = __fma_rn(fx, R[2], __dmul_rn(cx, R[8]));
        } else if (i == 1) {
            m0 = __fma_rn(fy, R[3], __dmul_rn(cy, R[6]));
            m1 = __fma_rn(fy, R[4], __dmul_rn(cy, R[7]));
            m2 = __fma_rn(fy, R[5], __dmul_rn(cy, R[8]));
        } else {
            m0 = R[6];
            m1 = R[7];
            m2 = R[8];
        }
        const double a = __dmul_rn(m0, L.ifx), b = __dmul_rn(m1, L.ify);
        proj[3 * i] = (float)a;
        proj[3 * i + 1] = (float)b;
        proj[3 * i + 2] = (float)(m2 - __fma_rn(a, cx, __dmul_rn(b, cy)));
    } else if (t == 3) {
        proj[9] = (float)__fma_rn(fx, tv[0], __dmul_rn(cx, tv[2]));
        proj[10] = (float)__fma_rn(fy, tv[1], __dmul_rn(cy, tv[2]));
        proj[11] = (float)tv[2];
    } else if (t < 16) {
        M[t - 4] = (float)pose[t - 4];
    }
}

__device__ __forceinline__ bool depth_ok(float z, float maxd) { return z > 0.f && z < maxd; }

// Pixel i = (u, v) of the previous frame: its pair in the current frame (j)
// and the intensity difference r, or false.
__device__ __forceinline__ bool find_pair(const Level &L, const float *P, int u, int v, float z, int &j, float &r) {
    if (!depth_ok(z, L.maxd)) return false;
    const float fu = (float)u, fv = (float)v;
    const float px = __fmaf_rn(z, __fmaf_rn(P[1], fv, __fmaf_rn(P[0], fu, P[2])), P[9]);
    const float py = __fmaf_rn(z, __fmaf_rn(P[4], fv, __fmaf_rn(P[3], fu, P[5])), P[10]);
    const float pz = __fmaf_rn(z, __fmaf_rn(P[7], fv, __fmaf_rn(P[6], fu, P[8])), P[11]);
    if (!(pz > 0.f)) return false;
    const float iz = __frcp_rn(pz);
    const int u2 = __float2int_rn(__fmul_rn(px, iz)), v2 = __float2int_rn(__fmul_rn(py, iz));
    if (u2 < 0 || v2 < 0 || u2 >= L.W || v2 >= L.H) return false;
    j = v2 * L.W + u2;
    const float z2 = __ldg(L.Dc + j);
    if (!depth_ok(z2, L.maxd) || !(fabsf(pz - z2) < L.mdd)) return false;
    if (L.dx) {  // no derivatives: the points were filtered beforehand
        const int gx = __ldg(L.dx + j), gy = __ldg(L.dy + j);
        if (!((float)(gx * gx + gy * gy) >= L.grad2)) return false;
    }
    r = (float)__ldg(L.Ic + j) - (float)__ldg(L.Ip + (size_t)v * L.W + u);
    return true;
}

// The previous frame's depth at K pixels (raster indices i[k]; entries at or
// past W*H are not pixels): independent of the pose, so the step kernels
// issue these loads before waiting for the previous step.
template <int K>
__device__ __forceinline__ void load_depths(const Level &L, const int (&i)[K], float (&z)[K]) {
    const int npix = L.W * L.H;
#pragma unroll
    for (int k = 0; k < K; ++k) z[k] = i[k] < npix ? __ldg(L.Dp + i[k]) : 0.f;
}

// find_pair for the K pixels of load_depths (depths z[k]): the projections,
// then the gathers of every candidate issued together, then the tests -- the
// same operations and results as find_pair, with K load chains in flight
// instead of one.  Bit k of the result is set for a kept pair; j[k], r[k] and
// the current frame's derivatives gx[k], gy[k] at j[k] are valid for those.
template <int K>
__device__ __forceinline__ unsigned find_pairs(const Level &L, const float *P, const int (&i)[K], int (&j)[K],
                                               float (&r)[K], const float (&z)[K], float (&gx)[K], float (&gy)[K]) {
    float pz[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        j[k] = -1;
        pz[k] = 0.f;
        if (!depth_ok(z[k], L.maxd)) continue;
        const float fu = (float)(i[k] % L.W), fv = (float)(i[k] / L.W);
        const float px = __fmaf_rn(z[k], __fmaf_rn(P[1], fv, __fmaf_rn(P[0], fu, P[2])), P[9]);
        const float py = __fmaf_rn(z[k], __fmaf_rn(P[4], fv, __fmaf_rn(P[3], fu, P[5])), P[10]);
        pz[k] = __fmaf_rn(z[k], __fmaf_rn(P[7], fv, __fmaf_rn(P[6], fu, P[8])), P[11]);
        if (!(pz[k] > 0.f)) continue;
        const float iz = __frcp_rn(pz[k]);
        const int u2 = __float2int_rn(__fmul_rn(px, iz)), v2 = __float2int_rn(__fmul_rn(py, iz));
        if (u2 < 0 || v2 < 0 || u2 >= L.W || v2 >= L.H) continue;
        j[k] = v2 * L.W + u2;
    }
    float z2[K];
    int ic[K], ip[K], dx[K], dy[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const bool c = j[k] >= 0;
        z2[k] = c ? __ldg(L.Dc + j[k]) : 0.f;
        dx[k] = c && L.dx ? __ldg(L.dx + j[k]) : 0;
        dy[k] = c && L.dx ? __ldg(L.dy + j[k]) : 0;
        ic[k] = c ? __ldg(L.Ic + j[k]) : 0;
        ip[k] = c ? __ldg(L.Ip + i[k]) : 0;
    }
    unsigned mask = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        bool ok = j[k] >= 0 && depth_ok(z2[k], L.maxd) && fabsf(pz[k] - z2[k]) < L.mdd;
        if (L.dx) ok = ok && (float)(dx[k] * dx[k] + dy[k] * dy[k]) >= L.grad2;
        r[k] = (float)ic[k] - (float)ip[k];
        gx[k] = (float)dx[k];
        gy[k] = (float)dy[k];
        mask |= (unsigned)ok << k;
    }
    return mask;
}

// The 7-vector (C0..C5, -w r) of a kept pair; M = R row-major, t (float).
__device__ __forceinline__ void pair_row(const Level &L, const float *M, int u, int v, float z, float gx, float gy,
                                         float r, float sigma, float ifx, float ify, float row[7]) {
    const float xn = __fmul_rn((float)u - L.cx, ifx), yn = __fmul_rn((float)v - L.cy, ify);
    const float X = __fmul_rn(z, xn), Y = __fmul_rn(z, yn);
    const float Px = __fmaf_rn(M[2], z, __fmaf_rn(M[1], Y, __fmul_rn(M[0], X))) + M[9];
    const float Py = __fmaf_rn(M[5], z, __fmaf_rn(M[4], Y, __fmul_rn(M[3], X))) + M[10];
    const float Pz = __fmaf_rn(M[8], z, __fmaf_rn(M[7], Y, __fmul_rn(M[6], X))) + M[11];
    const float wsum = sigma + fabsf(r);
    const float w = wsum > 2.220446049250313e-16f ? __frcp_rn(wsum) : 1.f;
    const float s0 = __fmul_rn(w, kSobelScale);
    const float iz = __frcp_rn(Pz);
    const float v0 = __fmul_rn(__fmul_rn(__fmul_rn(iz, L.fx), s0), gx);
    const float v1 = __fmul_rn(__fmul_rn(__fmul_rn(iz, L.fy), s0), gy);
    const float v2 = __fmul_rn(-__fmaf_rn(v1, Py, __fmul_rn(v0, Px)), iz);
    row[0] = __fmaf_rn(Py, v2, -__fmul_rn(Pz, v1));
    row[1] = __fmaf_rn(Pz, v0, -__fmul_rn(Px, v2));
    row[2] = __fmaf_rn(Px, v1, -__fmul_rn(Py, v0));
    row[3] = v0;
    row[4] = v1;
    row[5] = v2;
    row[6] = -__fmul_rn(w, r);
}

// Pass 1: kept count and sum of squared differences per block.
__global__ void __launch_bounds__(kOdoThreads) residual_kernel(const Level L, const double *__restrict__ pose,
                                                            unsigned long long *__restrict__ partials) {
    __shared__ float P[12], M[12];
    __shared__ unsigned s_n;
    __shared__ unsigned long long s_r2;
    // the second pass (launched with programmatic serialisation) may start its
    // pose-independent loads now
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    int idx[kPix], j[kPix];
    float r[kPix], z[kPix], gx[kPix], gy[kPix];
#pragma unroll
    for (int k = 0; k < kPix; ++k) idx[k] = blockIdx.x * kOdoThreads * kPix + k * kOdoThreads + threadIdx.x;
    load_depths<kPix>(L, idx, z);
    // launched with programmatic serialisation after the previous step's
    // second pass: its pose update and this pass's writes of the partials
    // that pass read come after this wait (0.507 against 0.514 ms per frame
    // with graphs, 0.551 against 0.595 eager, than a plain launch)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (threadIdx.x < 16) projective_part(threadIdx.x, pose, L, P, M);
    if (threadIdx.x == 0) {
        s_n = 0;
        s_r2 = 0ull;
    }
    __syncthreads();
    unsigned n = 0;
    unsigned long long r2 = 0;  // squared integer differences: exact
    const unsigned kept = find_pairs<kPix>(L, P, idx, j, r, z, gx, gy);
#pragma unroll
    for (int k = 0; k < kPix; ++k)
        if ((kept >> k) & 1u) {
            ++n;
            const int ri = (int)r[k];
            r2 += (unsigned long long)(ri * ri);
        }
    for (int o = 16; o > 0; o >>= 1) {
        n += __shfl_down_sync(0xffffffffu, n, o);
        r2 += __shfl_down_sync(0xffffffffu, r2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s_n, n);
        atomicAdd(&s_r2, r2);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = s_n;
        partials[2 * blockIdx.x + 1] = s_r2;
    }
}

// Pass 2: sigma from pass 1's blocks (integer sums: exact), the rows of the
// kept pairs, per-block float partials of the 27 terms and the count.  With
// SOLVE the last block to finish (a ticket on *counter, which it resets) sums
// every block's partials in float-float (warp w takes blocks w, w + NW, ...,
// then the warp sums in order), and warp 0 solves and moves the pose in
// place: the other blocks read the pose only before taking their tickets.
// Status: bit 0 for a failed solve (too few pairs or A not positive definite;
// the pose is kept), bit 1 for a solved step.  Against per-term butterflies
// with FP64 block and cross-block sums (28 conversions a warp on the FP64
// pipe), these reductions took the frame from 0.640 to 0.579 ms.
template <bool SOLVE>
__global__ void __launch_bounds__(kOdoThreads) lsm_kernel(const Level L, double *__restrict__ pose,
                                                          const unsigned long long *__restrict__ res_partials, int nres,
                                                          float *__restrict__ partials, float *__restrict__ sigma_out,
                                                          unsigned *__restrict__ counter, int *__restrict__ status) {
    constexpr int NW = kOdoThreads / 32;
    __shared__ float P[12], M[12];
    __shared__ float s_sigma;
    __shared__ float red[NW][32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    int idx[kPix], j[kPix];
    float r[kPix], z[kPix], gx[kPix], gy[kPix];
#pragma unroll
    for (int k = 0; k < kPix; ++k) idx[k] = blockIdx.x * kOdoThreads * kPix + k * kOdoThreads + tid;
    load_depths<kPix>(L, idx, z);
    // the first pass's partials and the pose are complete past this point
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (warp == 0) {
        unsigned long long n = 0, s = 0;
        for (int b = lane; b < nres; b += 32) {
            n += res_partials[2 * b];
            s += res_partials[2 * b + 1];
        }
        for (int o = 16; o > 0; o >>= 1) {
            n += __shfl_xor_sync(0xffffffffu, n, o);
            s += __shfl_xor_sync(0xffffffffu, s, o);
        }
        if (lane == 0) {
            s_sigma = n ? __fsqrt_rn((float)((double)s / (double)n)) : 0.f;
            if (sigma_out && blockIdx.x == 0) *sigma_out = s_sigma;
        }
    } else if (warp == 1 && lane < 16) {
        projective_part(lane, pose, L, P, M);
    }
    __syncthreads();
    const float sigma = s_sigma;
    const float ifx = __frcp_rn(L.fx), ify = __frcp_rn(L.fy);
    float acc[32];  // 27 terms and the count; 4 unused
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k] = 0.f;
    const unsigned kept = find_pairs<kPix>(L, P, idx, j, r, z, gx, gy);
#pragma unroll
    for (int k = 0; k < kPix; ++k) {
        if (!((kept >> k) & 1u)) continue;
        float row[7];
        pair_row(L, M, idx[k] % L.W, idx[k] / L.W, z[k], gx[k], gy[k], r[k], sigma, ifx, ify, row);
        int t = 0;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int b = a; b < 7; ++b) {
                acc[t] = __fmaf_rn(row[a], row[b], acc[t]);
                ++t;
            }
        acc[27] += 1.f;
    }
    // warp totals (transpose butterfly: lane l holds term l), then the warps
    // in order: float sums in a fixed order
    red[warp][lane] = warp_transpose_reduce(acc, lane);
    __syncthreads();
    if (tid < 28) {
        float s = red[0][tid];
#pragma unroll
        for (int w = 1; w < NW; ++w) s = __fadd_rn(s, red[w][tid]);
        partials[(size_t)blockIdx.x * 28 + tid] = s;
    }
    if (!SOLVE) return;
    __shared__ bool s_last;
    __threadfence();  // this block's partials visible before its ticket
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // the blocks' partials in float-float: warp w takes blocks w, w + NW, ...,
    // then the warp sums in order
    __shared__ ffl redf[NW][28];
    if (lane < 28) {
        ffl v{0.f, 0.f};
        for (int b = warp; b < (int)gridDim.x; b += NW) v = ffl_add_f(v, __ldcg(partials + (size_t)b * 28 + lane));
        redf[warp][lane] = v;
    }
    __syncthreads();
    if (warp != 0) return;
    if (lane == 0) *counter = 0u;
    __shared__ ffl Rs[9], ts[3];
    ffl term{0.f, 0.f};
    if (lane < 28) {
        term = redf[0][lane];
        for (int w = 1; w < NW; ++w) term = ffl_add(term, redf[w][lane]);
    }
    const double pv = lane < 12 ? pose[lane] : 0.0;
    if (lane < 9) Rs[lane] = ffl_from_double(pv);
    else if (lane < 12) ts[lane - 9] = ffl_from_double(pv);
    __syncwarp();
    const float count = __shfl_sync(0xffffffffu, term.hi, 27);  // an integer below 2^24: exact
    ffl o, xl;
    const bool ok = count >= (float)kIcpMinInliers && warp_solve_step(term, Rs, ts, lane, o, xl);
    if (lane < 12) pose[lane] = ok ? ffl_to_double(o) : pv;
    if (lane == 0) *status |= ok ? 2 : 1;
}

// The 28 sums of `nb` float partials in FP64: warp w takes blocks w, w + 8,
// ..., then the warp sums in order (the odometry solve's order).
__global__ void __launch_bounds__(256) sum_partials_kernel(const float *__restrict__ partials, int nb,
                                                           double *__restrict__ out) {
    __shared__ double part[8][28];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane < 28) {
        double s = 0.0;
        for (int b = warp; b < nb; b += 8) s += (double)partials[(size_t)b * 28 + lane];
        part[warp][lane] = s;
    }
    __syncthreads();
    if (threadIdx.x < 28) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += part[w][threadIdx.x];
        out[threadIdx.x] = s;
    }
}

struct Pose12 { double v[12]; };
__global__ void set_pose_kernel(const Pose12 p, double *__restrict__ pose, int *__restrict__ status,
                                unsigned *__restrict__ counter) {
    if (threadIdx.x < 12) pose[threadIdx.x] = p.v[threadIdx.x];
    if (threadIdx.x == 0 && status) *status = 0;
    if (threadIdx.x == 0 && counter) *counter = 0u;
}

// Fill_List: correspondence of listed previous-frame points (or every pixel).
struct Proj12 { float v[12]; };
__global__ void correspondences_kernel(const Level L, const Proj12 proj, const tde_point2i *__restrict__ points,
                                       uint32_t npoints, tde_point2i *__restrict__ cprev,
                                       tde_point2i *__restrict__ ccurr, float *__restrict__ diff,
                                       uint32_t *__restrict__ count, double *__restrict__ sum_r2) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    bool kept = false;
    float r = 0.f;
    if (id < npoints) {
        int u, v;
        if (points) {
            u = points[id].x;
            v = points[id].y;
        } else {
            u = (int)(id % (uint32_t)L.W);
            v = (int)(id / (uint32_t)L.W);
        }
        int j = 0;
        if (u >= 0 && v >= 0 && u < L.W && v < L.H)
            kept = find_pair(L, proj.v, u, v, __ldg(L.Dp + (size_t)v * L.W + u), j, r);
        cprev[id] = kept ? tde_point2i{u, v} : tde_point2i{0, 0};
        ccurr[id] = kept ? tde_point2i{j % L.W, j / L.W} : tde_point2i{0, 0};
        diff[id] = kept ? r : 100.f;
    }
    const unsigned m = __ballot_sync(0xffffffffu, kept);
    double r2 = kept ? (double)r * (double)r : 0.0;
    for (int o = 16; o > 0; o >>= 1) r2 += __shfl_down_sync(0xffffffffu, r2, o);
    if ((threadIdx.x & 31) == 0 && m) {
        atomicAdd(count, (uint32_t)__popc(m));
        atomicAdd(sum_r2, r2);  // sums of squared integers below 2^53: exact in any order
    }
}

// Launch with programmatic stream serialisation: the kernel may start while
// the previous one on the stream finishes; it waits (griddepcontrol.wait)
// before reading anything that one writes.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, cudaStream_t s, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kOdoThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

Level make_level(const uint8_t *ip, const float *dp, const uint8_t *ic, const float *dc, const int16_t *dx,
                 const int16_t *dy, const tde_intrinsics &in, float mdd, float maxd, float min_gradient) {
    Level L;
    L.Ip = ip; L.Dp = dp; L.Ic = ic; L.Dc = dc; L.dx = dx; L.dy = dy;
    L.W = in.cols; L.H = in.rows;
    L.fx = in.fx; L.fy = in.fy; L.cx = in.cx; L.cy = in.cy;
    L.mdd = mdd; L.maxd = maxd;
    const float g = min_gradient / kSobelScale;
    L.grad2 = g * g;
    L.ifx = 1.0 / (double)in.fx;
    L.ify = 1.0 / (double)in.fy;
    return L;
}

}  // namespace
}  // namespace tde

using namespace tde;

extern "C" {

int tde_rgbd_prepare(const uint16_t *depth_mm, const uint8_t *rgb, int cols, int rows, uint8_t *intensity,
                     float *depth_m, void *stream) {
    if (!depth_mm || !rgb || !intensity || !depth_m || cols <= 0 || rows <= 0)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_prepare: bad arguments");
    const int n = cols * rows;
    prepare_kernel<<<div_up(n, 256u), 256, 0, as_stream(stream)>>>(depth_mm, rgb, n, intensity, depth_m);
    return check_launch("rgbd_prepare");
}

int tde_rgbd_pyramid(const uint8_t *intensity, const float *depth_m, int cols, int rows, uint8_t *intensity_half,
                     float *depth_half, void *stream) {
    if (!intensity || !depth_m || !intensity_half || !depth_half || cols < 2 || rows < 2)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_pyramid: bad arguments");
    dim3 b(32, 8), g(div_up(cols >> 1, 32), div_up(rows >> 1, 8));
    pyramid_kernel<<<g, b, 0, as_stream(stream)>>>(intensity, depth_m, cols, rows, intensity_half, depth_half);
    return check_launch("rgbd_pyramid");
}

int tde_rgbd_derivatives(const uint8_t *intensity, int cols, int rows, int16_t *dx, int16_t *dy, void *stream) {
    if (!intensity || !dx || !dy || cols <= 0 || rows <= 0)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_derivatives: bad arguments");
    dim3 b(32, 8), g(div_up(cols, 32), div_up(rows, 8));
    sobel_kernel<<<g, b, 0, as_stream(stream)>>>(intensity, cols, rows, dx, dy);
    return check_launch("rgbd_derivatives");
}

size_t tde_rgbd_points_scratch_bytes(int cols, int rows) {
    if (cols <= 0 || rows <= 0) return 0;
    return ((size_t)rows * sizeof(uint32_t) + 255) & ~(size_t)255;
}

int tde_rgbd_points_of_interest(const int16_t *dx, const int16_t *dy, int cols, int rows, float scale, void *scratch,
                                size_t scratch_bytes, tde_point2i *points, uint32_t capacity, uint32_t *count_device,
                                void *stream) {
    if (!dx || !dy || !scratch || !count_device || cols <= 0 || rows <= 0 || (!points && capacity))
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_points_of_interest: bad arguments");
    if (scratch_bytes < tde_rgbd_points_scratch_bytes(cols, rows))
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_points_of_interest: scratch %zu < %zu bytes", scratch_bytes,
                         tde_rgbd_points_scratch_bytes(cols, rows));
    cudaStream_t s = as_stream(stream);
    uint32_t *counts = static_cast<uint32_t *>(scratch);
    points_count_kernel<<<rows, kThreads, 0, s>>>(dx, dy, cols, scale, counts);
    int st = check_launch("rgbd_points/count");
    if (st) return st;
    scan_counts_kernel<<<1, 1024, 0, s>>>(counts, rows, count_device);
    if ((st = check_launch("rgbd_points/scan"))) return st;
    points_scatter_kernel<<<rows, kThreads, 0, s>>>(dx, dy, cols, scale, counts, points, capacity);
    return check_launch("rgbd_points/scatter");
}

int tde_rgbd_projective(const double *pose12, const tde_intrinsics *intr, float *proj12) {
    if (!pose12 || !intr || !proj12) return set_error(TDE_ERR_INVALID_ARG, "rgbd_projective: null argument");
    // the device formula, on the host: FP64 with fused operations, then float
    const double fx = intr->fx, fy = intr->fy, cx = intr->cx, cy = intr->cy;
    const double *R = pose12, *t = pose12 + 9;
    double M[9];
    for (int j = 0; j < 3; ++j) {
        M[j] = std::fma(fx, R[j], cx * R[6 + j]);
        M[3 + j] = std::fma(fy, R[3 + j], cy * R[6 + j]);
        M[6 + j] = R[6 + j];
    }
    const double ifx = 1.0 / fx, ify = 1.0 / fy;
    for (int i = 0; i < 3; ++i) {
        const double a = M[3 * i] * ifx, b = M[3 * i + 1] * ify;
        proj12[3 * i] = (float)a;
        proj12[3 * i + 1] = (float)b;
        proj12[3 * i + 2] = (float)(M[3 * i + 2] - std::fma(a, cx, b * cy));
    }
    proj12[9] = (float)std::fma(fx, t[0], cx * t[2]);
    proj12[10] = (float)std::fma(fy, t[1], cy * t[2]);
    proj12[11] = (float)t[2];
    return TDE_OK;
}

int tde_rgbd_correspondences(const uint8_t *i_prev, const float *d_prev, const uint8_t *i_curr, const float *d_curr,
                             const int16_t *dx, const int16_t *dy, int cols, int rows, const tde_point2i *points,
                             uint32_t npoints, const float *proj12, float max_depth_diff, float max_depth,
                             float min_gradient, tde_point2i *corr_prev, tde_point2i *corr_curr, float *diff,
                             uint32_t *count_device, double *sum_r2_device, void *stream) {
    if (!i_prev || !d_prev || !i_curr || !d_curr || !dx != !dy || !proj12 || !corr_prev || !corr_curr || !diff ||
        !count_device || !sum_r2_device || cols <= 0 || rows <= 0)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_correspondences: bad arguments");
    if (!points) npoints = (uint32_t)(cols * rows);
    cudaStream_t s = as_stream(stream);
    TDE_CUDA(cudaMemsetAsync(count_device, 0, sizeof(uint32_t), s), "rgbd_correspondences");
    TDE_CUDA(cudaMemsetAsync(sum_r2_device, 0, sizeof(double), s), "rgbd_correspondences");
    if (npoints == 0) return TDE_OK;
    tde_intrinsics in = {0.f, 0.f, 0.f, 0.f, cols, rows};
    const Level L = make_level(i_prev, d_prev, i_curr, d_curr, dx, dy, in, max_depth_diff, max_depth, min_gradient);
    Proj12 P;
    for (int k = 0; k < 12; ++k) P.v[k] = proj12[k];
    correspondences_kernel<<<div_up(npoints, 256u), 256, 0, s>>>(L, P, points, npoints, corr_prev, corr_curr, diff,
                                                                 count_device, sum_r2_device);
    return check_launch("rgbd_correspondences");
}

size_t tde_rgbd_odometry_scratch_bytes(int cols, int rows) {
    if (cols <= 0 || rows <= 0) return 0;
    const size_t nb = odo_blocks(cols, rows);
    return ((nb * 2 + nb * 28 + 12 + 1) * sizeof(double) + 255) & ~(size_t)255;  // + pose, ticket
}

void tde_rgbd_default_params(tde_rgbd_params *p) {
    if (!p) return;
    p->levels = 4;
    const int it[4] = {7, 7, 7, 10};
    for (int l = 0; l < TDE_RGBD_MAX_LEVELS; ++l) {
        p->iters[l] = it[l];
        p->min_gradient[l] = 10.f;
    }
    p->max_depth_diff = 0.07f;
    p->max_depth = 35.f;
}

int tde_rgbd_lsm(const uint8_t *i_prev, const float *d_prev, const uint8_t *i_curr, const float *d_curr,
                 const int16_t *dx, const int16_t *dy, const tde_intrinsics *intr, const double *pose12,
                 float max_depth_diff, float max_depth, float min_gradient, void *scratch, size_t scratch_bytes,
                 double *sums_device, float *sigma_device, void *stream) {
    if (!i_prev || !d_prev || !i_curr || !d_curr || !dx || !dy || !intr || !pose12 || !scratch || !sums_device ||
        intr->cols <= 0 || intr->rows <= 0)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_lsm: bad arguments");
    if (scratch_bytes < tde_rgbd_odometry_scratch_bytes(intr->cols, intr->rows))
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_lsm: scratch %zu < %zu bytes", scratch_bytes,
                         tde_rgbd_odometry_scratch_bytes(intr->cols, intr->rows));
    cudaStream_t s = as_stream(stream);
    const unsigned nb = odo_blocks(intr->cols, intr->rows);
    unsigned long long *res = static_cast<unsigned long long *>(scratch);
    double *lsm = reinterpret_cast<double *>(res + 2 * nb), *pose = lsm + 28 * nb;
    Pose12 P;
    for (int k = 0; k < 12; ++k) P.v[k] = pose12[k];
    set_pose_kernel<<<1, 32, 0, s>>>(P, pose, nullptr, nullptr);
    const Level L = make_level(i_prev, d_prev, i_curr, d_curr, dx, dy, *intr, max_depth_diff, max_depth, min_gradient);
    float *lsm_partials = reinterpret_cast<float *>(lsm);  // 28 floats a block in the room of 28 doubles
    residual_kernel<<<nb, kOdoThreads, 0, s>>>(L, pose, res);
    lsm_kernel<false><<<nb, kOdoThreads, 0, s>>>(L, pose, res, (int)nb, lsm_partials, sigma_device, nullptr, nullptr);
    sum_partials_kernel<<<1, 256, 0, s>>>(lsm_partials, (int)nb, sums_device);
    return check_launch("rgbd_lsm");
}

int tde_rgbd_odometry(const tde_rgbd_frame *prev, const tde_rgbd_frame *curr, const tde_intrinsics *intr0,
                      const tde_rgbd_params *params, const double *init_pose12, double *pose12_device,
                      int *status_device, void *scratch, size_t scratch_bytes, void *stream) {
    if (!prev || !curr || !intr0 || !params || !pose12_device || !status_device || !scratch)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_odometry: null argument");
    const int levels = params->levels;
    if (levels < 1 || levels > TDE_RGBD_MAX_LEVELS || (intr0->cols >> (levels - 1)) < 4 ||
        (intr0->rows >> (levels - 1)) < 4)
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_odometry: %d levels for a %dx%d frame", levels, intr0->cols,
                         intr0->rows);
    for (int l = 0; l < levels; ++l) {
        if (!prev->intensity[l] || !prev->depth[l] || !curr->intensity[l] || !curr->depth[l] || !curr->dx[l] ||
            !curr->dy[l])
            return set_error(TDE_ERR_INVALID_ARG, "rgbd_odometry: level %d is missing a buffer", l);
        if (params->iters[l] < 0 || params->iters[l] > 100)
            return set_error(TDE_ERR_INVALID_ARG, "rgbd_odometry: iters[%d] = %d", l, params->iters[l]);
    }
    if (scratch_bytes < tde_rgbd_odometry_scratch_bytes(intr0->cols, intr0->rows))
        return set_error(TDE_ERR_INVALID_ARG, "rgbd_odometry: scratch %zu < %zu bytes", scratch_bytes,
                         tde_rgbd_odometry_scratch_bytes(intr0->cols, intr0->rows));
    cudaStream_t s = as_stream(stream);
    const unsigned nb0 = odo_blocks(intr0->cols, intr0->rows);
    unsigned long long *res = static_cast<unsigned long long *>(scratch);
    double *lsm = reinterpret_cast<double *>(res + 2 * nb0);
    unsigned *ticket = reinterpret_cast<unsigned *>(lsm + 28 * nb0 + 12);
    Pose12 P;
    const double ident[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    for (int k = 0; k < 12; ++k) P.v[k] = init_pose12 ? init_pose12[k] : ident[k];
    set_pose_kernel<<<1, 32, 0, s>>>(P, pose12_device, status_device, ticket);
    int st = check_launch("rgbd_odometry");
    if (st) return st;
    for (int l = levels - 1; l >= 0; --l) {
        const float div = (float)(1 << l);
        const tde_intrinsics in = {intr0->fx / div, intr0->fy / div, intr0->cx / div, intr0->cy / div,
                                   intr0->cols >> l, intr0->rows >> l};
        const Level L = make_level(prev->intensity[l], prev->depth[l], curr->intensity[l], curr->depth[l], curr->dx[l],
                                   curr->dy[l], in, params->max_depth_diff, params->max_depth,
                                   params->min_gradient[l]);
        const unsigned nb = odo_blocks(in.cols, in.rows);
        for (int it = 0; it < params->iters[l]; ++it) {
            TDE_CUDA(launch_pdl(residual_kernel, nb, s, L, (const double *)pose12_device, res), "rgbd_odometry");
            TDE_CUDA(launch_pdl(lsm_kernel<true>, nb, s, L, pose12_device, (const unsigned long long *)res, (int)nb,
                                reinterpret_cast<float *>(lsm), (float *)nullptr, ticket, status_device),
                     "rgbd_odometry");
        }
    }
    return TDE_OK;
}

}  // extern "C"
