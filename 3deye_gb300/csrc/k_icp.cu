// k_icp.cu -- projective point-to-plane ICP.
//
// One launch per ICP iteration: every thread associates a few pixels and
// accumulates the 27 upper-triangular terms of [J^T J | J^T r] (+ an inlier
// count); a warp transpose-reduction with TwoSum pairs and a block pass give
// each block's totals as float-float values; each block adds them, converted
// exactly to 126-bit fixed point, into integer accumulators with atomics --
// integer addition is associative, so the grid total is the same bits in any
// block order; the last block to finish reads the totals and, in the pipeline
// form, solves the 6x6 system to FP64 accuracy and updates the device pose.
//
// Built with -fmad=false so the per-pixel association and terms are the same
// IEEE float operations as the CPU oracle: inlier sets match exactly.
#include "tde_common.cuh"
#include "tde_icp.cuh"

namespace tde {
namespace {

constexpr int kThreads = 256;
constexpr int kPixPerThread = 4;
constexpr int kTailSlices = 9;  // 9 x 28 = 252 threads of the last block

struct f2 { float hi, lo; };

// Knuth TwoSum: hi + lo == a + b exactly.
__device__ __forceinline__ f2 two_sum(float a, float b) {
    float s = a + b;
    float bp = s - a;
    float ap = s - bp;
    float e = (a - ap) + (b - bp);
    return f2{s, e};
}
__device__ __forceinline__ f2 add_ff(f2 a, f2 b) {
    f2 s = two_sum(a.hi, b.hi);
    float lo = s.lo + (a.lo + b.lo);
    return two_sum(s.hi, lo);
}
__device__ __forceinline__ f2 add_f(f2 a, float b) {
    f2 s = two_sum(a.hi, b);
    s.lo = s.lo + a.lo;
    return two_sum(s.hi, s.lo);
}

__device__ __forceinline__ float3 mv(const float *M, float3 v) {
    float a = 0.f; a += M[0] * v.x; a += M[1] * v.y; a += M[2] * v.z;
    float b = 0.f; b += M[3] * v.x; b += M[4] * v.y; b += M[5] * v.z;
    float c = 0.f; c += M[6] * v.x; c += M[7] * v.y; c += M[8] * v.z;
    return make_float3(a, b, c);
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
    float d = 0.f; d += a.x * b.x; d += a.y * b.y; d += a.z * b.z; return d;
}
__device__ __forceinline__ float3 ld3(const float *p, size_t i) {
    return make_float3(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2));
}

// Per-pixel association, split in two so a thread can issue the loads of all
// its pixels before it needs any of them.
struct Assoc {
    float3 vg;    // current vertex, global frame
    float3 ng;    // current normal, global frame
    int j;        // model pixel, -1 when rejected
};

__device__ __forceinline__ Assoc project(const IcpArgs &a, const IcpPose &P, float3 n, float3 v) {
    Assoc r;
    r.j = -1;
    if (isnan(n.x)) return r;
    const float3 rv = mv(P.R_cur, v);
    r.vg = make_float3(rv.x + P.t_cur[0], rv.y + P.t_cur[1], rv.z + P.t_cur[2]);
    const float3 vcp = mv(P.R_prev_inv, make_float3(r.vg.x - P.t_prev[0], r.vg.y - P.t_prev[1], r.vg.z - P.t_prev[2]));
    if (!(vcp.z > 0.f)) return r;
    const int u = __float2int_rn(vcp.x * a.fx / vcp.z + a.cx);
    const int w = __float2int_rn(vcp.y * a.fy / vcp.z + a.cy);
    if (u < 0 || w < 0 || u >= a.W || w >= a.H) return r;
    r.ng = mv(P.R_cur, n);
    r.j = w * a.W + u;
    return r;
}

// Tests against the model point and writes the Jacobian row [vg x np, np]
// and residual np . (vp - vg); false when the pair is rejected.
__device__ __forceinline__ bool pair_terms(const IcpArgs &a, const Assoc &s, float3 np, float3 vp, float row[7]) {
    if (isnan(np.x)) return false;
    const float3 dv = make_float3(vp.x - s.vg.x, vp.y - s.vg.y, vp.z - s.vg.z);
    if (sqrtf(dot3(dv, dv)) > a.dist_thresh) return false;
    const float3 cr = cross3(s.ng, np);
    if (sqrtf(dot3(cr, cr)) >= a.angle_thresh) return false;
    const float3 c = cross3(s.vg, np);
    row[0] = c.x; row[1] = c.y; row[2] = c.z;
    row[3] = np.x; row[4] = np.y; row[5] = np.z;
    row[6] = dot3(np, dv);
    return true;
}

// ---------------------------------------------------------------------------
// FP64 solve and pose update, run by one warp of the last block.
//
// GB300 executes FP64 at a small fraction of the FP32 rate (a dependent DFMA
// takes ~64 cycles, a double reciprocal ~430, sqrt ~670, sincos ~1600), so the
// solve is arranged for latency: 3x3 blocks with adjugate inverses (two
// divisions, no square roots, short chains of 3-term dot products spread
// over lanes), and the SO(3) exponential from its Taylor series when the
// rotation step is small.
// ---------------------------------------------------------------------------
// A(theta) = sin(theta)/theta, B(theta) = (1 - cos(theta))/theta^2.
__device__ __forceinline__ void rodrigues_coeffs(double th2, double &A, double &B) {
    if (th2 < 1e-2) {  // theta < 0.1: truncation below 1e-17
        A = fma(th2, fma(th2, fma(th2, fma(th2, 1.0 / 362880.0, -1.0 / 5040.0), 1.0 / 120.0), -1.0 / 6.0), 1.0);
        B = fma(th2, fma(th2, fma(th2, fma(th2, 1.0 / 3628800.0, -1.0 / 40320.0), 1.0 / 720.0), -1.0 / 24.0), 0.5);
    } else {
        double th = sqrt(th2), sn, cs;
        sincos(th, &sn, &cs);
        A = sn / th;
        B = (1.0 - cs) / th2;
    }
}

// Term index of entry (r, c) of [A | b] in the 27-term upper-triangular
// order of opencl_wrappers.cpp:426-437 (row k holds columns k..6).
__device__ __forceinline__ int term_index(int r, int c) {
    const int k = r < c ? r : c, j = r < c ? c : r;  // A is symmetric
    return k * 7 - (k * (k - 1)) / 2 + (j - k);
}

// Cofactor (r, c) of a symmetric 3x3 matrix held row-major in M; the cyclic
// index form gives the sign.  adj(M) = cofactors (symmetric M).
__device__ __forceinline__ double cofactor3(const double *M, int r, int c) {
    const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    return fma(M[3 * r1 + c1], M[3 * r2 + c2], -M[3 * r1 + c2] * M[3 * r2 + c1]);
}

// FP64 solve of the 6x6 system by 3x3 blocks: with A = [[P, Q], [Q^T, R]],
// S = R - Q^T P^-1 Q, x2 = S^-1 (b2 - Q^T P^-1 b1), x1 = P^-1 b1 - P^-1 Q x2,
// each 3x3 inverse as adjugate / determinant.  Two reciprocals and chains of
// 3-term dot products keep the dependent FP64 latency short.  False when A is
// not positive definite (a pivot of P or S at or below 1e-30, tested through
// the leading minors).  Lanes 0..11 work; the result is in xo.
__device__ bool fp64_block_solve(const double *sums, int lane, double (&xo)[6]) {
    __shared__ double P[9], Q[9], R[9], b[6], CP[9], iP[9], T[9], S[9], CS[9], iS[9], u[3], w[3];
    __shared__ int ok;
    const int r = lane / 3, c = lane % 3;
    if (lane < 9) {
        P[lane] = sums[term_index(r, c)];
        Q[lane] = sums[term_index(r, 3 + c)];
        R[lane] = sums[term_index(3 + r, 3 + c)];
    } else if (lane < 15) {
        b[lane - 9] = sums[term_index(lane - 9, 6)];
    }
    if (lane == 0) ok = 1;
    __syncwarp();
    if (lane < 9) CP[lane] = cofactor3(P, r, c);
    __syncwarp();
    // det P through the first row; leading minors P00, P00 P11 - P01^2 (= CP[8]), det P
    const double detP = fma(P[0], CP[0], fma(P[1], CP[1], P[2] * CP[2]));
    if (lane == 0 && !(P[0] > 1e-30 && CP[8] > 1e-30 * P[0] && detP > 1e-30 * CP[8])) ok = 0;
    const double invP = 1.0 / detP;
    if (lane < 9) iP[lane] = CP[lane] * invP;
    __syncwarp();
    // T = Q^T P^-1 (3x3), w = P^-1 b1
    if (lane < 9) T[lane] = fma(Q[r], iP[c], fma(Q[3 + r], iP[3 + c], Q[6 + r] * iP[6 + c]));
    else if (lane < 12) {
        const int i = lane - 9;
        w[i] = fma(iP[3 * i], b[0], fma(iP[3 * i + 1], b[1], iP[3 * i + 2] * b[2]));
    }
    __syncwarp();
    // S = R - T Q, u = b2 - T b1
    if (lane < 9) S[lane] = R[lane] - fma(T[3 * r], Q[c], fma(T[3 * r + 1], Q[3 + c], T[3 * r + 2] * Q[6 + c]));
    else if (lane < 12) {
        const int i = lane - 9;
        u[i] = b[3 + i] - fma(T[3 * i], b[0], fma(T[3 * i + 1], b[1], T[3 * i + 2] * b[2]));
    }
    __syncwarp();
    if (lane < 9) CS[lane] = cofactor3(S, r, c);
    __syncwarp();
    const double detS = fma(S[0], CS[0], fma(S[1], CS[1], S[2] * CS[2]));
    if (lane == 0 && !(S[0] > 1e-30 && CS[8] > 1e-30 * S[0] && detS > 1e-30 * CS[8])) ok = 0;
    const double invS = 1.0 / detS;
    if (lane < 9) iS[lane] = CS[lane] * invS;
    __syncwarp();
    // x2 = S^-1 u; x1 = w - T^T x2
    if (lane < 3) xo[3 + lane] = fma(iS[3 * lane], u[0], fma(iS[3 * lane + 1], u[1], iS[3 * lane + 2] * u[2]));
    __syncwarp();
    if (lane < 3) xo[lane] = w[lane] - fma(T[lane], xo[3], fma(T[3 + lane], xo[4], T[6 + lane] * xo[5]));
    __syncwarp();
    return ok != 0;
}

// The pose a solve updates: FP64 estimate, its float mirror, the last step.
struct PoseRefs {
    double *R, *t;
    float *Rf, *tf;
    double *x;
};

// Solve and apply the update to the pose; false (pose unchanged) when A is
// not positive definite.
__device__ bool warp_solve_update(const PoseRefs &P, const double *sums, int lane) {
    __shared__ double Rinc[9];
    __shared__ double x[6];
    if (!fp64_block_solve(sums, lane, x)) return false;
    // Rinc = I + A [w]x + B (w w^T - th2 I), lanes 0..8 one entry each
    const double wx = x[0], wy = x[1], wz = x[2];
    const double th2 = fma(wx, wx, fma(wy, wy, wz * wz));
    double Ac, Bc;
    rodrigues_coeffs(th2, Ac, Bc);
    if (lane < 9) {
        const int r = lane / 3, c = lane % 3;
        const double w[3] = {wx, wy, wz};
        double e = Bc * w[r] * w[c];
        if (r == c) e += fma(-Bc, th2, 1.0);
        // skew part: [w]x = [[0,-wz,wy],[wz,0,-wx],[-wy,wx,0]]
        const double sk = (r == 0 && c == 1) ? -wz : (r == 0 && c == 2) ? wy : (r == 1 && c == 0) ? wz
                        : (r == 1 && c == 2) ? -wx : (r == 2 && c == 0) ? -wy : (r == 2 && c == 1) ? wx : 0.0;
        Rinc[lane] = fma(Ac, sk, e);
    }
    __syncwarp();
    // R <- Rinc R, t <- Rinc t + v (lanes 0..8 rotation, 9..11 translation)
    double out = 0.0;
    if (lane < 9) {
        const int r = lane / 3, c = lane % 3;
        out = fma(Rinc[3 * r], P.R[c], fma(Rinc[3 * r + 1], P.R[3 + c], Rinc[3 * r + 2] * P.R[6 + c]));
    } else if (lane < 12) {
        const int r = lane - 9;
        out = fma(Rinc[3 * r], P.t[0], fma(Rinc[3 * r + 1], P.t[1], fma(Rinc[3 * r + 2], P.t[2], x[3 + r])));
    }
    __syncwarp();
    if (lane < 9) { P.R[lane] = out; P.Rf[lane] = (float)out; }
    else if (lane < 12) { P.t[lane - 9] = out; P.tf[lane - 9] = (float)out; }
    if (lane < 6) P.x[lane] = x[lane];
    __syncwarp();
    return true;
}

__device__ bool warp_solve_and_update(IcpState *st, const double *sums, int lane) {
    const PoseRefs P{st->R, st->t, st->pose.R_cur, st->pose.t_cur, st->x};
    return warp_solve_update(P, sums, lane);
}

// ---------------------------------------------------------------------------
// Exact fixed point: value * 2^64 as a 128-bit integer.  A float is M * 2^(E-150)
// with a 24-bit M, so the product is M shifted by E - 86; bits below 2^-64
// are dropped (truncation toward zero), nothing else is rounded.
// ---------------------------------------------------------------------------
__device__ __forceinline__ __int128 to_fixed(float f) {
    const unsigned u = __float_as_uint(f);
    const int E = (int)((u >> 23) & 0xffu);
    if (E == 0 || E == 0xff) return 0;  // zero, subnormal (< 1.2e-38), or not finite
    const unsigned long long M = (unsigned long long)((u & 0x7fffffu) | 0x800000u);
    const int sh = E - 86;
    __int128 q;
    if (sh >= 0) q = sh > 100 ? ((__int128)1 << 124) : ((__int128)M << sh);  // saturate far beyond any sum
    else q = sh > -24 ? (__int128)(M >> -sh) : 0;
    return (u >> 31) ? -q : q;
}

// Sum of the three 42-bit limbs modulo 2^126, read as a signed value.
__device__ __forceinline__ double from_fixed(unsigned long long a0, unsigned long long a1, unsigned long long a2) {
    unsigned __int128 S = (unsigned __int128)a0 + ((unsigned __int128)a1 << 42) + ((unsigned __int128)a2 << 84);
    S &= ((unsigned __int128)1 << 126) - 1;
    __int128 v = (__int128)S;
    if ((S >> 125) & 1) v -= (__int128)1 << 126;
    const long long hi = (long long)(v >> 64);  // floor(v / 2^64)
    const unsigned long long lo = (unsigned long long)v;
    return (double)hi + (double)lo * 0x1p-64;
}

// Warp transpose-reduction: every lane holds 32 per-thread sums (28 used);
// five butterfly stages, each halving the values a lane keeps, leave lane l
// with the warp total of term l as a float-float pair (31 compensated adds
// and 62 shuffles instead of 32 x 5 of each).
__device__ __forceinline__ f2 warp_transpose_reduce(const float (&s)[32], int lane) {
    f2 v[16];
    {
        const bool up = lane & 16;
        #pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float send = up ? s[i] : s[i + 16];
            const float keep = up ? s[i + 16] : s[i];
            v[i] = two_sum(keep, __shfl_xor_sync(0xffffffffu, send, 16));
        }
    }
    #pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
        const bool up = lane & o;
        #pragma unroll
        for (int i = 0; i < o; ++i) {
            const f2 send = up ? v[i] : v[i + o];
            const f2 keep = up ? v[i + o] : v[i];
            const f2 recv{__shfl_xor_sync(0xffffffffu, send.hi, o), __shfl_xor_sync(0xffffffffu, send.lo, o)};
            v[i] = add_ff(keep, recv);
        }
    }
    return v[0];
}

template <bool SOLVE>
__global__ void __launch_bounds__(kThreads) icp_kernel(const IcpArgs a, IcpState *__restrict__ st,
                                                       float *__restrict__ gbuf, float *__restrict__ mbuf) {
    __shared__ IcpPose P;
    __shared__ f2 red[kThreads / 32][32];
    __shared__ unsigned ticket;
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    // Let the next ICP launch start: it only reads this launch's results
    // (pose, accumulators, counter) after its own griddepcontrol.wait.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    const int npix = a.W * a.H;
    const int base = blockIdx.x * kThreads * kPixPerThread + tid;
    // this thread's current-frame maps do not depend on the pose: load them
    // before waiting for the previous iteration
    float3 nc[kPixPerThread], vc[kPixPerThread];
    const float qnan = __int_as_float(0x7fffffff);
    #pragma unroll
    for (int k = 0; k < kPixPerThread; ++k) {
        const int p = base + k * kThreads;
        if (p < npix) { nc[k] = ld3(a.ncur, (size_t)p); vc[k] = ld3(a.vcur, (size_t)p); }
        else { nc[k] = make_float3(qnan, qnan, qnan); vc[k] = nc[k]; }
    }
    // wait for the previous launch in the stream (a no-op without a
    // programmatic dependency)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (tid < (int)(sizeof(IcpPose) / sizeof(float)))
        reinterpret_cast<float *>(&P)[tid] = reinterpret_cast<const float *>(&st->pose)[tid];
    __syncthreads();

    float s[32];
    #pragma unroll
    for (int t = 0; t < 32; ++t) s[t] = 0.f;
    Assoc as[kPixPerThread];
    #pragma unroll
    for (int k = 0; k < kPixPerThread; ++k) as[k] = project(a, P, nc[k], vc[k]);
    float3 np[kPixPerThread], vp[kPixPerThread];
    #pragma unroll
    for (int k = 0; k < kPixPerThread; ++k)
        if (as[k].j >= 0) { np[k] = ld3(a.nprev, (size_t)as[k].j); vp[k] = ld3(a.vprev, (size_t)as[k].j); }
    #pragma unroll
    for (int k = 0; k < kPixPerThread; ++k) {
        float row[7];
        if (as[k].j >= 0 && pair_terms(a, as[k], np[k], vp[k], row)) {
            int t = 0;
            #pragma unroll
            for (int i = 0; i < 6; ++i)
                #pragma unroll
                for (int j = i; j < 7; ++j) { s[t] = s[t] + row[i] * row[j]; ++t; }
            s[27] = s[27] + 1.f;
        }
    }
    const f2 wsum = warp_transpose_reduce(s, lane);
    red[warp][lane] = wsum;
    __syncthreads();
    if (tid < kIcpTerms) {
        f2 v = red[0][tid];
        #pragma unroll
        for (int w = 1; w < kThreads / 32; ++w) v = add_ff(v, red[w][tid]);
        const unsigned __int128 q = (unsigned __int128)(to_fixed(v.hi) + to_fixed(v.lo));
        const unsigned long long m42 = (1ull << 42) - 1ull;
        unsigned long long *acc = st->acc[blockIdx.x % kIcpAccCopies][tid];
        atomicAdd(acc + 0, (unsigned long long)q & m42);
        atomicAdd(acc + 1, (unsigned long long)(q >> 42) & m42);
        atomicAdd(acc + 2, (unsigned long long)(q >> 84) & m42);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) ticket = atomicAdd(&st->counter, 1u);
    __syncthreads();
    if (ticket != (unsigned)gridDim.x - 1) return;

    // ---- last block: read the exact integer totals, reset them, solve ----
    __shared__ double s_sums[kIcpTerms];
    __threadfence();
    if (tid < kIcpTerms) {
        unsigned long long a[kIcpAccCopies][3];
        #pragma unroll
        for (int c = 0; c < kIcpAccCopies; ++c)
            #pragma unroll
            for (int l = 0; l < 3; ++l) a[c][l] = __ldcg(&st->acc[c][tid][l]);
        unsigned long long a0 = 0, a1 = 0, a2 = 0;
        #pragma unroll
        for (int c = 0; c < kIcpAccCopies; ++c) {
            a0 += a[c][0]; a1 += a[c][1]; a2 += a[c][2];
            st->acc[c][tid][0] = 0ull; st->acc[c][tid][1] = 0ull; st->acc[c][tid][2] = 0ull;
        }
        const double d = from_fixed(a0, a1, a2);
        s_sums[tid] = d;
        if (mbuf && tid < 27) mbuf[tid] = (float)d;
    }
    __syncthreads();
    if (warp != 0) return;
    if (lane < kIcpTerms) st->sums[lane] = s_sums[lane];
    const int inliers = (int)s_sums[27];
    bool ok = true;
    if (SOLVE) ok = inliers >= kIcpMinInliers && warp_solve_and_update(st, s_sums, lane);
    if (lane == 0) {
        st->counter = 0u;
        st->inliers = inliers;
        if (SOLVE) {
            if (!ok) st->status |= kIcpStatusSolveFailed;
            st->iterations += 1;
        }
    }
}

// transform_estimation.cl:4-53: group g sums its row of the partial buffer.
__global__ void transform_estimation_kernel(const float *__restrict__ gbuf, float *__restrict__ out, int len,
                                            int stride) {
    __shared__ float s[256];
    const int tid = threadIdx.x;
    const size_t start = (size_t)blockIdx.x * stride;
    float sum = 0.f;
    for (int i = tid; i < len; i += 256) sum += gbuf[start + i];
    s[tid] = sum;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (tid < off) s[tid] = s[tid] + s[tid + off];
        __syncthreads();
    }
    if (tid == 0) out[blockIdx.x] = s[0];
}

__global__ void clean_buff_kernel(float *__restrict__ g, int width) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= width) return;
    for (int i = 0; i < 27; ++i) g[(size_t)i * width + id] = 0.f;
}

__global__ void icp_begin_frame_kernel(IcpState *st) {
    // the previous frame's pose becomes the association reference
    for (int k = 0; k < 9; ++k) st->pose.R_prev_inv[k] = (float)st->R[3 * (k % 3) + k / 3];
    for (int k = 0; k < 3; ++k) st->pose.t_prev[k] = (float)st->t[k];
    st->status = 0;
    st->iterations = 0;
}

}  // namespace

size_t icp_gbuf_floats(int W, int H) {
    // cross-block sums go through the state's integer accumulators
    (void)W;
    (void)H;
    return 64;
}

int launch_icp(const IcpArgs &a, IcpState *st, float *gbuf, float *mbuf, bool solve, bool overlap_previous,
               cudaStream_t stream) {
    const unsigned nb = div_up((unsigned)(a.W * a.H), (unsigned)(kThreads * kPixPerThread));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = overlap_previous ? 1 : 0;
    cudaError_t e = solve ? cudaLaunchKernelEx(&cfg, icp_kernel<true>, a, st, gbuf, mbuf)
                          : cudaLaunchKernelEx(&cfg, icp_kernel<false>, a, st, gbuf, mbuf);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "estimate_combined: %s", cudaGetErrorString(e));
    return check_launch("estimate_combined");
}

int launch_icp_begin_frame(IcpState *st, cudaStream_t stream) {
    icp_begin_frame_kernel<<<1, 1, 0, stream>>>(st);
    return check_launch("icp_begin_frame");
}

int launch_transform_estimation(const float *gbuf, float *out, int len, int stride, cudaStream_t stream) {
    transform_estimation_kernel<<<27, 256, 0, stream>>>(gbuf, out, len, stride);
    return check_launch("transform_estimation");
}

int launch_clean_buff(float *g, int width, cudaStream_t stream) {
    clean_buff_kernel<<<div_up(width, 256), 256, 0, stream>>>(g, width);
    return check_launch("clean_buff");
}

}  // namespace tde
