// k_icp.cu -- projective point-to-plane ICP.
//
// One launch per ICP iteration: every thread associates a few pixels and
// accumulates the 27 upper-triangular terms of [J^T J | J^T r] (+ an inlier
// count); a warp transpose-reduction and a block pass give each block's
// totals in float, in a fixed order; each block adds them, converted exactly
// to 126-bit fixed point, into integer accumulators with atomics -- integer
// addition is associative, so the grid total is the same bits in any block
// order.
//
// Pipeline form: launch i's blocks, once the programmatic dependency on
// launch i - 1 has resolved (its atomics complete and visible), read its
// exact totals and solve the 6x6 system themselves (tde_solve.cuh) -- every
// block the same operations on the same bits, so the same pose -- instead of a last
// block of launch i - 1 solving after a grid-wide ticket.  That takes the
// ticket, its fence and one dependent read off every iteration; only the
// frame's last launch keeps the ticket, to solve its own totals.
//
// Built with -fmad=false so the per-pixel association and terms are the same
// IEEE float operations as the CPU oracle: inlier sets match exactly.
#include "tde_common.cuh"
#include "tde_icp.cuh"
#include "tde_integrate.cuh"
#include "tde_solve.cuh"

namespace tde {
namespace {

constexpr int kThreads = 256;                  // the one-shot sums
constexpr int kPixPerThread = 4;
constexpr int kPixCoarse = 4;                  // pixels a thread on the coarse levels
constexpr int kCoarseThreads = 256;            // threads a block on the coarse levels
constexpr int kPixWide = 4;                    // pixels a thread on large levels
constexpr int kWideThreads = 512;              // threads a block on large levels
constexpr int kPixWideMinPixels = 1 << 18;     // "large": 640x480, not 320x240

// The association's float operations, written as explicit fused
// multiply-adds (one rounding each, as C's fmaf in the CPU oracle); the unit
// is compiled without contraction, so nothing else fuses.
__device__ __forceinline__ float3 mv(const float *M, float3 v) {
    return make_float3(__fmaf_rn(M[2], v.z, __fmaf_rn(M[1], v.y, __fmul_rn(M[0], v.x))),
                       __fmaf_rn(M[5], v.z, __fmaf_rn(M[4], v.y, __fmul_rn(M[3], v.x))),
                       __fmaf_rn(M[8], v.z, __fmaf_rn(M[7], v.y, __fmul_rn(M[6], v.x))));
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
                       __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
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
    const float iz = __frcp_rn(vcp.z);
    const int u = __float2int_rn(__fmaf_rn(vcp.x, __fmul_rn(a.fx, iz), a.cx));
    const int w = __float2int_rn(__fmaf_rn(vcp.y, __fmul_rn(a.fy, iz), a.cy));
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
    if (dot3(dv, dv) > a.dist2) return false;
    const float3 cr = cross3(s.ng, np);
    if (dot3(cr, cr) >= a.angle2) return false;
    const float3 c = cross3(s.vg, np);
    row[0] = c.x; row[1] = c.y; row[2] = c.z;
    row[3] = np.x; row[4] = np.y; row[5] = np.z;
    row[6] = dot3(np, dv);
    return true;
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

// Sum of the three 42-bit limbs modulo 2^126, read as a signed value v:
// v * 2^-64 rounded to the nearest double (ties to even), built with integer
// operations only, and the integer part floor(v / 2^64) in *whole.
__device__ __forceinline__ double from_fixed(unsigned long long a0, unsigned long long a1, unsigned long long a2,
                                             long long *whole) {
    unsigned __int128 S = (unsigned __int128)a0 + ((unsigned __int128)a1 << 42) + ((unsigned __int128)a2 << 84);
    S &= ((unsigned __int128)1 << 126) - 1;
    const bool neg = (S >> 125) & 1;
    __int128 v = (__int128)S;
    if (neg) v -= (__int128)1 << 126;
    *whole = (long long)(v >> 64);
    const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;  // |v| < 2^125
    const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
    if ((mh | ml) == 0ull) return 0.0;
    const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);
    const unsigned __int128 norm = m << lz;                    // leading one at bit 127
    const unsigned long long top = (unsigned long long)(norm >> 64), rest = (unsigned long long)norm;
    unsigned long long mant = (top >> 11) & ((1ull << 52) - 1ull);  // the 52 bits after the leading one
    const bool round = (top >> 10) & 1ull, sticky = (top & 0x3ffull) != 0ull || rest != 0ull;
    unsigned long long bexp = (unsigned long long)(127 - lz - 64 + 1023);  // value = 2^(msb - 64) * 1.mant
    if (round && (sticky || (mant & 1ull))) {
        if (++mant == (1ull << 52)) { mant = 0ull; ++bexp; }
    }
    return __longlong_as_double((long long)(((unsigned long long)neg << 63) | (bexp << 52) | mant));
}

// The same sum as a float-float pair (hi = its leading 24 bits, lo = the next
// 32 rounded to a float, then renormalised; relative error below 2^-48),
// with integer operations and one integer-to-float conversion.
__device__ __forceinline__ ffl from_fixed_ff(unsigned long long a0, unsigned long long a1, unsigned long long a2,
                                             long long *whole) {
    unsigned __int128 S = (unsigned __int128)a0 + ((unsigned __int128)a1 << 42) + ((unsigned __int128)a2 << 84);
    S &= ((unsigned __int128)1 << 126) - 1;
    const bool neg = (S >> 125) & 1;
    __int128 v = (__int128)S;
    if (neg) v -= (__int128)1 << 126;
    *whole = (long long)(v >> 64);
    const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;  // |v| <= 2^125
    const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
    if ((mh | ml) == 0ull) return ffl{0.f, 0.f};
    const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);  // 2 .. 127
    const unsigned long long top = (unsigned long long)((m << lz) >> 64);   // leading one at bit 63
    // the leading one weighs 2^(63 - lz): biased exponent 190 - lz; bit 8 of
    // top weighs 2^(8 - lz): the power of two with biased exponent 135 - lz
    const float hi = __uint_as_float(((unsigned)(190 - lz) << 23) | (unsigned)((top >> 40) & 0x7fffffull));
    const float lo = __fmul_rn(__uint2float_rn((unsigned)(top >> 8)), __uint_as_float((unsigned)(135 - lz) << 23));
    const ffl r = ffl_fast_two_sum(hi, lo);  // lo < ulp(hi)
    return neg ? ffl_neg(r) : r;
}

// Association, the per-block sums, and their exact addition into
// accumulator buffer `acc` (copy blockIdx % kIcpAccCopies).
template <int PIX, int THREADS>
__device__ __forceinline__ void accumulate_block(const IcpArgs &a, const IcpPose &P, const float3 (&nc)[PIX],
                                                 const float3 (&vc)[PIX], float (*red)[32],
                                                 unsigned long long (*acc)[kIcpAccCopies][kIcpTerms][3]) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float s[32];
    #pragma unroll
    for (int t = 0; t < 32; ++t) s[t] = 0.f;
    Assoc as[PIX];
    #pragma unroll
    for (int k = 0; k < PIX; ++k) as[k] = project(a, P, nc[k], vc[k]);
    float3 np[PIX], vp[PIX];
    #pragma unroll
    for (int k = 0; k < PIX; ++k)
        if (as[k].j >= 0) { np[k] = ld3(a.nprev, (size_t)as[k].j); vp[k] = ld3(a.vprev, (size_t)as[k].j); }
    #pragma unroll
    for (int k = 0; k < PIX; ++k) {
        float row[7];
        if (as[k].j >= 0 && pair_terms(a, as[k], np[k], vp[k], row)) {
            int t = 0;
            #pragma unroll
            for (int i = 0; i < 6; ++i)
                #pragma unroll
                for (int j = i; j < 7; ++j) { s[t] = __fmaf_rn(row[i], row[j], s[t]); ++t; }
            s[27] = s[27] + 1.f;
        }
    }
    red[warp][lane] = warp_transpose_reduce(s, lane);
    __syncthreads();
    if (tid < kIcpTerms) {
        float v = red[0][tid];
        #pragma unroll
        for (int w = 1; w < THREADS / 32; ++w) v = __fadd_rn(v, red[w][tid]);
        const unsigned __int128 q = (unsigned __int128)to_fixed(v);
        const unsigned long long m42 = (1ull << 42) - 1ull;
        unsigned long long *dst = (*acc)[blockIdx.x % kIcpAccCopies][tid];
        atomicAdd(dst + 0, (unsigned long long)q & m42);
        atomicAdd(dst + 1, (unsigned long long)(q >> 42) & m42);
        atomicAdd(dst + 2, (unsigned long long)(q >> 84) & m42);
    }
}

// Exact total of term `term` in accumulator buffer `acc` (all copies), and
// its integer part in *whole (the inlier count for the last term).
__device__ __forceinline__ double read_total(const unsigned long long (*acc)[kIcpAccCopies][kIcpTerms][3], int term,
                                            long long *whole) {
    unsigned long long v[kIcpAccCopies][3];
    #pragma unroll
    for (int c = 0; c < kIcpAccCopies; ++c)
        #pragma unroll
        for (int l = 0; l < 3; ++l) v[c][l] = __ldcg(&(*acc)[c][term][l]);
    unsigned long long a0 = 0, a1 = 0, a2 = 0;
    #pragma unroll
    for (int c = 0; c < kIcpAccCopies; ++c) { a0 += v[c][0]; a1 += v[c][1]; a2 += v[c][2]; }
    return from_fixed(a0, a1, a2, whole);
}

// read_total as a float-float pair.
__device__ __forceinline__ ffl read_total_ff(const unsigned long long (*acc)[kIcpAccCopies][kIcpTerms][3], int term,
                                            long long *whole) {
    unsigned long long v[kIcpAccCopies][3];
    #pragma unroll
    for (int c = 0; c < kIcpAccCopies; ++c)
        #pragma unroll
        for (int l = 0; l < 3; ++l) v[c][l] = __ldcg(&(*acc)[c][term][l]);
    unsigned long long a0 = 0, a1 = 0, a2 = 0;
    #pragma unroll
    for (int c = 0; c < kIcpAccCopies; ++c) { a0 += v[c][0]; a1 += v[c][1]; a2 += v[c][2]; }
    return from_fixed_ff(a0, a1, a2, whole);
}

// Last block of a launch: true for exactly one block, after every block's
// atomics are complete.
__device__ __forceinline__ bool last_block(IcpState *st, unsigned *ticket) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) *ticket = atomicAdd(&st->counter, 1u);
    __syncthreads();
    if (*ticket != gridDim.x - 1) return false;
    __threadfence();
    return true;
}

// Loads this thread's current-frame maps (independent of the pose).
template <int PIX, int THREADS>
__device__ __forceinline__ void load_current(const IcpArgs &a, float3 (&nc)[PIX], float3 (&vc)[PIX]) {
    const int npix = a.W * a.H;
    const int base = blockIdx.x * THREADS * PIX + threadIdx.x;
    const float qnan = __int_as_float(0x7fffffff);
    #pragma unroll
    for (int k = 0; k < PIX; ++k) {
        const int p = base + k * THREADS;
        if (p < npix) { nc[k] = ld3(a.ncur, (size_t)p); vc[k] = ld3(a.vcur, (size_t)p); }
        else { nc[k] = make_float3(qnan, qnan, qnan); vc[k] = nc[k]; }
    }
}

// One-shot sums for the pose in st->pose (the Estimate_Combined drop-in):
// the last block writes the exact totals to st->sums / mbuf and resets the
// accumulators.
__global__ void __launch_bounds__(kThreads) icp_sums_kernel(const IcpArgs a, IcpState *__restrict__ st,
                                                            float *__restrict__ mbuf) {
    __shared__ IcpPose P;
    __shared__ float red[kThreads / 32][32];
    __shared__ unsigned ticket;
    const int tid = threadIdx.x;
    float3 nc[kPixPerThread], vc[kPixPerThread];
    load_current<kPixPerThread, kThreads>(a, nc, vc);
    if (tid < (int)(sizeof(IcpPose) / sizeof(float)))
        reinterpret_cast<float *>(&P)[tid] = reinterpret_cast<const float *>(&st->pose)[tid];
    __syncthreads();
    accumulate_block<kPixPerThread, kThreads>(a, P, nc, vc, red, &st->acc[0]);
    if (!last_block(st, &ticket)) return;
    if (tid < kIcpTerms) {
        long long whole;
        const double d = read_total(&st->acc[0], tid, &whole);
        #pragma unroll
        for (int c = 0; c < kIcpAccCopies; ++c)
            #pragma unroll
            for (int l = 0; l < 3; ++l) st->acc[0][c][tid][l] = 0ull;
        st->sums[tid] = d;
        if (tid < 27) mbuf[tid] = (float)d;
        if (tid == 27) st->inliers = (int)whole;
    }
    if (tid == 0) st->counter = 0u;
}

// Pipeline form, launch `iter` of the frame (see the file comment).
template <int PIX, int THREADS, bool LAST>
__global__ void __launch_bounds__(THREADS) icp_step_kernel(const IcpArgs a, IcpState *__restrict__ st, int iter,
                                                           const IcpPublish pub) {
    __shared__ IcpPose P;
    __shared__ float red[THREADS / 32][32];
    __shared__ ffl Rs[9], ts[3];  // this launch's pose (float-float)
    __shared__ unsigned ticket;
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    // Let the next launch start: it reads this launch's accumulators and
    // pose slot only after its own griddepcontrol.wait.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    float3 nc[PIX], vc[PIX];
    load_current<PIX, THREADS>(a, nc, vc);
    asm volatile("griddepcontrol.wait;" ::: "memory");

    // ---- the pose this launch associates with ----
    // Solver warp: 0, or 2 for every other wave of blocks, so that two blocks
    // resident on one SM (blocks b and b + SM count) solve on different
    // sub-partitions: each solve is one long dependent instruction stream,
    // and two of them on one scheduler interleave.  Warp 1 loads the frame's
    // start pose meanwhile.
    const int solver = ((blockIdx.x / a.sm_count) & 1) * 2;
    if (warp == solver) {
        // the previous pose and the previous launch's totals, loads in flight
        // together; launch 0 converts the frame's FP64 start pose instead
        ffl pv{0.f, 0.f}, term{0.f, 0.f};
        double pd = 0.0;
        long long whole = 0;
        if (iter == 0) {
            if (lane < 12) pd = __ldcg(lane < 9 ? st->R + lane : st->t + (lane - 9));
            pv = ffl_from_double(pd);
        } else {
            if (lane < 12) {
                const float2 q = __ldcg(&st->pose_it[(iter - 1) & 1][lane]);
                pv = ffl{q.x, q.y};
            }
            if (lane < kIcpTerms) term = read_total_ff(&st->acc[(iter - 1) % kIcpAccBuffers], lane, &whole);
        }
        if (lane < 9) Rs[lane] = pv;
        else if (lane < 12) ts[lane - 9] = pv;
        __syncwarp();
        bool ok = true;
        int inliers = 0;
        if (iter > 0) {
            inliers = __shfl_sync(0xffffffffu, (int)whole, 27);
            ffl o, xl;
            ok = warp_solve_step(term, Rs, ts, lane, o, xl) && inliers >= kIcpMinInliers;
            if (ok) pv = o;
            __syncwarp();
            if (lane < 9) Rs[lane] = pv;
            else if (lane < 12) ts[lane - 9] = pv;
        }
        if (lane < 9) P.R_cur[lane] = pv.hi;
        else if (lane < 12) P.t_cur[lane - 9] = pv.hi;
        if (iter == 0) {
            // the frame's start pose is the association reference: R^T, t
            if (lane < 9) P.R_prev_inv[3 * (lane % 3) + lane / 3] = pv.hi;
            else if (lane < 12) P.t_prev[lane - 9] = pv.hi;
        }
        if (blockIdx.x == 0) {
            // publish the pose for the next launch, and the bookkeeping of the solve
            if (lane < 12) st->pose_it[iter & 1][lane] = make_float2(pv.hi, pv.lo);
            if (iter == 0) {
                if (lane < 9) {
                    st->R_start[lane] = pd;
                    st->pose.R_prev_inv[3 * (lane % 3) + lane / 3] = pv.hi;
                } else if (lane < 12) {
                    st->t_start[lane - 9] = pd;
                    st->pose.t_prev[lane - 9] = pv.hi;
                }
                if (lane == 0) { st->status = 0; st->iterations = 0; }
            }
            if (iter > 0 && lane == 0) {
                // stores only: a read-modify-write here would put an L2
                // round trip before this block's association
                st->inliers = inliers;
                if (!ok) st->status |= kIcpStatusSolveFailed;
                st->iterations = iter;
            }
        }
    } else if (iter > 0 && warp == 1 && lane < 12) {
        // the frame's start pose (launch 0 wrote it)
        const int k = tid - 32;
        if (k < 9) P.R_prev_inv[k] = st->pose.R_prev_inv[k];
        else P.t_prev[k - 9] = st->pose.t_prev[k - 9];
    }
    if (blockIdx.x == 0) {
        // the buffer launch iter + 1 adds into; launch iter - 1 read its
        // previous contents, and it has completed (zeroing it from every
        // block, a few words each, measured slower: the stores of 150 blocks
        // meet on the same few lines)
        unsigned long long *z = &st->acc[(iter + 1) % kIcpAccBuffers][0][0][0];
        for (int i = tid; i < kIcpAccCopies * kIcpTerms * 3; i += THREADS) z[i] = 0ull;
    }
    __syncthreads();

    accumulate_block<PIX, THREADS>(a, P, nc, vc, red, &st->acc[iter % kIcpAccBuffers]);
    if (!LAST) return;

    // ---- the frame's last launch: its last block solves its own totals ----
    if (!last_block(st, &ticket)) return;
    ffl term{0.f, 0.f};
    long long whole = 0;
    if (warp == 0 && lane < kIcpTerms) term = read_total_ff(&st->acc[iter % kIcpAccBuffers], lane, &whole);
    __syncthreads();
    // every launch of the frame has read what it needed: clear all buffers
    // so that the next frame's first launch adds into zeros
    {
        unsigned long long *z = &st->acc[0][0][0][0];
        for (int i = tid; i < kIcpAccBuffers * kIcpAccCopies * kIcpTerms * 3; i += THREADS) z[i] = 0ull;
    }
    if (warp != 0) return;
    const int inliers = __shfl_sync(0xffffffffu, (int)whole, 27);
    ffl o, xl;
    const bool ok = warp_solve_step(term, Rs, ts, lane, o, xl) && inliers >= kIcpMinInliers;
    // accept the estimate (in FP64), or keep the start pose when any solve failed
    const bool lost = !ok || (*(volatile int *)&st->status & kIcpStatusSolveFailed);
    double nv = 0.0;
    if (lane < 9) nv = lost ? st->R_start[lane] : ffl_to_double(o);
    else if (lane < 12) nv = lost ? st->t_start[lane - 9] : ffl_to_double(o);
    if (lane < 9) {
        st->R[lane] = nv;
        st->pose.R_cur[lane] = (float)nv;
        pub.cam->R[lane] = (float)nv;
        pub.cam->R_inv[3 * (lane % 3) + lane / 3] = (float)nv;
        pub.pose12[lane] = nv;
    } else if (lane < 12) {
        st->t[lane - 9] = nv;
        st->pose.t_cur[lane - 9] = (float)nv;
        pub.cam->t[lane - 9] = (float)nv;
        pub.pose12[lane] = nv;
    }
    if (lane == 0) {
        st->counter = 0u;
        st->inliers = inliers;
        if (!ok) st->status |= kIcpStatusSolveFailed;
        st->iterations = iter + 1;
        pub.cam->tracking_ok = !lost;
        *pub.status = lost ? pub.lost_status : 0;
        *pub.inliers = inliers;
    }
}

// Solve-and-update steps for `n` systems, one warp each (the device solve
// on its own, for tests): sums[28 n] (27 terms + inlier count), pose[12 n]
// updated in place, x[6 n], ok[n].
__global__ void icp_solve_kernel(const double *__restrict__ sums, int n, double *__restrict__ pose,
                                 double *__restrict__ x, int *__restrict__ okv) {
    __shared__ ffl Rs[4][9], ts[4][3];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * 4 + warp;
    if (i >= n) return;  // whole warps leave together
    const ffl term = ffl_from_double(lane < kIcpTerms ? sums[(size_t)28 * i + lane] : 0.0);
    const double pv = lane < 12 ? pose[(size_t)12 * i + lane] : 0.0;
    if (lane < 9) Rs[warp][lane] = ffl_from_double(pv);
    else if (lane < 12) ts[warp][lane - 9] = ffl_from_double(pv);
    __syncwarp();
    ffl o, xl;
    const bool ok = warp_solve_step(term, Rs[warp], ts[warp], lane, o, xl);
    if (lane < 12) pose[(size_t)12 * i + lane] = ok ? ffl_to_double(o) : pv;
    if (ok && lane < 6) x[(size_t)6 * i + lane] = ffl_to_double(xl);
    if (lane == 0) okv[i] = ok;
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

}  // namespace

size_t icp_gbuf_floats(int W, int H) {
    // cross-block sums go through the state's integer accumulators
    (void)W;
    (void)H;
    return 64;
}

int launch_icp(const IcpArgs &a, IcpState *st, float *mbuf, cudaStream_t stream) {
    const unsigned nb = div_up((unsigned)(a.W * a.H), (unsigned)(kThreads * kPixPerThread));
    icp_sums_kernel<<<nb, kThreads, 0, stream>>>(a, st, mbuf);
    return check_launch("estimate_combined");
}

int launch_icp_step(const IcpArgs &a, IcpState *st, int iter, bool last, const IcpPublish &pub, cudaStream_t stream) {
    // Large levels take blocks of kWideThreads threads with kPixWide pixels
    // each: 150 blocks at 640x480, one per SM, which leaves room to the next
    // frame's preprocessing running beside.  Measured with 640x480 frames
    // (ICP per frame, frames/s overlapped): 256 threads x 4 pixels (300
    // blocks) 0.1531 ms, 3026; 256 x 8 0.1516 ms, 3043 (0.1489 ms, 3095 after
    // the float-float solve); 512 x 4 0.1452 ms, 3147 -- the same pixels per
    // SM with twice the warps to cover the gather and reduction latencies.
    // Eight pixels a thread on the coarse levels too gave 3094 frames/s but
    // 0.162 ms and a slower end-to-end line (3007 against 3053).  Coarse
    // levels with 256 x 4 against 512 x 2, 256 x 2 and 512 x 1 (later build,
    // ICP ms / frames/s / end-to-end frames/s): 0.1206 / 3364 / 3338,
    // 0.1198 / 3391 / 3330, 0.1165 / 3345 / 3320, 0.1181 / 3363 / 3309 --
    // a faster serial ICP with more blocks loses to the overlapped
    // preprocessing they crowd.  With a.narrow (the learned refiner running
    // beside the tracking) large levels take 256 x 4 too: such a block (24.6k
    // registers) fits on an SM beside one of the refiner's convolution blocks
    // (113.7 KB of shared memory, at most 32.5k registers), a 512 x 4 one
    // (47.6k) does not -- learned line 2553 against 2500 frames/s, while the
    // plain line prefers 512 x 4 (3381 against 3275).
    const bool wide = a.W * a.H >= kPixWideMinPixels && !a.narrow;
    const unsigned nb = div_up((unsigned)(a.W * a.H), wide ? (unsigned)(kWideThreads * kPixWide) : (unsigned)(kCoarseThreads * kPixCoarse));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(wide ? kWideThreads : kCoarseThreads);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (wide)
        e = last ? cudaLaunchKernelEx(&cfg, icp_step_kernel<kPixWide, kWideThreads, true>, a, st, iter, pub)
                 : cudaLaunchKernelEx(&cfg, icp_step_kernel<kPixWide, kWideThreads, false>, a, st, iter, pub);
    else
        e = last ? cudaLaunchKernelEx(&cfg, icp_step_kernel<kPixCoarse, kCoarseThreads, true>, a, st, iter, pub)
                 : cudaLaunchKernelEx(&cfg, icp_step_kernel<kPixCoarse, kCoarseThreads, false>, a, st, iter, pub);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "icp_step: %s", cudaGetErrorString(e));
    return check_launch("icp_step");
}

int launch_icp_solve(const double *sums, int n, double *pose, double *x, int *ok, cudaStream_t stream) {
    if (n <= 0) return TDE_OK;
    icp_solve_kernel<<<div_up(n, 4), 128, 0, stream>>>(sums, n, pose, x, ok);
    return check_launch("icp_solve");
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
