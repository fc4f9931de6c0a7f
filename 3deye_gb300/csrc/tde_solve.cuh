// tde_solve.cuh -- the 6x6 solve and pose update shared by the ICP
// iterations (k_icp.cu) and the RGB-D odometry steps (k_rgbd.cu), run by one
// warp in float-float arithmetic.
#pragma once
#include "tde_common.cuh"

namespace tde {
namespace {

// Term index of entry (r, c) of [A | b] in the 27-term upper-triangular
// order of opencl_wrappers.cpp:426-437 (row k holds columns k..6).
__host__ __device__ __forceinline__ int term_index(int r, int c) {
    const int k = r < c ? r : c, j = r < c ? c : r;  // A is symmetric
    return k * 7 - (k * (k - 1)) / 2 + (j - k);
}

// ---------------------------------------------------------------------------
// Float-float arithmetic on the FP32 pipe.
//
// GB300 executes FP64 at a small fraction of the FP32 rate: an FP64 warp
// instruction occupies a sub-partition's FP64 pipe for ~64 cycles and a
// dependent one waits longer still (measured), so a solve written in FP64 is
// a chain of slow steps.  Here a value is hi + lo in two floats with
// |lo| <= ulp(hi) / 2: 48 significant bits.  Products are split exactly with
// one fused multiply-add (Dekker's product, FMA form), high parts are added
// exactly with Knuth's TwoSum, and the low-order parts are added in float in
// a fixed order, as in the double-double algorithms of Hida, Li and Bailey
// (2001) with float parts: about 2^-46 relative precision (against 2^-53 for
// FP64), far below the rounding of the float association terms the solve
// takes.  The solve below uses it only where precision is made: the residual
// of iterative refinement and the pose update.
// ---------------------------------------------------------------------------
struct ffl {
    float hi, lo;
};

__device__ __forceinline__ ffl ffl_two_sum(float a, float b) {  // a + b exactly
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ffl{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ffl ffl_fast_two_sum(float a, float b) {  // exact when |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return ffl{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ffl ffl_neg(ffl a) { return ffl{-a.hi, -a.lo}; }
__device__ __forceinline__ ffl ffl_scale(ffl a, float pow2) { return ffl{__fmul_rn(a.hi, pow2), __fmul_rn(a.lo, pow2)}; }
__device__ __forceinline__ ffl ffl_mul(ffl a, ffl b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);  // p + e = a.hi b.hi exactly
    const float x = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
    return ffl_fast_two_sum(p, __fadd_rn(e, x));
}
__device__ __forceinline__ ffl ffl_add_f(ffl a, float b) {
    const ffl s = ffl_two_sum(a.hi, b);
    return ffl_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ ffl ffl_add(ffl a, ffl b) {
    const ffl s = ffl_two_sum(a.hi, b.hi), t = ffl_two_sum(a.lo, b.lo);
    const ffl u = ffl_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return ffl_fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}
// z + sum_{i < N} a_i b_i (z = 0 without Z): each product's high part with
// its exact rounding error, the high parts (and z's) added exactly in a
// pairwise TwoSum tree, every low-order part added in float in a fixed order.
template <int N, bool Z>
__device__ __forceinline__ ffl ffl_dot(const ffl (&a)[N], const ffl (&b)[N], ffl z) {
    constexpr int M = N + (Z ? 1 : 0);
    float h[M];
    float lo = Z ? z.lo : 0.f;
    #pragma unroll
    for (int i = 0; i < N; ++i) {
        h[i] = __fmul_rn(a[i].hi, b[i].hi);
        const float e = __fmaf_rn(a[i].hi, b[i].hi, -h[i]);
        const float x = __fmaf_rn(a[i].hi, b[i].lo, __fmul_rn(a[i].lo, b[i].hi));
        lo = __fadd_rn(lo, __fadd_rn(e, x));
    }
    if constexpr (Z) h[N] = z.hi;
    #pragma unroll
    for (int w = 1; w < M; w *= 2)
        #pragma unroll
        for (int i = 0; i + w < M; i += 2 * w) {
            const ffl s = ffl_two_sum(h[i], h[i + w]);
            h[i] = s.hi;
            lo = __fadd_rn(lo, s.lo);
        }
    return ffl_two_sum(h[0], lo);
}
// Conversions through the FP64 pipe: for values that enter or leave the
// solve once per frame, not for every step.
__device__ __forceinline__ ffl ffl_from_double(double d) {
    const float hi = __double2float_rn(d);
    return ffl{hi, __double2float_rn(d - (double)hi)};
}
__device__ __forceinline__ double ffl_to_double(ffl a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ ffl shfl(ffl v, int src) {
    return ffl{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}
__device__ __forceinline__ ffl pick3(int i, ffl a, ffl b, ffl c) { return i == 0 ? a : (i == 1 ? b : c); }

// Biased binary exponent of a float (0 for +-0 and subnormals, 255 for Inf /
// NaN), and "clearly positive" against a reference exponent, as for FP64.
__device__ __forceinline__ int fexp(float x) { return (int)((__float_as_uint(x) >> 23) & 0xffu); }
__device__ __forceinline__ bool clearly_pos_f(float x, int e_ref) {
    return __float_as_int(x) > 0 && fexp(x) < 255 && fexp(x) > e_ref - 100;
}
// 2^-floor(e / 2) for a positive normal d = m 2^e (so d scaled by its square
// lies in [1, 4)); 1 for anything else.
__device__ __forceinline__ float diag_scale(float d) {
    if (!(__float_as_int(d) > 0 && fexp(d) > 0 && fexp(d) < 255)) return 1.f;
    const int k = -((fexp(d) - 127) >> 1);
    return __uint_as_float((unsigned)(127 + k) << 23);
}

// Float-float constants of the series below: hi = the float nearest the
// coefficient, lo = the float nearest the rest (folded at compile time).
constexpr double kInv6 = -1.0 / 6.0, kInv24 = -1.0 / 24.0, kInv120 = 1.0 / 120.0, kInv720 = 1.0 / 720.0;
constexpr float kInv6h = (float)kInv6, kInv6l = (float)(kInv6 - (double)kInv6h);
constexpr float kInv24h = (float)kInv24, kInv24l = (float)(kInv24 - (double)kInv24h);
constexpr float kInv120h = (float)kInv120, kInv120l = (float)(kInv120 - (double)kInv120h);
constexpr float kInv720h = (float)kInv720, kInv720l = (float)(kInv720 - (double)kInv720h);

// A(theta) = sin(theta)/theta, B(theta) = (1 - cos(theta))/theta^2 for all
// lanes (even lanes evaluate A's series, odd lanes B's): below 0.1 rad the
// series to theta^8, in Estrin's form (c0 + c1 t) + t^2 (c2 + t (c3 + c4 t)),
// t = theta^2, the innermost part in float (it is below 1e-6 of the sum);
// above, sin and cos in FP64 (a step of over 0.1 rad is rare).
__device__ __forceinline__ void rodrigues_coeffs_ff(ffl th2, int lane, ffl &A, ffl &B) {
    if (th2.hi < 1e-2f) {
        const bool odd = lane & 1;
        const float c4 = odd ? 1.f / 3628800.f : 1.f / 362880.f, c3 = odd ? -1.f / 40320.f : -1.f / 5040.f;
        const ffl c2 = odd ? ffl{kInv720h, kInv720l} : ffl{kInv120h, kInv120l};
        const ffl c1 = odd ? ffl{kInv24h, kInv24l} : ffl{kInv6h, kInv6l};
        const ffl c0{odd ? 0.5f : 1.f, 0.f};
        const ffl tail{__fmaf_rn(th2.hi, c4, c3), 0.f};
        const ffl t2 = ffl_mul(th2, th2);
        const ffl lo_part = ffl_dot<1, true>({th2}, {c1}, c0);
        const ffl hi_part = ffl_dot<1, true>({th2}, {tail}, c2);
        const ffl v = ffl_dot<1, true>({t2}, {hi_part}, lo_part);
        A = shfl(v, 0);
        B = shfl(v, 1);
    } else {
        const double t2 = ffl_to_double(th2);
        double th = sqrt(t2), sn, cs;
        sincos(th, &sn, &cs);
        A = ffl_from_double(sn / th);
        B = ffl_from_double((1.0 - cs) / t2);
    }
}

// Warp transpose-reduction: every lane holds 32 per-thread sums (28 used);
// five butterfly stages, each halving the values a lane keeps, leave lane l
// with the warp total of term l (31 additions and 31 shuffles instead of
// 32 x 5 of each), in a fixed order: float sums like the reference's
// transform_estimation.cl.  Compensated (TwoSum) additions here measured
// 0.55-0.84 us of a 640x480 ICP iteration's 3.3 us association at 16 warps
// per SM (about 440 instructions a thread against 125), for sums already
// rounded per thread; the rounding they add averages to ~1e-8 of a frame's
// totals.  Used by the ICP association and the RGB-D least-squares pass.
__device__ __forceinline__ float warp_transpose_reduce(const float (&s)[32], int lane) {
    float v[16];
    {
        const bool up = lane & 16;
        #pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float send = up ? s[i] : s[i + 16];
            const float keep = up ? s[i + 16] : s[i];
            v[i] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, 16));
        }
    }
    #pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
        const bool up = lane & o;
        #pragma unroll
        for (int i = 0; i < o; ++i) {
            const float send = up ? v[i] : v[i + o];
            const float keep = up ? v[i + o] : v[i];
            v[i] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, o));
        }
    }
    return v[0];
}

// Refinement steps after the FP32 solve: one leaves a relative error of about
// (cond(DAD) 2^-24)^2 (2.5e-13 of max |x| on the device solve's test systems,
// in a float-float emulation), two reach the float-float precision (2.2e-14)
// and cost 0.2 us more per Gauss-Newton step (ICP at 640x480: 0.1361 against
// 0.1404 ms per frame).
constexpr int kSolveRefinements = 1;

// One Gauss-Newton step, executed by all 32 lanes of a warp: lanes share every
// instruction (one matrix or vector entry each, operands chosen by lane) and
// exchange values by shuffles.  Lane l < 27 holds term l of [A | b] (term 27,
// the inlier count, is not used).  [A | b] is first scaled by powers of two
// (D A D y = D b, x = D y; D = diag(2^k) with every diagonal entry of D A D in
// [1, 4): exact, and the adjugate products below stay far inside the float
// range).  The scaled system is factored and solved in FP32 -- with
// A = [[P, Q], [Q^T, R]] and adjugates, no division until the end:
//   S' = det(P) R - Q^T adj(P) Q   (= det(P) S, S the Schur complement),
//   u' = det(P) b2 - Q^T adj(P) b1,   U = adj(S') u',   W = (Q^T adj(P))^T U,
//   y2 = U / det(S'),   y1 = adj(P) b1 / det(P) - W / (det(P) det(S')),
// both inverses from one reciprocal of det(P) det(S') -- and then refined,
// y <- y + A^-1 (b - A y), the residual formed in float-float from the exact
// float-float sums and the correction solved with the FP32 factors
// (mixed-precision iterative refinement: each step multiplies the error by
// about cond(DAD) 2^-24).  The pose (R_old, t_old: shared memory) moves by
// exp([x1]x), x2 in float-float:
//   R <- R + A (w x R) + B (w (w . R) - th2 R)   column by column, and
//   t <- t + A (w x t) + B (w (w . t) - th2 t) + x2,   w = x1.
// Lane l < 9 returns entry l of the new R (row-major) in `out`, lanes 9..11
// entry l - 9 of the new t; lane l < 6 returns x[l] in `xl`.  False (out =
// the old entry) when A is not positive definite: a leading minor of the
// scaled P or S at or below 2^-100 of its reference (integer tests on the
// exponent bits), or a determinant product outside the normal float range.
__device__ bool warp_solve_step(ffl term, const ffl *R_old, const ffl *t_old, int lane, ffl &out, ffl &xl) {
    const unsigned full = 0xffffffffu;
    const bool vec = lane >= 9;                       // lanes 9..11: vector entries
    const int vi = (lane >= 9 && lane < 12) ? lane - 9 : 0;
    const int l9 = lane < 9 ? lane : 0;
    const int r = l9 / 3, c = l9 % 3;
    const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    // ---- the scaling: lane l < 27 holds entry (i, j), i <= j (j = 6: b_i) ----
    float sx1, sx2;  // the scales of unknowns vi and 3 + vi (lanes 9..11)
    {
        const int i = (lane >= 7) + (lane >= 13) + (lane >= 18) + (lane >= 22) + (lane >= 25);
        const int j = lane - term_index(i, i) + i;
        const int jd = j < 6 ? j : 0;
        const float si = diag_scale(__shfl_sync(full, term.hi, term_index(i, i)));
        const float sj = diag_scale(__shfl_sync(full, term.hi, term_index(jd, jd)));
        sx1 = diag_scale(__shfl_sync(full, term.hi, term_index(vi, vi)));
        sx2 = diag_scale(__shfl_sync(full, term.hi, term_index(3 + vi, 3 + vi)));
        if (lane < 27) term = ffl_scale(ffl_scale(term, si), j < 6 ? sj : 1.f);
    }
    const float th = term.hi;
    auto T = [&](int src) { return __shfl_sync(full, th, src); };
    // ---- FP32 factors and first solution ----
    // adj(P): cofactors (lane r, c), det(P) through the first row
    const float CP = __fmaf_rn(T(term_index(r1, c1)), T(term_index(r2, c2)),
                               -__fmul_rn(T(term_index(r1, c2)), T(term_index(r2, c1))));
    auto CPs = [&](int src) { return __shfl_sync(full, CP, src); };
    const float P0 = T(0);
    const float detP = __fmaf_rn(P0, CPs(0), __fmaf_rn(T(1), CPs(1), __fmul_rn(T(2), CPs(2))));
    const float CP8 = CPs(8);  // P00 P11 - P01^2
    bool ok = clearly_pos_f(P0, 127) && clearly_pos_f(CP8, fexp(P0)) && clearly_pos_f(detP, fexp(CP8));
    // the factors' entries a vector lane (9 + vi) needs for a right-hand side
    float cpv[3], twr[3], csr[3], twc[3];
    #pragma unroll
    for (int k = 0; k < 3; ++k) cpv[k] = CPs(3 * k + vi);
    // T' = Q^T adj(P) (lane r, c); v = adj(P) b1 (lane 9 + i)
    float TW;
    {
        const int col = vec ? vi : c;
        const float a0 = T(vec ? term_index(0, 6) : term_index(0, 3 + r));
        const float a1 = T(vec ? term_index(1, 6) : term_index(1, 3 + r));
        const float a2 = T(vec ? term_index(2, 6) : term_index(2, 3 + r));
        TW = __fmaf_rn(a0, CPs(col), __fmaf_rn(a1, CPs(3 + col), __fmul_rn(a2, CPs(6 + col))));
    }
    auto TWs = [&](int src) { return __shfl_sync(full, TW, src); };
    #pragma unroll
    for (int k = 0; k < 3; ++k) { twr[k] = TWs(3 * vi + k); twc[k] = TWs(3 * k + vi); }
    // S' = det(P) R - T' Q (lane r, c); u' = det(P) b2 - T' b1 (lane 9 + i)
    float SU;
    {
        const int row = vec ? vi : r;
        const float base = __fmul_rn(detP, T(vec ? term_index(3 + vi, 6) : term_index(3 + r, 3 + c)));
        SU = __fmaf_rn(-TWs(3 * row), T(vec ? term_index(0, 6) : term_index(0, 3 + c)),
                       __fmaf_rn(-TWs(3 * row + 1), T(vec ? term_index(1, 6) : term_index(1, 3 + c)),
                                 __fmaf_rn(-TWs(3 * row + 2), T(vec ? term_index(2, 6) : term_index(2, 3 + c)), base)));
    }
    auto SUs = [&](int src) { return __shfl_sync(full, SU, src); };
    // adj(S'), det(S'); U = adj(S') u' (lane 9 + i); the tests of S = S' / det(P)
    const float CS = __fmaf_rn(SUs(3 * r1 + c1), SUs(3 * r2 + c2), -__fmul_rn(SUs(3 * r1 + c2), SUs(3 * r2 + c1)));
    auto CSs = [&](int src) { return __shfl_sync(full, CS, src); };
    #pragma unroll
    for (int k = 0; k < 3; ++k) csr[k] = CSs(3 * vi + k);
    const float S0 = SUs(0);
    const float detS = __fmaf_rn(S0, CSs(0), __fmaf_rn(SUs(1), CSs(1), __fmul_rn(SUs(2), CSs(2))));
    const float CS8 = CSs(8);
    const int eP = fexp(detP) - 127;
    ok = ok && clearly_pos_f(S0, 127 + eP) && clearly_pos_f(CS8, fexp(S0) + eP) && clearly_pos_f(detS, fexp(CS8) + eP);
    // both inverses from one reciprocal (of a normal product), one Newton step
    const float dPS = __fmul_rn(detP, detS);
    ok = ok && fexp(dPS) > 0 && fexp(dPS) < 255;
    float rPS;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rPS) : "f"(dPS));
    rPS = __fmaf_rn(rPS, __fmaf_rn(-dPS, rPS, 1.f), rPS);
    const float rS = __fmul_rn(detP, rPS), rP = __fmul_rn(detS, rPS), rSP = __fmul_rn(rS, rP);
    // y for a right-hand side: v = adj(P) h1 and u' (lane 9 + i) in, y1 and
    // y2 (lane 9 + i) out
    auto back = [&](float v, float u, float &y1, float &y2) {
        const float u0 = __shfl_sync(full, u, 9), u1 = __shfl_sync(full, u, 10), u2 = __shfl_sync(full, u, 11);
        const float U = __fmaf_rn(csr[0], u0, __fmaf_rn(csr[1], u1, __fmul_rn(csr[2], u2)));
        const float U0 = __shfl_sync(full, U, 9), U1 = __shfl_sync(full, U, 10), U2 = __shfl_sync(full, U, 11);
        const float W = __fmaf_rn(twc[0], U0, __fmaf_rn(twc[1], U1, __fmul_rn(twc[2], U2)));
        y2 = __fmul_rn(U, rS);
        y1 = __fmaf_rn(-W, rSP, __fmul_rn(v, rP));
    };
    float y1f, y2f;
    back(TW, SU, y1f, y2f);
    ffl y1{y1f, 0.f}, y2{y2f, 0.f};
    // ---- refinement: residual b - A y in float-float (lane i < 6 takes row
    // i), correction from the FP32 factors ----
    {
        const int ri = lane < 6 ? lane : 0;
        ffl Arow[6];
        #pragma unroll
        for (int j = 0; j < 6; ++j) Arow[j] = ffl_neg(shfl(term, term_index(ri, j)));
        const ffl brow = shfl(term, term_index(ri, 6));
        #pragma unroll
        for (int step = 0; step < kSolveRefinements; ++step) {
            const ffl yv[6] = {shfl(y1, 9), shfl(y1, 10), shfl(y1, 11), shfl(y2, 9), shfl(y2, 10), shfl(y2, 11)};
            const float res = ffl_dot<6, true>(Arow, yv, brow).hi;
            const float h0 = __shfl_sync(full, res, 0), h1 = __shfl_sync(full, res, 1), h2 = __shfl_sync(full, res, 2);
            const float hb = __shfl_sync(full, res, 3 + vi);
            const float v = __fmaf_rn(cpv[0], h0, __fmaf_rn(cpv[1], h1, __fmul_rn(cpv[2], h2)));
            const float u = __fmaf_rn(-twr[0], h0, __fmaf_rn(-twr[1], h1, __fmaf_rn(-twr[2], h2, __fmul_rn(detP, hb))));
            float d1, d2;
            back(v, u, d1, d2);
            y1 = ffl_add_f(y1, d1);
            y2 = ffl_add_f(y2, d2);
        }
    }
    // x = D y (lane 9 + i)
    const ffl X1 = ffl_scale(y1, sx1), X2 = ffl_scale(y2, sx2);
    const ffl wx = shfl(X1, 9), wy = shfl(X1, 10), wz = shfl(X1, 11);
    const ffl x20 = shfl(X2, 9), x21 = shfl(X2, 10), x22 = shfl(X2, 11);
    xl = lane < 3 ? pick3(lane, wx, wy, wz) : pick3(lane - 3, x20, x21, x22);
    // the pose update: this lane's column (of R, or t) and row
    const int row = vec ? vi : r;
    const ffl th2 = ffl_dot<3, false>({wx, wy, wz}, {wx, wy, wz}, ffl{});
    const ffl k0 = vec ? t_old[0] : R_old[c], k1 = vec ? t_old[1] : R_old[3 + c], k2 = vec ? t_old[2] : R_old[6 + c];
    // (w x k)[row] = w[row+1] k[row+2] - w[row+2] k[row+1]
    const int ra = row == 2 ? 0 : row + 1, rb = row == 0 ? 2 : row - 1;
    const ffl cr = ffl_dot<2, false>({pick3(ra, wx, wy, wz), ffl_neg(pick3(rb, wx, wy, wz))},
                                     {pick3(rb, k0, k1, k2), pick3(ra, k0, k1, k2)}, ffl{});
    const ffl dt = ffl_dot<3, false>({wx, wy, wz}, {k0, k1, k2}, ffl{});
    const ffl kr = pick3(row, k0, k1, k2);
    const ffl M = ffl_dot<2, false>({pick3(row, wx, wy, wz), ffl_neg(th2)}, {dt, kr}, ffl{});
    const ffl base = vec ? ffl_add(kr, pick3(vi, x20, x21, x22)) : kr;
    ffl A, B;
    rodrigues_coeffs_ff(th2, lane, A, B);
    const ffl o = ffl_dot<2, true>({A, B}, {cr, M}, base);
    out = ok ? o : kr;
    return ok;
}

}  // namespace
}  // namespace tde
