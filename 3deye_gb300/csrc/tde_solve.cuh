// tde_solve.cuh -- the FP64 6x6 solve and pose update shared by the ICP
// iterations (k_icp.cu) and the RGB-D odometry steps (k_rgbd.cu).
#pragma once
#include "tde_common.cuh"

namespace tde {
namespace {

// ---------------------------------------------------------------------------
// FP64 solve and pose update, run by one warp per block.
//
// GB300 executes FP64 at a small fraction of the FP32 rate: each FP64 warp
// instruction occupies a sub-partition's FP64 pipe for ~64 cycles, whether
// one lane or 32 are active and whether or not it depends on the previous one
// (measured).  The solve's time is therefore its count of FP64 instructions:
// lanes share every instruction (one matrix or vector entry each, operands
// chosen by lane), exchange values by shuffles, test positivity on exponent
// bits in the integer pipe, form both inverses from one reciprocal, and
// evaluate the SO(3) exponential's two series in one instruction stream.
// ---------------------------------------------------------------------------
// A(theta) = sin(theta)/theta, B(theta) = (1 - cos(theta))/theta^2, for all
// lanes of the warp: even lanes evaluate A's series, odd lanes B's, in the
// same instructions.
__device__ __forceinline__ void rodrigues_coeffs(double th2, int lane, double &A, double &B) {
    if (__double_as_longlong(th2) < __double_as_longlong(1e-2)) {  // theta < 0.1 (th2 >= 0): truncation below 1e-17
        const bool odd = lane & 1;
        const double c4 = odd ? 1.0 / 3628800.0 : 1.0 / 362880.0, c3 = odd ? -1.0 / 40320.0 : -1.0 / 5040.0;
        const double c2 = odd ? 1.0 / 720.0 : 1.0 / 120.0, c1 = odd ? -1.0 / 24.0 : -1.0 / 6.0, c0 = odd ? 0.5 : 1.0;
        const double v = fma(th2, fma(th2, fma(th2, fma(th2, c4, c3), c2), c1), c0);
        A = __shfl_sync(0xffffffffu, v, 0);
        B = __shfl_sync(0xffffffffu, v, 1);
    } else {
        double th = sqrt(th2), sn, cs;
        sincos(th, &sn, &cs);
        A = sn / th;
        B = (1.0 - cs) / th2;
    }
}

// Biased binary exponent (0 for +-0 and subnormals, 2047 for Inf / NaN).
__device__ __forceinline__ int dexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }
// x positive and finite, and x > 2^(e_ref - 1023 - 100) to within a factor of
// two: "clearly positive" against a reference exponent (integer pipe).
__device__ __forceinline__ bool clearly_pos(double x, int e_ref) {
    const long long bx = __double_as_longlong(x);
    return bx > 0 && dexp(x) < 2047 && dexp(x) > e_ref - 100;
}

// Term index of entry (r, c) of [A | b] in the 27-term upper-triangular
// order of opencl_wrappers.cpp:426-437 (row k holds columns k..6).
__host__ __device__ __forceinline__ int term_index(int r, int c) {
    const int k = r < c ? r : c, j = r < c ? c : r;  // A is symmetric
    return k * 7 - (k * (k - 1)) / 2 + (j - k);
}

// 1/d for a positive normal d: the hardware approximation (relative error
// below 2^-20, measured), then two Newton-Raphson steps x <- x + x (1 - d x),
// each squaring the relative error (measured on 2^20 inputs from 2^-200 to
// 2^199: equal to the IEEE quotient 1.0 / d for every one).
__device__ __forceinline__ double rcp_nr(double d) {
    double x;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(x) : "d"(d));
    #pragma unroll
    for (int k = 0; k < 2; ++k) x = fma(x, fma(-d, x, 1.0), x);
    return x;
}

__device__ __forceinline__ double shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double pick3(int i, double a, double b, double c) { return i == 0 ? a : (i == 1 ? b : c); }

// One Gauss-Newton step, executed by all 32 lanes of a warp.  Lane l < 28
// holds term l of [A | b] (27 terms, then the inlier count).  With
// A = [[P, Q], [Q^T, R]] and adjugates (no division until the end):
//   S' = det(P) R - Q^T adj(P) Q   (= det(P) S, S the Schur complement),
//   u' = det(P) b2 - Q^T adj(P) b1,
//   x2 = adj(S') u' / det(S'),   x1 = (adj(P) b1 - adj(P) Q x2) / det(P),
// so 1/det(P) is formed while S' is, off the dependent chain.  The pose
// (R_old, t_old: shared, FP64) moves by exp([x1]x), x2:
//   R <- R + A (w x R) + B (w (w . R) - th2 R)   column by column, and
//   t <- t + A (w x t) + B (w (w . t) - th2 t) + x2,   w = x1.
// Lane l < 9 returns entry l of the new R (row-major) in `out`, lanes 9..11
// entry l - 9 of the new t; lane l < 6 returns x[l] in `xl`.  False (out =
// the old entry) when A is not positive definite (a pivot of P or S at or
// below 1e-30, tested through the leading minors).
__device__ bool warp_solve_step(double term, const double *R_old, const double *t_old, int lane, double &out,
                                double &xl) {
    const bool vec = lane >= 9;                       // lanes 9..11: vector entries
    const int vi = (lane >= 9 && lane < 12) ? lane - 9 : 0;
    const int l9 = lane < 9 ? lane : 0;
    const int r = l9 / 3, c = l9 % 3;
    const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    // adj(P): cofactors (lane r, c), det(P) through the first row
    const double CP = fma(shfl(term, term_index(r1, c1)), shfl(term, term_index(r2, c2)),
                          -(shfl(term, term_index(r1, c2)) * shfl(term, term_index(r2, c1))));
    const double P0 = shfl(term, 0), P1 = shfl(term, 1), P2 = shfl(term, 2);
    const double detP = fma(P0, shfl(CP, 0), fma(P1, shfl(CP, 1), P2 * shfl(CP, 2)));
    const double CP8 = shfl(CP, 8);  // P00 P11 - P01^2
    // leading minors clearly positive: P00 > 2^-100, CP8 > 2^-100 P00, det P > 2^-100 CP8
    bool ok = clearly_pos(P0, 1023) && clearly_pos(CP8, dexp(P0)) && clearly_pos(detP, dexp(CP8));
    // T' = Q^T adj(P) (lane r, c: sum_k Q(k, r) adj(P)(k, c)); v = adj(P) b1 (lane 9 + i)
    const int col = vec ? vi : c;
    double TW = 0.0;
    {
        double a[3], g[3];
        #pragma unroll
        for (int k = 0; k < 3; ++k) {
            a[k] = shfl(term, vec ? term_index(k, 6) : term_index(k, 3 + r));
            g[k] = shfl(CP, 3 * k + col);
        }
        TW = fma(a[0], g[0], fma(a[1], g[1], a[2] * g[2]));
    }
    // S' = det(P) R - T' Q (lane r, c); u' = det(P) b2 - T' b1 (lane 9 + i)
    const int row = vec ? vi : r;
    double SU;
    {
        const double base = detP * shfl(term, vec ? term_index(3 + vi, 6) : term_index(3 + r, 3 + c));
        double t[3], y[3];
        #pragma unroll
        for (int k = 0; k < 3; ++k) {
            t[k] = shfl(TW, 3 * row + k);
            y[k] = shfl(term, vec ? term_index(k, 6) : term_index(k, 3 + c));
        }
        SU = fma(-t[0], y[0], fma(-t[1], y[1], fma(-t[2], y[2], base)));
    }
    // adj(S'), det(S'); the tests of S = S' / det(P) scaled accordingly
    const double CS = fma(shfl(SU, 3 * r1 + c1), shfl(SU, 3 * r2 + c2), -(shfl(SU, 3 * r1 + c2) * shfl(SU, 3 * r2 + c1)));
    const double S0 = shfl(SU, 0);
    const double detS = fma(S0, shfl(CS, 0), fma(shfl(SU, 1), shfl(CS, 1), shfl(SU, 2) * shfl(CS, 2)));
    const double CS8 = shfl(CS, 8);
    // the same tests on S = S' / det(P)
    const int eP = dexp(detP) - 1023;
    ok = ok && clearly_pos(S0, 1023 + eP) && clearly_pos(CS8, dexp(S0) + eP) && clearly_pos(detS, dexp(CS8) + eP);
    // both inverses from one reciprocal (of a finite product)
    const double dPS = detP * detS;
    ok = ok && dexp(dPS) < 2047;
    const double rPS = rcp_nr(dPS);
    const double rS = detP * rPS, rP = detS * rPS;
    // x2 = adj(S') u' / det(S') (lane 9 + i)
    const double X2 = fma(shfl(CS, 3 * vi), shfl(SU, 9), fma(shfl(CS, 3 * vi + 1), shfl(SU, 10), shfl(CS, 3 * vi + 2) * shfl(SU, 11))) * rS;
    // x1 = (v - T'^T x2) / det(P) (lane 9 + i)
    const double x20 = shfl(X2, 9), x21 = shfl(X2, 10), x22 = shfl(X2, 11);
    const double X1 = fma(-shfl(TW, vi), x20, fma(-shfl(TW, 3 + vi), x21, fma(-shfl(TW, 6 + vi), x22, TW))) * rP;
    const double wx = shfl(X1, 9), wy = shfl(X1, 10), wz = shfl(X1, 11);
    xl = lane < 3 ? pick3(lane, wx, wy, wz) : pick3(lane - 3, x20, x21, x22);
    // the pose update: this lane's column (of R, or t) and row
    const double th2 = fma(wx, wx, fma(wy, wy, wz * wz));
    double A, B;
    rodrigues_coeffs(th2, lane, A, B);
    const double k0 = vec ? t_old[0] : R_old[c], k1 = vec ? t_old[1] : R_old[3 + c], k2 = vec ? t_old[2] : R_old[6 + c];
    // (w x k)[row] = w[row+1] k[row+2] - w[row+2] k[row+1]
    const int ra = row == 2 ? 0 : row + 1, rb = row == 0 ? 2 : row - 1;
    const double cr = fma(pick3(ra, wx, wy, wz), pick3(rb, k0, k1, k2), -(pick3(rb, wx, wy, wz) * pick3(ra, k0, k1, k2)));
    const double dt = fma(wx, k0, fma(wy, k1, wz * k2));
    const double kr = pick3(row, k0, k1, k2);
    const double M = fma(pick3(row, wx, wy, wz), dt, -(th2 * kr));
    double o = fma(A, cr, fma(B, M, kr));
    if (vec) o += pick3(vi, x20, x21, x22);
    out = ok ? o : kr;
    return ok;
}

}  // namespace
}  // namespace tde
