/*
 * oracle_rgbd.c -- CPU restatement of dense RGB-D (photometric) odometry.
 * TEST INFRASTRUCTURE ONLY: the checker of 3deye_gb300/csrc/k_rgbd.cu.
 *
 * The reference's RGB-D tracker (common/src/opencl_wrappers.cpp:1008-1466,
 * kernels GPU/opencl/scan_for_interest_point.cl, scan_list_of_valid_
 * correspondence.cl, compute_least_squares_equation.cl) follows the RGB-D
 * odometry of OpenCV's contrib rgbd module (odometry.cpp, named at
 * common/inc/common_defines.h:18; an un-vendored dependency under
 * $(MY_HOME)/3rdparty, Makefile.common:29-30, version not pinned), itself the
 * method of Steinbruecker, Sturm and Cremers, "Real-time visual odometry from
 * dense RGB-D images" (ICCV workshops 2011).  The reference copy does not
 * work as written (x and y both from get_global_id(0), unsigned 8-bit
 * derivatives, the depth test inverted, overlapping Indexes[id + k] writes,
 * the solvability test inverted, a read of uninitialised memory); this file
 * restates the published method with the reference's conventions:
 *
 *   intensity  8-bit grey (Intensity {uchar}, types/base_points.h:61-74),
 *              ITU-R BT.601 luma in 14-bit fixed point as OpenCV's RGB2GRAY;
 *   depth      metres, raw millimetres x 0.001, valid in (0, max_depth)
 *              (scan_list_of_valid_correspondence.cl:9-15: 35 m);
 *   pyramid    intrinsics::operator() (intrinsics.cpp:7-18); intensity 2x2
 *              mean rounded, depth the top-left sample of each 2x2 block;
 *   gradients  3x3 Sobel, SOBEL_SCALE 1/8 (compute_least_squares_equation.cl:8);
 *   pairs      a pixel (u, v) of the previous frame with depth z maps to
 *              p = z R' [u v 1]^T + t', R' = K R K^-1, t' = K t
 *              (Calculate_Supplementary_Isometry_Using_Camera_Matrix,
 *              opencl_wrappers.cpp:1176-1196), to pixel round(p.xy / p.z) of
 *              the current frame, kept when that pixel has depth within
 *              max_depth_diff of p.z (DEFAULT_DEPTH_THRESHOLD_RGBD 0.07 m) and
 *              a Sobel gradient of at least min_gradient / SOBEL_SCALE;
 *              residual r = I_curr(u', v') - I_prev(u, v);
 *   weights    sigma = sqrt(mean r^2); w = 1 / (sigma + |r|)
 *              (compute_least_squares_equation.cl:53-55);
 *   rows       C = w J for the left perturbation exp(xi) of the point
 *              P' = R P + t in the current camera (the kernel's v0, v1, v2
 *              and C[0..5], :72-80), and -w r: [A | b] += row row^T, the
 *              27-term layout of the ICP path;
 *   solve      FP64 6x6 solve and T <- exp(xi) T, coarse to fine, a fixed
 *              number of iterations per level.
 *
 * Float expressions are written with fmaf and correctly rounded reciprocals,
 * operation for operation as the GPU kernels (compiled without contraction),
 * so correspondences and weights agree bit for bit; the 27 sums agree to
 * accumulation order.  Pose T maps previous-frame camera coordinates to
 * current-frame ones: P_curr = R P_prev + t.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define RGBD_SOBEL_SCALE 0.125f

static int rint_i(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)nearbyintf(v);
}

int or_rgbd_prepare(const uint16_t *depth_mm, const uint8_t *rgb, int W, int H, uint8_t *I, float *D) {
    for (int i = 0; i < W * H; ++i) {
        const unsigned r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        I[i] = (uint8_t)((r * 4899u + g * 9617u + b * 1868u + 8192u) >> 14);
        D[i] = (float)depth_mm[i] * 0.001f;
    }
    return 0;
}

int or_rgbd_pyramid(const uint8_t *I, const float *D, int W, int H, uint8_t *I2, float *D2) {
    const int W2 = W >> 1, H2 = H >> 1;
    for (int y = 0; y < H2; ++y)
        for (int x = 0; x < W2; ++x) {
            const size_t s = (size_t)(2 * y) * W + 2 * x;
            I2[(size_t)y * W2 + x] = (uint8_t)((I[s] + I[s + 1] + I[s + W] + I[s + W + 1] + 2u) >> 2);
            D2[(size_t)y * W2 + x] = D[s];
        }
    return 0;
}

int or_rgbd_sobel(const uint8_t *I, int W, int H, int16_t *dx, int16_t *dy) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * W + x;
            if (x == 0 || y == 0 || x == W - 1 || y == H - 1) { dx[o] = 0; dy[o] = 0; continue; }
            const int a = I[o - W - 1], b = I[o - W], c = I[o - W + 1];
            const int d = I[o - 1], f = I[o + 1];
            const int g = I[o + W - 1], h = I[o + W], k = I[o + W + 1];
            dx[o] = (int16_t)((c + 2 * f + k) - (a + 2 * d + g));
            dy[o] = (int16_t)((g + 2 * h + k) - (a + 2 * b + c));
        }
    return 0;
}

/* Pixels whose Sobel gradient satisfies dx^2 + dy^2 >= scale, raster order
 * (Accumulate_Points_Of_Interest_For_RGBD, opencl_wrappers.cpp:1072-1119);
 * points[2 i], points[2 i + 1] = x, y.  Returns the count; writes at most
 * `capacity`. */
int or_rgbd_points(const int16_t *dx, const int16_t *dy, int W, int H, float scale, int *points, int capacity) {
    int n = 0;
    for (int i = 0; i < W * H; ++i) {
        const int g = dx[i] * dx[i] + dy[i] * dy[i];
        if ((float)g >= scale) {
            if (n < capacity) { points[2 * n] = i % W; points[2 * n + 1] = i / W; }
            ++n;
        }
    }
    return n;
}

/* R' = K R K^-1 and t' = K t in FP64 with fused operations (K^-1 through
 * the FP64 reciprocals of fx, fy), then to float: proj[0..8] = R' row-major,
 * proj[9..11] = t'. */
void or_rgbd_projective(const double *R, const double *t, const tde_intrinsics *in, float *proj) {
    const double fx = in->fx, fy = in->fy, cx = in->cx, cy = in->cy;
    double M[9];
    for (int j = 0; j < 3; ++j) {
        M[j] = fma(fx, R[j], cx * R[6 + j]);
        M[3 + j] = fma(fy, R[3 + j], cy * R[6 + j]);
        M[6 + j] = R[6 + j];
    }
    const double ifx = 1.0 / fx, ify = 1.0 / fy;
    for (int i = 0; i < 3; ++i) {
        const double a = M[3 * i] * ifx, b = M[3 * i + 1] * ify;
        proj[3 * i] = (float)a;
        proj[3 * i + 1] = (float)b;
        proj[3 * i + 2] = (float)(M[3 * i + 2] - fma(a, cx, b * cy));
    }
    proj[9] = (float)fma(fx, t[0], cx * t[2]);
    proj[10] = (float)fma(fy, t[1], cy * t[2]);
    proj[11] = (float)t[2];
}

typedef struct {
    const uint8_t *Ip, *Ic;
    const float *Dp, *Dc;
    const int16_t *dx, *dy;
    int W, H;
    float proj[12];  /* R', t' */
    float Rm[12];    /* R, t as float (the Jacobian's metric point) */
    float fx, fy, cx, cy, ifx, ify;
    float max_depth_diff, max_depth, grad2;
} rgbd_level_t;

static int depth_ok(float z, float max_depth) { return z > 0.f && z < max_depth; }

/* Correspondence of previous-frame pixel i: 1 and (j, r) when kept. */
static int rgbd_pair(const rgbd_level_t *L, int i, int *j_out, float *r_out) {
    const int u = i % L->W, v = i / L->W;
    const float z = L->Dp[i];
    if (!depth_ok(z, L->max_depth)) return 0;
    const float fu = (float)u, fv = (float)v;
    const float *P = L->proj;
    const float px = fmaf(z, fmaf(P[1], fv, fmaf(P[0], fu, P[2])), P[9]);
    const float py = fmaf(z, fmaf(P[4], fv, fmaf(P[3], fu, P[5])), P[10]);
    const float pz = fmaf(z, fmaf(P[7], fv, fmaf(P[6], fu, P[8])), P[11]);
    if (!(pz > 0.f)) return 0;
    const float iz = 1.f / pz;
    const int u2 = rint_i(px * iz), v2 = rint_i(py * iz);
    if (u2 < 0 || v2 < 0 || u2 >= L->W || v2 >= L->H) return 0;
    const int j = v2 * L->W + u2;
    const float z2 = L->Dc[j];
    if (!depth_ok(z2, L->max_depth) || !(fabsf(pz - z2) < L->max_depth_diff)) return 0;
    const int g = L->dx[j] * L->dx[j] + L->dy[j] * L->dy[j];
    if (!((float)g >= L->grad2)) return 0;
    *j_out = j;
    *r_out = (float)L->Ic[j] - (float)L->Ip[i];
    return 1;
}

/* The 7-vector (C0..C5, -w r) of a kept pair. */
static void rgbd_row(const rgbd_level_t *L, int i, int j, float r, float sigma, float row[7]) {
    const int u = i % L->W, v = i / L->W;
    const float z = L->Dp[i];
    const float xn = ((float)u - L->cx) * L->ifx, yn = ((float)v - L->cy) * L->ify;
    const float X = z * xn, Y = z * yn;
    const float *M = L->Rm;
    const float Px = fmaf(M[2], z, fmaf(M[1], Y, M[0] * X)) + M[9];
    const float Py = fmaf(M[5], z, fmaf(M[4], Y, M[3] * X)) + M[10];
    const float Pz = fmaf(M[8], z, fmaf(M[7], Y, M[6] * X)) + M[11];
    const float wsum = sigma + fabsf(r);
    const float w = wsum > 2.220446049250313e-16f ? 1.f / wsum : 1.f;
    const float s0 = w * RGBD_SOBEL_SCALE;
    const float iz = 1.f / Pz;
    const float v0 = iz * L->fx * s0 * (float)L->dx[j];
    const float v1 = iz * L->fy * s0 * (float)L->dy[j];
    const float v2 = -fmaf(v1, Py, v0 * Px) * iz;
    row[0] = fmaf(Py, v2, -(Pz * v1));
    row[1] = fmaf(Pz, v0, -(Px * v2));
    row[2] = fmaf(Px, v1, -(Py * v0));
    row[3] = v0;
    row[4] = v1;
    row[5] = v2;
    row[6] = -(w * r);
}

static void rgbd_setup(rgbd_level_t *L, const uint8_t *Ip, const float *Dp, const uint8_t *Ic, const float *Dc,
                       const int16_t *dx, const int16_t *dy, const tde_intrinsics *in, const double *R,
                       const double *t, float max_depth_diff, float max_depth, float min_gradient) {
    L->Ip = Ip; L->Dp = Dp; L->Ic = Ic; L->Dc = Dc; L->dx = dx; L->dy = dy;
    L->W = in->cols; L->H = in->rows;
    or_rgbd_projective(R, t, in, L->proj);
    for (int k = 0; k < 9; ++k) L->Rm[k] = (float)R[k];
    for (int k = 0; k < 3; ++k) L->Rm[9 + k] = (float)t[k];
    L->fx = in->fx; L->fy = in->fy; L->cx = in->cx; L->cy = in->cy;
    L->ifx = 1.f / in->fx; L->ify = 1.f / in->fy;
    L->max_depth_diff = max_depth_diff;
    L->max_depth = max_depth;
    const float g = min_gradient / RGBD_SOBEL_SCALE;
    L->grad2 = g * g;
}

/* One level's pairs for pose (R, t): kept[i] = 1 + j of the pair (0 when
 * none), resid[i] = r; returns the count and Sigma r^2 in *sum_r2. */
int or_rgbd_pairs(const uint8_t *Ip, const float *Dp, const uint8_t *Ic, const float *Dc, const int16_t *dx,
                  const int16_t *dy, const tde_intrinsics *in, const double *R, const double *t, float max_depth_diff,
                  float max_depth, float min_gradient, int *kept, float *resid, double *sum_r2) {
    rgbd_level_t L;
    rgbd_setup(&L, Ip, Dp, Ic, Dc, dx, dy, in, R, t, max_depth_diff, max_depth, min_gradient);
    int n = 0;
    double s = 0.0;  /* sums of squared integers: exact in any order */
#pragma omp parallel for schedule(static) reduction(+ : n, s)
    for (int i = 0; i < L.W * L.H; ++i) {
        int j = -1;
        float r = 0.f;
        const int ok = rgbd_pair(&L, i, &j, &r);
        if (kept) kept[i] = ok ? j + 1 : 0;
        if (resid) resid[i] = ok ? r : 0.f;
        if (ok) { ++n; s += (double)r * (double)r; }
    }
    if (sum_r2) *sum_r2 = s;
    return n;
}

static float rgbd_sigma(int n, double s) { return n > 0 ? sqrtf((float)(s / (double)n)) : 0.f; }

/* The 27 sums of [A | b] and the count (sums[27]) for pose (R, t). */
int or_rgbd_lsm(const uint8_t *Ip, const float *Dp, const uint8_t *Ic, const float *Dc, const int16_t *dx,
                const int16_t *dy, const tde_intrinsics *in, const double *R, const double *t, float max_depth_diff,
                float max_depth, float min_gradient, double *sums, float *sigma_out) {
    rgbd_level_t L;
    rgbd_setup(&L, Ip, Dp, Ic, Dc, dx, dy, in, R, t, max_depth_diff, max_depth, min_gradient);
    double s2 = 0.0;  /* sums of squared integers: exact in any order */
    int n = 0;
#pragma omp parallel for schedule(static) reduction(+ : n, s2)
    for (int i = 0; i < L.W * L.H; ++i) {
        int j;
        float r;
        if (rgbd_pair(&L, i, &j, &r)) { ++n; s2 += (double)r * (double)r; }
    }
    const float sigma = rgbd_sigma(n, s2);
    if (sigma_out) *sigma_out = sigma;
    /* per image row, then the rows in order: the same bits for any thread count */
    double *rs = (double *)calloc((size_t)L.H * 28, sizeof(double));
    if (!rs) return -1;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < L.H; ++v) {
        double *acc = rs + (size_t)v * 28;
        for (int i = v * L.W; i < (v + 1) * L.W; ++i) {
            int j;
            float r;
            if (!rgbd_pair(&L, i, &j, &r)) continue;
            float row[7];
            rgbd_row(&L, i, j, r, sigma, row);
            int s = 0;
            for (int a = 0; a < 6; ++a)
                for (int b = a; b < 7; ++b) acc[s++] += (double)row[a] * (double)row[b];
            acc[27] += 1.0;
        }
    }
    for (int k = 0; k < 28; ++k) sums[k] = 0.0;
    for (int v = 0; v < L.H; ++v)
        for (int k = 0; k < 28; ++k) sums[k] += rs[(size_t)v * 28 + k];
    free(rs);
    return n;
}

/* One correspondence's row for given inputs (the pin against the
 * reference kernel compute_least_squares_equation.cl): P' is formed from
 * (u, v, z) and the metric pose; dIdx, dIdy the Sobel derivatives at the
 * current pixel. */
int or_rgbd_row_single(int u, int v, float z, const float *Rt12, const tde_intrinsics *in, float dIdx, float dIdy,
                       float r, float sigma, float *row7) {
    const float ifx = 1.f / in->fx, ify = 1.f / in->fy;
    const float xn = ((float)u - in->cx) * ifx, yn = ((float)v - in->cy) * ify;
    const float X = z * xn, Y = z * yn;
    const float *M = Rt12;
    const float Px = fmaf(M[2], z, fmaf(M[1], Y, M[0] * X)) + M[9];
    const float Py = fmaf(M[5], z, fmaf(M[4], Y, M[3] * X)) + M[10];
    const float Pz = fmaf(M[8], z, fmaf(M[7], Y, M[6] * X)) + M[11];
    const float wsum = sigma + fabsf(r);
    const float w = wsum > 2.220446049250313e-16f ? 1.f / wsum : 1.f;
    const float s0 = w * RGBD_SOBEL_SCALE;
    const float iz = 1.f / Pz;
    const float v0 = iz * in->fx * s0 * dIdx;
    const float v1 = iz * in->fy * s0 * dIdy;
    const float v2 = -fmaf(v1, Py, v0 * Px) * iz;
    row7[0] = fmaf(Py, v2, -(Pz * v1));
    row7[1] = fmaf(Pz, v0, -(Px * v2));
    row7[2] = fmaf(Px, v1, -(Py * v0));
    row7[3] = v0;
    row7[4] = v1;
    row7[5] = v2;
    row7[6] = -(w * r);
    return 0;
}

/* The odometry: per level (coarsest first) iters[level] Gauss-Newton steps
 * T <- exp(xi) T.  I*, D*, dx, dy hold `levels` pointers each (level 0
 * finest; derivatives of the current frame).  pose12 (R row-major, t) is the
 * initial estimate on entry and the result on exit.  Returns the number of
 * failed solves (a failed solve keeps the pose). */
int or_rgbd_odometry(const uint8_t *const *Ip, const float *const *Dp, const uint8_t *const *Ic,
                     const float *const *Dc, const int16_t *const *dx, const int16_t *const *dy,
                     const tde_intrinsics *in0, int levels, const int *iters, float max_depth_diff, float max_depth,
                     const float *min_gradient, double *pose12) {
    int failed = 0;
    for (int l = levels - 1; l >= 0; --l) {
        const float div = (float)(1 << l);
        tde_intrinsics in = {in0->fx / div, in0->fy / div, in0->cx / div, in0->cy / div, in0->cols >> l,
                             in0->rows >> l};
        for (int it = 0; it < iters[l]; ++it) {
            double sums[28];
            const int n = or_rgbd_lsm(Ip[l], Dp[l], Ic[l], Dc[l], dx[l], dy[l], &in, pose12, pose12 + 9,
                                      max_depth_diff, max_depth, min_gradient[l], sums, NULL);
            if (n < 6 || or_icp_solve(sums, pose12, pose12 + 9, NULL) != 0) ++failed;
        }
    }
    return failed;
}

/* ---- synthetic colour: a procedural texture on the scene's surfaces ----
 * Triangle waves of the hit point (exact or correctly rounded operations
 * only), so the GPU sensor renders the same bytes. */
static double tri(double a) { return fabs(a - floor(a) - 0.5); }

void or_texture_rgb(const double *X, uint8_t *rgb) {
    const double a = tri(X[0] * 7.0 + X[1] * 3.0), b = tri(X[1] * 9.0 - X[2] * 5.0), c = tri(X[2] * 11.0 + X[0] * 4.0);
    const double d = tri((X[0] + X[1] + X[2]) * 23.0);
    rgb[0] = (uint8_t)(40.0 + 400.0 * a * 0.5 + 200.0 * d * 0.5);
    rgb[1] = (uint8_t)(40.0 + 400.0 * b * 0.5 + 200.0 * d * 0.5);
    rgb[2] = (uint8_t)(40.0 + 400.0 * c * 0.5 + 200.0 * d * 0.5);
}
