/*
 * oracle_scene.c -- CPU renderer of the seeded procedural scenes and the
 * Kinect-style depth noise model.  TEST INFRASTRUCTURE ONLY (synthetic
 * sensor for CPU tests and the CPU baseline; the GPU sensor in
 * 3deye_gb300/csrc/k_synth.cu uses the same scene encoding, counter-based
 * hash and noise model, operation for operation, and renders the same bits).
 *
 * Scene: nprim primitives of 8 doubles each, [type, a0..a6]:
 *   type 0  plane   n . p + d = 0          a = (nx, ny, nz, d)
 *   type 1  sphere  |p - c| = r            a = (cx, cy, cz, r)
 *   type 2  box     axis aligned           a = (xmin, ymin, zmin, xmax, ymax, zmax)
 * Pose: row-major R (camera -> world) then t (camera centre), 12 doubles.
 * Depth is the camera-frame z of the nearest hit (metres), 0 without a hit.
 */
#include "oracle.h"

#include <math.h>
#include <string.h>

static double hit_prim(const double *P, const double o[3], const double d[3]) {
    const double inf = 1e300;
    int type = (int)P[0];
    const double *a = P + 1;
    if (type == 0) {
        double den = a[0] * d[0] + a[1] * d[1] + a[2] * d[2];
        if (fabs(den) < 1e-12) return inf;
        double t = -(a[0] * o[0] + a[1] * o[1] + a[2] * o[2] + a[3]) / den;
        return t > 1e-9 ? t : inf;
    }
    if (type == 1) {
        double oc[3] = {o[0] - a[0], o[1] - a[1], o[2] - a[2]};
        double A = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double B = oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2];
        double C = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - a[3] * a[3];
        double disc = B * B - A * C;
        if (disc < 0) return inf;
        double s = sqrt(disc);
        double t0 = (-B - s) / A, t1 = (-B + s) / A;
        if (t0 > 1e-9) return t0;
        if (t1 > 1e-9) return t1;
        return inf;
    }
    if (type == 2) {
        double tmin = -inf, tmax = inf;
        for (int k = 0; k < 3; ++k) {
            if (fabs(d[k]) < 1e-15) {
                if (o[k] < a[k] || o[k] > a[3 + k]) return inf;
                continue;
            }
            double t1 = (a[k] - o[k]) / d[k], t2 = (a[3 + k] - o[k]) / d[k];
            if (t1 > t2) { double tt = t1; t1 = t2; t2 = tt; }
            if (t1 > tmin) tmin = t1;
            if (t2 < tmax) tmax = t2;
        }
        if (tmax < tmin) return inf;
        if (tmin > 1e-9) return tmin;
        if (tmax > 1e-9) return tmax;
        return inf;
    }
    return inf;
}

int or_render_depth(const double *scene, int nprim, const double *pose, const tde_intrinsics *in, float *depth) {
    const double *R = pose, *t = pose + 9;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < in->rows; ++v)
        for (int u = 0; u < in->cols; ++u) {
            double dc[3] = {((double)u - in->cx) / in->fx, ((double)v - in->cy) / in->fy, 1.0};
            double d[3] = {R[0] * dc[0] + R[1] * dc[1] + R[2] * dc[2], R[3] * dc[0] + R[4] * dc[1] + R[5] * dc[2],
                           R[6] * dc[0] + R[7] * dc[1] + R[8] * dc[2]};
            double best = 1e300;
            for (int p = 0; p < nprim; ++p) {
                double h = hit_prim(scene + 8 * p, t, d);
                if (h < best) best = h;
            }
            depth[(size_t)v * in->cols + u] = best < 1e299 ? (float)best : 0.f;
        }
    return 0;
}

/* Colour of the nearest hit of each pixel's ray: the procedural texture of
 * oracle_rgbd.c at the hit point, black without a hit (rgb: 3 bytes a pixel). */
void or_texture_rgb(const double *X, uint8_t *rgb);
int or_render_rgb(const double *scene, int nprim, const double *pose, const tde_intrinsics *in, uint8_t *rgb) {
    const double *R = pose, *t = pose + 9;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < in->rows; ++v)
        for (int u = 0; u < in->cols; ++u) {
            double dc[3] = {((double)u - in->cx) / in->fx, ((double)v - in->cy) / in->fy, 1.0};
            double d[3] = {R[0] * dc[0] + R[1] * dc[1] + R[2] * dc[2], R[3] * dc[0] + R[4] * dc[1] + R[5] * dc[2],
                           R[6] * dc[0] + R[7] * dc[1] + R[8] * dc[2]};
            double best = 1e300;
            for (int p = 0; p < nprim; ++p) {
                double h = hit_prim(scene + 8 * p, t, d);
                if (h < best) best = h;
            }
            uint8_t *o = rgb + 3 * ((size_t)v * in->cols + u);
            if (best < 1e299) {
                const double X[3] = {t[0] + best * d[0], t[1] + best * d[1], t[2] + best * d[2]};
                or_texture_rgb(X, o);
            } else {
                o[0] = o[1] = o[2] = 0;
            }
        }
    return 0;
}

/* 32-bit integer hash (lowbias32 constants by C. Wellons, public domain). */
static uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
static float u01(uint32_t h) { return ((float)(h >> 8) + 0.5f) * (1.0f / 16777216.0f); }

/* Standard normal deviate as the Irwin-Hall sum of 12 uniforms minus 6
 * (mean 0, variance 1, support [-6, 6]): twelve 16-bit uniforms u_k from six
 * hashes, U_k = (u_k + 1/2) / 2^16, g = (sum u_k + 6 - 6 * 2^16) / 2^16.  The
 * numerator is an integer below 2^19 and the scale a power of two, so g is
 * exact in float and the GPU sensor (k_synth.cu) produces the same bits. */
static float gauss12(uint32_t key) {
    static const uint32_t salt[6] = {0x02e5be93U, 0x967a889bU, 0x1b873593U, 0xcc9e2d51U, 0x85ebca6bU, 0xc2b2ae35U};
    int32_t sum = 0;
    for (int k = 0; k < 6; ++k) {
        uint32_t h = hash32(key ^ salt[k]);
        sum += (int32_t)(h & 0xFFFFu) + (int32_t)(h >> 16);
    }
    return (float)(sum + 6 - 6 * 65536) * (1.0f / 65536.0f);
}

/* Kinect noise: axial sigma = 0.0012 + 0.0019 (z - 0.4)^2 m (Nguyen et al.
 * 2012), 1 mm quantisation, `dropout` fraction of holes, invalid beyond
 * max_range.  Every operation is exact or correctly rounded, in the same
 * order as the GPU sensor (compiled without contraction there and here). */
int or_apply_noise(const float *depth_m, uint16_t *depth_mm, int W, int H, uint32_t seed, uint32_t frame,
                   float max_range, float dropout) {
    for (int i = 0; i < W * H; ++i) {
        float z = depth_m[i];
        uint32_t key = hash32(seed ^ hash32(frame * 0x9e3779b9U ^ hash32((uint32_t)i)));
        float ud = u01(hash32(key ^ 0x68bc21ebU));
        uint16_t out = 0;
        if (z > 0.f && z <= max_range && ud >= dropout) {
            float g = gauss12(key);
            float s = 0.0012f + 0.0019f * (z - 0.4f) * (z - 0.4f);
            float zn = z + s * g;
            float mm = nearbyintf(zn * 1000.f);
            if (mm > 0.f && mm <= max_range * 1000.f && mm < 65535.f) out = (uint16_t)mm;
        }
        depth_mm[i] = out;
    }
    return 0;
}
