/*
 * oracle.c -- CPU oracle of the KinectFusion per-frame pipeline.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Plain C, single-threaded per
 * pixel/column with OpenMP over rows/columns where results cannot depend on
 * the schedule.
 */
#include "oracle.h"

#include <limits.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define OR_QNAN (__builtin_nanf(""))
#define MAXDV 32767

int or_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

/* ---------------- conversions (CUDA cvt semantics: saturate, NaN -> 0) ---- */
static int sat_i32(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v < -2147483648.0f) return (int)0x80000000;
    return (int)v;
}
static int floor_sat(float v) { return sat_i32(floorf(v)); }
static int rint_sat(float v) { return sat_i32(nearbyintf(v)); }
static int trunc_sat(float v) { return sat_i32(truncf(v)); }
static float fmax_cl(float a, float b) { return a < b ? b : a; }
static float fmin_cl(float a, float b) { return b < a ? b : a; }
static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* IEEE binary16 round-to-nearest-even, written from the format definition. */
uint16_t or_float_to_half(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7fffu : 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax >= 0x38800000u) {
        uint32_t m = ax - 0x38000000u, r = m >> 13, rem = m & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
        return (uint16_t)(sign | r);
    }
    uint32_t E = ax >> 23;
    if (E < 102) return (uint16_t)sign;
    uint32_t mant = (ax & 0x7fffffu) | 0x800000u, shift = 126 - E;
    uint32_t r = mant >> shift, rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (r & 1u))) r++;
    return (uint16_t)(sign | r);
}

float or_half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu, x;
    float f;
    if (e == 0) {
        f = (float)m * 5.9604644775390625e-8f;
        memcpy(&x, &f, 4);
        x |= sign;
    } else if (e == 31) {
        x = sign | 0x7f800000u | (m << 13);
    } else {
        x = sign | ((e + 112u) << 23) | (m << 13);
    }
    memcpy(&f, &x, 4);
    return f;
}

/* ---------------- cyclic addressing: GPU/opencl/raycast.cl:29-47 --------- */
size_t or_voxel_address(int x, int y, int z, const tde_round_buffer *rb) {
    int px = (x + rb->origin_GRID.x) % rb->voxels_size.x;
    int py = (y + rb->origin_GRID.y) % rb->voxels_size.y;
    int pz = (z + rb->origin_GRID.z) % rb->voxels_size.z;
    size_t a = (size_t)(long)(rb->voxels_size.x * rb->voxels_size.y * pz + rb->voxels_size.x * py + px);
    a += (size_t)(long)rb->start_index;
    if (a > (size_t)(long)rb->buffer_length) a %= (size_t)(long)rb->buffer_length;
    return a;
}

/* ---------------- TSDF records ------------------------------------------- */
typedef struct { int fmt; size_t n; } vol_t;

static void rec_load(const void *vol, vol_t v, size_t i, float *f, int *w, uint32_t *raw) {
    if (v.fmt == TDE_TSDF_I16) {
        const tde_tsdf_i16 *p = (const tde_tsdf_i16 *)vol + i;
        *f = (float)p->value / (float)MAXDV;
        *w = p->weight;
        memcpy(raw, p, 4);
    } else if (v.fmt == TDE_TSDF_F16) {
        const uint16_t *p = (const uint16_t *)vol + 2 * i;
        *f = or_half_to_float(p[0]);
        *w = p[1];
        memcpy(raw, p, 4);
    } else {
        *f = ((const float *)vol)[i];
        *w = ((const uint16_t *)((const float *)vol + v.n))[i];
        memcpy(raw, f, 4);
    }
}
static float rec_value(const void *vol, vol_t v, size_t i) {
    float f; int w; uint32_t r;
    rec_load(vol, v, i, &f, &w, &r);
    return f;
}
/* set_tsdf: raycast.cl:18-27 for I16; returns 1 when the stored bits change */
static int rec_store(void *vol, vol_t v, size_t i, float f, int w) {
    if (v.fmt == TDE_TSDF_I16) {
        int q = trunc_sat(f * (float)MAXDV);
        q = imax(-MAXDV, imin(MAXDV, q));
        tde_tsdf_i16 *p = (tde_tsdf_i16 *)vol + i;
        int changed = p->value != (int16_t)q || p->weight != (int16_t)w;
        p->value = (int16_t)q;
        p->weight = (int16_t)w;
        return changed;
    } else if (v.fmt == TDE_TSDF_F16) {
        uint16_t *p = (uint16_t *)vol + 2 * i;
        uint16_t h = or_float_to_half(f);
        int changed = p[0] != h || p[1] != (uint16_t)w;
        p[0] = h;
        p[1] = (uint16_t)w;
        return changed;
    } else {
        float *pf = (float *)vol + i;
        uint16_t *pw = (uint16_t *)((float *)vol + v.n) + i;
        uint32_t a, b;
        memcpy(&a, pf, 4);
        memcpy(&b, &f, 4);
        int changed = a != b || *pw != (uint16_t)w;
        *pf = f;
        *pw = (uint16_t)w;
        return changed;
    }
}
static size_t vox_count(const tde_round_buffer *rb) {
    return (size_t)rb->voxels_size.x * rb->voxels_size.y * rb->voxels_size.z;
}

/* ---------------- raycast: GPU/opencl/raycast.cl:182-405 ----------------- */
typedef struct { float x, y, z; } v3;
static v3 mat_vec(const float *M, v3 v) {
    v3 r;
    float a = 0.f; a += M[0] * v.x; a += M[1] * v.y; a += M[2] * v.z; r.x = a;
    float b = 0.f; b += M[3] * v.x; b += M[4] * v.y; b += M[5] * v.z; r.y = b;
    float c = 0.f; c += M[6] * v.x; c += M[7] * v.y; c += M[8] * v.z; r.z = c;
    return r;
}
static v3 normalized(v3 v) {
    float d = 0.f; d += v.x * v.x; d += v.y * v.y; d += v.z * v.z;
    float rs = 1.f / sqrtf(d);
    v3 r = {v.x * rs, v.y * rs, v.z * rs};
    return r;
}
static v3 along(const float *o, v3 d, float t) {
    v3 r = {o[0] + d.x * t, o[1] + d.y * t, o[2] + d.z * t};
    return r;
}
typedef struct { const void *vol; vol_t v; const tde_round_buffer *rb; const float *cell; uint32_t *touched; } rc_ctx;
static float rc_read(const rc_ctx *c, int x, int y, int z) {
    const size_t a = or_voxel_address(x, y, z, c->rb);
    if (c->touched) __atomic_fetch_or(c->touched + (a >> 5), 1u << (a & 31), __ATOMIC_RELAXED);
    return rec_value(c->vol, c->v, a);
}
/* interpolateTrilineary: raycast.cl:95-145 */
static float rc_trilinear(const rc_ctx *c, v3 p) {
    const tde_point3i N = c->rb->voxels_size;
    const float *cs = c->cell;
    int gx = floor_sat(p.x / cs[0]), gy = floor_sat(p.y / cs[1]), gz = floor_sat(p.z / cs[2]);
    if (gx <= 0 || gx >= N.x - 1) return OR_QNAN;
    if (gy <= 0 || gy >= N.y - 1) return OR_QNAN;
    if (gz <= 0 || gz >= N.z - 1) return OR_QNAN;
    float vx = ((float)gx + 0.5f) * cs[0], vy = ((float)gy + 0.5f) * cs[1], vz = ((float)gz + 0.5f) * cs[2];
    gx = (p.x < vx) ? gx - 1 : gx;
    gy = (p.y < vy) ? gy - 1 : gy;
    gz = (p.z < vz) ? gz - 1 : gz;
    float a = p.x / cs[0] - ((float)gx + 0.5f); if (a < 0) { gx--; a += 1.0f; }
    float b = p.y / cs[1] - ((float)gy + 0.5f); if (b < 0) { gy--; b += 1.0f; }
    float cc = p.z / cs[2] - ((float)gz + 0.5f); if (cc < 0) { gz--; cc += 1.0f; }
    float r000 = rc_read(c, gx, gy, gz), r001 = rc_read(c, gx, gy, gz + 1);
    float r010 = rc_read(c, gx, gy + 1, gz), r011 = rc_read(c, gx, gy + 1, gz + 1);
    float r100 = rc_read(c, gx + 1, gy, gz), r101 = rc_read(c, gx + 1, gy, gz + 1);
    float r110 = rc_read(c, gx + 1, gy + 1, gz), r111 = rc_read(c, gx + 1, gy + 1, gz + 1);
    float oa = 1.f - a, ob = 1.f - b, oc = 1.f - cc;
    float x0 = ob * (r000 * oc + r001 * cc) + b * (r010 * oc + r011 * cc);
    float x1 = ob * (r100 * oc + r101 * cc) + b * (r110 * oc + r111 * cc);
    return oa * x0 + a * x1;
}

static int raycast_impl(const void *vol, int fmt, float *vmap, float *nmap, const float *t, const float *R, float trunc,
                        const tde_intrinsics *intr, const tde_round_buffer *rb, const float *cell, uint32_t *touched);

int or_raycast(const void *vol, int fmt, float *vmap, float *nmap, const float *t, const float *R, float trunc,
               const tde_intrinsics *intr, const tde_round_buffer *rb, const float *cell) {
    return raycast_impl(vol, fmt, vmap, nmap, t, R, trunc, intr, rb, cell, NULL);
}

/* The raycast of or_raycast, also marking every voxel record it reads in
 * `touched` (one bit per record); returns the number of distinct records. */
int64_t or_raycast_records(const void *vol, int fmt, float *vmap, float *nmap, const float *t, const float *R,
                           float trunc, const tde_intrinsics *intr, const tde_round_buffer *rb, const float *cell,
                           uint32_t *touched) {
    raycast_impl(vol, fmt, vmap, nmap, t, R, trunc, intr, rb, cell, touched);
    int64_t n = 0;
    const size_t words = (vox_count(rb) + 31) / 32;
    for (size_t i = 0; i < words; ++i) n += __builtin_popcount(touched[i]);
    return n;
}

static int raycast_impl(const void *vol, int fmt, float *vmap, float *nmap, const float *t, const float *R, float trunc,
                        const tde_intrinsics *intr, const tde_round_buffer *rb, const float *cell, uint32_t *touched) {
    rc_ctx c = {vol, {fmt, vox_count(rb)}, rb, cell, touched};
    const int W = intr->cols, H = intr->rows;
    const float step = (float)((double)trunc * 0.8);
    const tde_point3f V = rb->volume_size;
    const tde_point3i N = rb->voxels_size;
    const float max_time = 3.f * ((V.x + V.y) + V.z);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            size_t pix = (size_t)W * y + x;
            float out[6] = {OR_QNAN, OR_QNAN, OR_QNAN, OR_QNAN, OR_QNAN, OR_QNAN};
            v3 rnu = {((float)x - intr->cx) / intr->fx, ((float)y - intr->cy) / intr->fy, 1.f};
            v3 rn2 = mat_vec(R, rnu);
            v3 nxt = {rn2.x + t[0], rn2.y + t[1], rn2.z + t[2]};
            v3 fn = {nxt.x - t[0], nxt.y - t[1], nxt.z - t[2]};
            v3 d = normalized(fn);
            d.x = (d.x == 0.f) ? 1e-15f : d.x;
            d.y = (d.y == 0.f) ? 1e-15f : d.y;
            d.z = (d.z == 0.f) ? 1e-15f : d.z;
            float txmin = ((d.x > 0 ? 0.f : V.x) - t[0]) / d.x;
            float tymin = ((d.y > 0 ? 0.f : V.y) - t[1]) / d.y;
            float tzmin = ((d.z > 0 ? 0.f : V.z) - t[2]) / d.z;
            float ts = fmax_cl(fmax_cl(txmin, tymin), tzmin);
            float txmax = ((d.x > 0 ? V.x : 0.f) - t[0]) / d.x;
            float tymax = ((d.y > 0 ? V.y : 0.f) - t[1]) / d.y;
            float tzmax = ((d.z > 0 ? V.z : 0.f) - t[2]) / d.z;
            float te = fmin_cl(fmin_cl(txmax, tymax), tzmax);
            ts = fmax_cl(ts, 0.f);
            if (!(ts >= te)) {
                float tc = ts;
                v3 pu = along(t, d, tc);
                int gx = floor_sat(pu.x / cell[0]), gy = floor_sat(pu.y / cell[1]), gz = floor_sat(pu.z / cell[2]);
                gx = imax(0, imin(gx, N.x - 1));
                gy = imax(0, imin(gy, N.y - 1));
                gz = imax(0, imin(gz, N.z - 1));
                float tsdf = rc_read(&c, gx, gy, gz);
                for (; tc < max_time; tc += step) {
                    float prev = tsdf;
                    float ct = tc + step;
                    v3 q = along(t, d, ct);
                    int sx = floor_sat(q.x / cell[0]), sy = floor_sat(q.y / cell[1]), sz = floor_sat(q.z / cell[2]);
                    if (!(sx >= 0 && sy >= 0 && sz >= 0 && sx < N.x && sy < N.y && sz < N.z)) break;
                    tsdf = rc_read(&c, sx, sy, sz);
                    if (prev < 0.f && tsdf > 0.f) break;
                    if (prev > 0.f && tsdf < 0.f) {
                        float Ftdt = rc_trilinear(&c, along(t, d, ct));
                        if (isnan(Ftdt)) break;
                        float Ft = rc_trilinear(&c, along(t, d, tc));
                        if (isnan(Ft)) break;
                        float Ts = tc - step * Ft / (Ftdt - Ft);
                        v3 vf = along(t, d, Ts);
                        out[0] = vf.x; out[1] = vf.y; out[2] = vf.z;
                        v3 p3 = along(t, d, tc);
                        int hx = floor_sat(p3.x / cell[0]), hy = floor_sat(p3.y / cell[1]), hz = floor_sat(p3.z / cell[2]);
                        if (hx > 1 && hy > 1 && hz > 1 && hx < N.x - 2 && hy < N.y - 2 && hz < N.z - 2) {
                            v3 tt = vf; tt.x = tt.x + cell[0]; float Fx1 = rc_trilinear(&c, tt);
                            tt = vf; tt.x = tt.x - cell[0]; float Fx2 = rc_trilinear(&c, tt);
                            tt = vf; tt.y = tt.y + cell[1]; float Fy1 = rc_trilinear(&c, tt);
                            tt = vf; tt.y = tt.y - cell[1]; float Fy2 = rc_trilinear(&c, tt);
                            tt = vf; tt.z = tt.z + cell[2]; float Fz1 = rc_trilinear(&c, tt);
                            tt = vf; tt.z = tt.z - cell[2]; float Fz2 = rc_trilinear(&c, tt);
                            v3 nn = {Fx1 - Fx2, Fy1 - Fy2, Fz1 - Fz2};
                            v3 n = normalized(nn);
                            out[3] = n.x; out[4] = n.y; out[5] = n.z;
                        }
                        break;
                    }
                }
            }
            memcpy(vmap + 3 * pix, out, 12);
            memcpy(nmap + 3 * pix, out + 3, 12);
        }
    return 0;
}

/* ---------------- bilateral: compute_bilateral_filtering.cl:8-57 --------- */
int or_bilateral(const uint16_t *src, uint16_t *dst, int W, int H, float ss, float sc, uint32_t max_mm,
                 float *ratio_out) {
    const float inv_ss = 0.5f / (ss * ss), inv_sc = 0.5f / (sc * sc);
#pragma omp parallel for schedule(static)
    for (int row = 0; row < H; ++row)
        for (int col = 0; col < W; ++col) {
            int value = src[(size_t)row * W + col];
            int max_x = imin(col + 7, W - 1), max_y = imin(row + 7, H - 1);
            int min_x = imax(col - 6, 0), min_y = imax(row - 6, 0);
            float sum1 = 0.f, sum2 = 0.f;
            for (int cy = min_y; cy < max_y; ++cy)
                for (int cx = min_x; cx < max_x; ++cx) {
                    int tmp = src[(size_t)cy * W + cx];
                    int space2 = (col - cx) * (col - cx) + (row - cy) * (row - cy);
                    int color2 = (value - tmp) * (value - tmp);
                    float w = expf(-((float)space2 * inv_ss + (float)color2 * inv_sc));
                    sum1 = fmaf((float)tmp, w, sum1);
                    sum2 += w;
                }
            float ratio = sum1 / sum2;
            if (ratio_out) ratio_out[(size_t)row * W + col] = ratio;
            int res = imax(0, imin(rint_sat(ratio), MAXDV));
            if ((uint32_t)res > max_mm) res = 0;
            dst[(size_t)row * W + col] = (uint16_t)res;
        }
    return 0;
}

/* ---------------- depth pyramid (kernel absent; KinectFusion pyrDown) ---- */
int or_pyramid(const uint16_t *src, uint16_t *dst, int sW, int sH, float sigma_color) {
    const int dW = sW >> 1, dH = sH >> 1, th = (int)(3.f * sigma_color);
    for (int y = 0; y < dH; ++y)
        for (int x = 0; x < dW; ++x) {
            int center = src[(size_t)(2 * y) * sW + 2 * x], out = 0;
            if (center != 0) {
                int sum = 0, cnt = 0;
                for (int cy = imax(0, 2 * y - 2); cy < imin(sH, 2 * y + 3); ++cy)
                    for (int cx = imax(0, 2 * x - 2); cx < imin(sW, 2 * x + 3); ++cx) {
                        int v = src[(size_t)cy * sW + cx];
                        if (v != 0 && abs(v - center) < th) { sum += v; ++cnt; }
                    }
                out = (sum + cnt / 2) / cnt;
            }
            dst[(size_t)y * dW + x] = (uint16_t)out;
        }
    return 0;
}

/* ---------------- scale_depth (absent; opencl_wrappers.cpp:37-43) ------- */
int or_scale_depth(const uint16_t *depth, float *scaled, const tde_intrinsics *in) {
    for (int y = 0; y < in->rows; ++y)
        for (int x = 0; x < in->cols; ++x) {
            size_t o = (size_t)y * in->cols + x;
            float xl = ((float)x - in->cx) / in->fx, yl = ((float)y - in->cy) / in->fy;
            float lambda = sqrtf(xl * xl + yl * yl + 1.f);
            scaled[o] = (float)depth[o] * lambda / 1000.f;
        }
    return 0;
}

/* ---------------- vertex map (absent; opencl_wrappers.cpp:281-305) ------ */
int or_vertex_map(const uint16_t *depth, float *vmap, const tde_intrinsics *in) {
    for (int y = 0; y < in->rows; ++y)
        for (int x = 0; x < in->cols; ++x) {
            size_t o = (size_t)y * in->cols + x;
            int d = depth[o];
            float z = (float)d / 1000.f, vx = OR_QNAN, vy = OR_QNAN, vz = OR_QNAN;
            if (d != 0) { vx = z * (((float)x - in->cx) / in->fx); vy = z * (((float)y - in->cy) / in->fy); vz = z; }
            vmap[3 * o] = vx; vmap[3 * o + 1] = vy; vmap[3 * o + 2] = vz;
        }
    return 0;
}

/* ---------------- normal map: FP64 PCA with Jacobi eigenvectors --------- */
static void jacobi3(double A[3][3], double V[3][3], double ev[3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) V[i][j] = i == j;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        if (off < 1e-300) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (fabs(A[p][q]) < 1e-300) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(tt * tt + 1.0), s = tt * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; ++i) ev[i] = A[i][i];
}

int or_normal_map(const float *vmap, float *nmap, int W, int H) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            size_t o = 3 * ((size_t)y * W + x);
            float out[3] = {OR_QNAN, OR_QNAN, OR_QNAN};
            if (!isnan(vmap[o])) {
                double px = vmap[o], py = vmap[o + 1], pz = vmap[o + 2];
                double mx = 0, my = 0, mz = 0;
                int cnt = 0;
                for (int dy = -3; dy <= 3; ++dy)
                    for (int dx = -3; dx <= 3; ++dx) {
                        int xx = x + dx, yy = y + dy;
                        if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
                        size_t q = 3 * ((size_t)yy * W + xx);
                        if (isnan(vmap[q])) continue;
                        mx += vmap[q] - px; my += vmap[q + 1] - py; mz += vmap[q + 2] - pz;
                        ++cnt;
                    }
                if (cnt >= 24) {
                    mx /= cnt; my /= cnt; mz /= cnt;
                    double C[3][3] = {{0}};
                    for (int dy = -3; dy <= 3; ++dy)
                        for (int dx = -3; dx <= 3; ++dx) {
                            int xx = x + dx, yy = y + dy;
                            if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
                            size_t q = 3 * ((size_t)yy * W + xx);
                            if (isnan(vmap[q])) continue;
                            double u[3] = {vmap[q] - px - mx, vmap[q + 1] - py - my, vmap[q + 2] - pz - mz};
                            for (int i = 0; i < 3; ++i)
                                for (int j = 0; j < 3; ++j) C[i][j] += u[i] * u[j];
                        }
                    double V[3][3], ev[3];
                    jacobi3(C, V, ev);
                    int k = 0;
                    if (ev[1] < ev[k]) k = 1;
                    if (ev[2] < ev[k]) k = 2;
                    double n[3] = {V[0][k], V[1][k], V[2][k]};
                    double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                    if (nn > 0) {
                        for (int i = 0; i < 3; ++i) n[i] /= nn;
                        if (n[0] * px + n[1] * py + n[2] * pz > 0) for (int i = 0; i < 3; ++i) n[i] = -n[i];
                        out[0] = (float)n[0]; out[1] = (float)n[1]; out[2] = (float)n[2];
                    }
                }
            }
            memcpy(nmap + o, out, 12);
        }
    return 0;
}

/* ---------------- ICP association (estimate_combined absent;
 * opencl_wrappers.cpp:386-437 fixes the argument order and the 27-term
 * [A | b] layout) ----------------------------------------------------------
 * Float operations are written out with fused multiply-adds (fmaf: one
 * rounding, the same result as CUDA's __fmaf_rn), one correctly rounded
 * reciprocal per projection, and the distance and angle thresholds compared
 * on squares, so that the GPU association (k_icp.cu) performs exactly these
 * operations with fewer instructions and selects the same pairs. */
static v3 mat_vec_fma(const float *M, v3 v) {
    v3 r;
    r.x = fmaf(M[2], v.z, fmaf(M[1], v.y, M[0] * v.x));
    r.y = fmaf(M[5], v.z, fmaf(M[4], v.y, M[3] * v.x));
    r.z = fmaf(M[8], v.z, fmaf(M[7], v.y, M[6] * v.x));
    return r;
}
static float dot3_fma(v3 a, v3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
static v3 cross3_fma(v3 a, v3 b) {
    v3 r = {fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x))};
    return r;
}

int or_icp_terms(const float *vcur, const float *ncur, const float *vprev, const float *nprev, const float *P,
                 const tde_intrinsics *in, float dist_thresh, float angle_thresh, double *sums, uint8_t *mask) {
    const int W = in->cols, H = in->rows;
    const float *Rc = P, *tc = P + 9, *Rpi = P + 12, *tp = P + 21;
    const float dist2 = dist_thresh * dist_thresh, angle2 = angle_thresh * angle_thresh;
    for (int k = 0; k < 28; ++k) sums[k] = 0.0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            size_t i = (size_t)y * W + x;
            if (mask) mask[i] = 0;
            v3 n = {ncur[3 * i], ncur[3 * i + 1], ncur[3 * i + 2]};
            if (isnan(n.x)) continue;
            v3 v = {vcur[3 * i], vcur[3 * i + 1], vcur[3 * i + 2]};
            v3 rv = mat_vec_fma(Rc, v);
            v3 vg = {rv.x + tc[0], rv.y + tc[1], rv.z + tc[2]};
            v3 dd = {vg.x - tp[0], vg.y - tp[1], vg.z - tp[2]};
            v3 vcp = mat_vec_fma(Rpi, dd);
            if (!(vcp.z > 0.f)) continue;
            const float iz = 1.f / vcp.z;
            int u = rint_sat(fmaf(vcp.x, in->fx * iz, in->cx));
            int w = rint_sat(fmaf(vcp.y, in->fy * iz, in->cy));
            if (u < 0 || w < 0 || u >= W || w >= H) continue;
            size_t j = (size_t)w * W + u;
            v3 np = {nprev[3 * j], nprev[3 * j + 1], nprev[3 * j + 2]};
            if (isnan(np.x)) continue;
            v3 vp = {vprev[3 * j], vprev[3 * j + 1], vprev[3 * j + 2]};
            v3 dv = {vp.x - vg.x, vp.y - vg.y, vp.z - vg.z};
            if (dot3_fma(dv, dv) > dist2) continue;
            v3 ng = mat_vec_fma(Rc, n);
            v3 cr = cross3_fma(ng, np);
            if (dot3_fma(cr, cr) >= angle2) continue;
            v3 c = cross3_fma(vg, np);
            float row[7] = {c.x, c.y, c.z, np.x, np.y, np.z, dot3_fma(np, dv)};
            int s = 0;
            for (int a = 0; a < 6; ++a)
                for (int b = a; b < 7; ++b) sums[s++] += (double)row[a] * (double)row[b];
            sums[27] += 1.0;
            if (mask) mask[i] = 1;
        }
    return 0;
}

static void so3_exp_d(const double *x, double *R) {
    double wx = x[0], wy = x[1], wz = x[2], th2 = wx * wx + wy * wy + wz * wz, A, B;
    if (th2 < 1e-20) { A = 1.0 - th2 / 6.0; B = 0.5 - th2 / 24.0; }
    else { double th = sqrt(th2); A = sin(th) / th; B = (1.0 - cos(th)) / th2; }
    R[0] = 1.0 + B * (wx * wx - th2); R[1] = -A * wz + B * wx * wy; R[2] = A * wy + B * wx * wz;
    R[3] = A * wz + B * wx * wy; R[4] = 1.0 + B * (wy * wy - th2); R[5] = -A * wx + B * wy * wz;
    R[6] = -A * wy + B * wx * wz; R[7] = A * wx + B * wy * wz; R[8] = 1.0 + B * (wz * wz - th2);
}

/* FP64 Cholesky + SO(3) exponential; the reference's 6x6 solve lives in the
 * missing application layer. */
int or_icp_solve(const double *sums, double *R9, double *t3, double *x6) {
    double A[6][6], b[6], L[6][6] = {{0}}, y[6], x[6];
    int s = 0;
    for (int k = 0; k < 6; ++k)
        for (int j = k; j < 7; ++j) {
            double v = sums[s++];
            if (j == 6) b[k] = v; else { A[k][j] = v; A[j][k] = v; }
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j <= i; ++j) {
            double acc = A[i][j];
            for (int k = 0; k < j; ++k) acc -= L[i][k] * L[j][k];
            if (i == j) { if (!(acc > 1e-30)) return -1; L[i][i] = sqrt(acc); }
            else L[i][j] = acc / L[j][j];
        }
    for (int i = 0; i < 6; ++i) { double acc = b[i]; for (int k = 0; k < i; ++k) acc -= L[i][k] * y[k]; y[i] = acc / L[i][i]; }
    for (int i = 5; i >= 0; --i) { double acc = y[i]; for (int k = i + 1; k < 6; ++k) acc -= L[k][i] * x[k]; x[i] = acc / L[i][i]; }
    double Ri[9], Rn[9], tn[3];
    so3_exp_d(x, Ri);
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) Rn[3 * r + c] = Ri[3 * r] * R9[c] + Ri[3 * r + 1] * R9[3 + c] + Ri[3 * r + 2] * R9[6 + c];
        tn[r] = Ri[3 * r] * t3[0] + Ri[3 * r + 1] * t3[1] + Ri[3 * r + 2] * t3[2] + x[3 + r];
    }
    memcpy(R9, Rn, sizeof(Rn));
    memcpy(t3, tn, sizeof(tn));
    if (x6) memcpy(x6, x, sizeof(x));
    return 0;
}

/* ---------------- integration (integrate_tsdf_volume absent;
 * Integrate_Tsdf_Data opencl_wrappers.cpp:21-64).  Every voxel of every
 * column is visited: the CUDA kernel's analytic z bounds must not change the
 * result. */
int or_integrate(const float *depth, void *vol, int fmt, float trunc, const float *Ri, const float *t,
                 const tde_intrinsics *in, const float *cell, const tde_round_buffer *rb, int max_weight,
                 uint64_t *stats) {
    vol_t v = {fmt, vox_count(rb)};
    const int W = in->cols, H = in->rows, Nx = rb->voxels_size.x, Ny = rb->voxels_size.y, Nz = rb->voxels_size.z;
    const float ntrunc = -trunc, itrunc = 1.f / trunc;
    uint64_t n_read = 0, n_written = 0;
    /* Written with fused multiply-adds (fmaf) and correctly rounded
     * reciprocals in place of divisions, operation for operation as the GPU
     * sweep (k_integrate.cu), which is compiled without contraction. */
#pragma omp parallel for schedule(static) reduction(+ : n_read, n_written)
    for (int y = 0; y < Ny; ++y)
        for (int x = 0; x < Nx; ++x) {
            const float gx = ((float)x + 0.5f) * cell[0] - t[0];
            const float gy = ((float)y + 0.5f) * cell[1] - t[1];
            for (int z = 0; z < Nz; ++z) {
                const float gz = ((float)z + 0.5f) * cell[2] - t[2];
                const float vx = fmaf(Ri[2], gz, fmaf(Ri[1], gy, Ri[0] * gx));
                const float vy = fmaf(Ri[5], gz, fmaf(Ri[4], gy, Ri[3] * gx));
                const float vz = fmaf(Ri[8], gz, fmaf(Ri[7], gy, Ri[6] * gx));
                if (!(vz > 0.f)) continue;
                const float iz = 1.f / vz;
                int u = rint_sat(fmaf(vx, in->fx * iz, in->cx));
                int w = rint_sat(fmaf(vy, in->fy * iz, in->cy));
                if (u < 0 || u >= W || w < 0 || w >= H) continue;
                float Dp = depth[(size_t)w * W + u];
                if (Dp == 0.f) continue;
                const float n2 = fmaf(gz, gz, fmaf(gy, gy, gx * gx));
                float sdf = Dp - sqrtf(n2);
                if (!(sdf >= ntrunc)) continue;
                size_t idx = or_voxel_address(x, y, z, rb);
                float fo; int wo; uint32_t raw;
                rec_load(vol, v, idx, &fo, &wo, &raw);
                ++n_read;
                float tsdf = fminf(1.f, sdf * itrunc);
                float fw = (float)wo;
                /* the running mean as an increment: f + (tsdf - f) / (w + 1), so
                 * that a voxel at f = tsdf (free space at 1) keeps its bits */
                float fnew = fmaf(tsdf - fo, 1.f / (fw + 1.f), fo);
                int wnew = imin(wo + 1, max_weight);
                n_written += (uint64_t)rec_store(vol, v, idx, fnew, wnew);
            }
        }
    if (stats) { stats[0] = n_read; stats[1] = n_written; }
    return 0;
}

/* ---------------- resize (kernels absent; opencl_wrappers.cpp:97-146) ---- */
int or_resize_map(const float *src, float *dst, int sc, int sr, int normal) {
    int dc = sc >> 1, dr = sr >> 1;
    for (int y = 0; y < dr; ++y)
        for (int x = 0; x < dc; ++x) {
            float sx = 0.f, sy = 0.f, sz = 0.f;
            int ok = 1;
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    size_t i = 3 * ((size_t)(2 * y + dy) * sc + (2 * x + dx));
                    ok = ok && !isnan(src[i]);
                    sx = sx + src[i]; sy = sy + src[i + 1]; sz = sz + src[i + 2];
                }
            float o[3] = {OR_QNAN, OR_QNAN, OR_QNAN};
            if (ok) {
                if (normal) {
                    float d = 0.f; d += sx * sx; d += sy * sy; d += sz * sz;
                    float rs = 1.f / sqrtf(d);
                    o[0] = sx * rs; o[1] = sy * rs; o[2] = sz * rs;
                } else {
                    o[0] = sx * 0.25f; o[1] = sy * 0.25f; o[2] = sz * 0.25f;
                }
            }
            memcpy(dst + 3 * ((size_t)y * dc + x), o, 12);
        }
    return 0;
}

/* ---------------- transform_map.cl:6-65 ---------------------------------- */
int or_transform_maps(const float *vs, const float *ns, float *vd, float *nd, const float *R, const float *t, int W,
                      int H) {
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        v3 v = {vs[3 * i], vs[3 * i + 1], vs[3 * i + 2]}, vo = {OR_QNAN, OR_QNAN, OR_QNAN};
        if (!isnan(v.x)) { v3 r = mat_vec(R, v); vo.x = r.x + t[0]; vo.y = r.y + t[1]; vo.z = r.z + t[2]; }
        v3 n = {ns[3 * i], ns[3 * i + 1], ns[3 * i + 2]}, no = {OR_QNAN, OR_QNAN, OR_QNAN};
        if (!isnan(n.x)) no = mat_vec(R, n);
        memcpy(vd + 3 * i, &vo, 12);
        memcpy(nd + 3 * i, &no, 12);
    }
    return 0;
}

/* ---------------- transform_estimation.cl:4-53 (FP64 row sums) ---------- */
int or_transform_estimation(const float *gbuf, float *out, int len, int stride) {
    for (int g = 0; g < 27; ++g) {
        double s = 0.0;
        for (int i = 0; i < len; ++i) s += gbuf[(size_t)g * stride + i];
        out[g] = (float)s;
    }
    return 0;
}

/* ---------------- slab extraction ----------------------------------------
 * scan_slice_of_both_volumes.cl:76-208 (predicates, +z test bounded by the
 * chunk end), exclusive scan (scan_wrapper, absent; exclusive semantics from
 * extract_slice_as_cloud.cl:125-133) and extract_slice_as_cloud.cl:72-201
 * (point = neighbour voxel index, w = 1; colour of the named voxel).
 * Order: chunk, plane (+x, +y, +z, colour), (z, y, x). */
static int crossing(float F, float Fn, int Wn) {
    return (Wn != 0 && Fn != 1.f) && ((F > 0 && Fn < 0) || (F < 0 && Fn > 0));
}
static int black_zone(int x, int y, int z, const int *mn, const int *mx, const tde_round_buffer *rb) {
    int ix = x + rb->origin_GRID.x, iy = y + rb->origin_GRID.y, iz = z + rb->origin_GRID.z;
    return (ix >= mn[0] && ix <= mx[0]) || (iy >= mn[1] && iy <= mx[1]) || (iz >= mn[2] && iz <= mx[2]);
}

int64_t or_extract_slice(const void *vol, int fmt, const tde_color *color, const int *mn, const int *mx,
                         const tde_round_buffer *rb, int step, tde_xyzi *pts, tde_color *cols, float *wts,
                         int64_t capacity) {
    vol_t v = {fmt, vox_count(rb)};
    const int W = rb->voxels_size.x, H = rb->voxels_size.y, D = rb->voxels_size.z;
    if (step <= 0 || D % step) return -1;
    size_t plane = (size_t)W * H * step;
    uint8_t *bits = (uint8_t *)calloc(plane, 1);
    if (!bits) return -1;
    int64_t count = 0;
    for (int c0 = 0; c0 < D; c0 += step) {
        const int c1 = c0 + step;
#pragma omp parallel for schedule(static)
        for (int z = c0; z < c1; ++z)
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x) {
                    uint8_t b = 0;
                    if (black_zone(x, y, z, mn, mx, rb)) {
                        float F, Fn; int Wt, Wn; uint32_t r;
                        rec_load(vol, v, or_voxel_address(x, y, z, rb), &F, &Wt, &r);
                        if (Wt != 0 && F != 1.f) {
                            if (x + 1 < W) { rec_load(vol, v, or_voxel_address(x + 1, y, z, rb), &Fn, &Wn, &r); if (crossing(F, Fn, Wn)) b |= 1; }
                            if (y + 1 < H) { rec_load(vol, v, or_voxel_address(x, y + 1, z, rb), &Fn, &Wn, &r); if (crossing(F, Fn, Wn)) b |= 2; }
                            if (z + 1 < c1) { rec_load(vol, v, or_voxel_address(x, y, z + 1, rb), &Fn, &Wn, &r); if (crossing(F, Fn, Wn)) b |= 4; }
                        }
                        if (color) {
                            tde_color cc = color[or_voxel_address(x, y, z, rb)];
                            if (cc.r | cc.g | cc.b | cc.w) b |= 8;
                        }
                    }
                    bits[(size_t)(z - c0) * W * H + (size_t)y * W + x] = b;
                }
        for (int q = 0; q < 4; ++q)
            for (size_t r = 0; r < plane; ++r) {
                if (!((bits[r] >> q) & 1)) continue;
                if (count < capacity) {
                    int z = c0 + (int)(r / ((size_t)W * H)), y = (int)((r / W) % H), x = (int)(r % W);
                    int nx = x + (q == 0), ny = y + (q == 1), nz = z + (q == 2);
                    tde_xyzi p = {(float)nx, (float)ny, (float)nz, 1.0f};
                    pts[count] = p;
                    size_t a = or_voxel_address(nx, ny, nz, rb);
                    if (cols) { tde_color z0 = {0, 0, 0, 0}; cols[count] = color ? color[a] : z0; }
                    if (wts) { float f; int w; uint32_t raw; rec_load(vol, v, a, &f, &w, &raw); wts[count] = (float)w; }
                }
                ++count;
            }
    }
    free(bits);
    return count;
}

/* Extract_Tsdf_Volume (common/src/opencl_wrappers.cpp:440-543; its kernels
 * scan_the_whole_array / extract_tsdf_cloud are not in the reference): the
 * slab scan above with every voxel in the zone and no colour plane, chunks of
 * `step`, and each point moved to the metric centre (i + 0.5f) * cell of the
 * voxel it names (the V of extract_slice_as_cloud.cl:99-112), each operation
 * rounded to float. */
int64_t or_extract_tsdf_volume(const void *vol, int fmt, const tde_round_buffer *rb, int step, const float *cell,
                               tde_xyzi *pts, float *wts, int64_t capacity) {
    const int lo[3] = {INT_MIN, INT_MIN, INT_MIN}, hi[3] = {INT_MAX, INT_MAX, INT_MAX};
    int64_t n = or_extract_slice(vol, fmt, NULL, lo, hi, rb, step, pts, NULL, wts, capacity);
    int64_t k = n < capacity ? n : capacity;
    for (int64_t i = 0; i < k; ++i) {
        float x = pts[i].x + 0.5f, y = pts[i].y + 0.5f, z = pts[i].z + 0.5f;
        pts[i].x = x * cell[0];
        pts[i].y = y * cell[1];
        pts[i].z = z * cell[2];
    }
    return n;
}

/* Extract_Color_Volume (common/src/opencl_wrappers.cpp:545-581; kernel
 * extract_colors not in the reference): the colour of voxel floor(p / cell)
 * per axis, zero outside the volume. */
void or_extract_color_volume(const tde_color *color, const tde_round_buffer *rb, const tde_xyzi *pts, int64_t n,
                             const float *cell, tde_color *out) {
    for (int64_t i = 0; i < n; ++i) {
        float fx = floorf(pts[i].x / cell[0]), fy = floorf(pts[i].y / cell[1]), fz = floorf(pts[i].z / cell[2]);
        tde_color c = {0, 0, 0, 0};
        if (fx >= 0.f && fy >= 0.f && fz >= 0.f && fx < (float)rb->voxels_size.x && fy < (float)rb->voxels_size.y &&
            fz < (float)rb->voxels_size.z)
            c = color[or_voxel_address((int)fx, (int)fy, (int)fz, rb)];
        out[i] = c;
    }
}

int or_clean_tsdf_slice(void *vol, int fmt, const int *mn, const int *mx, const tde_round_buffer *rb) {
    vol_t v = {fmt, vox_count(rb)};
    for (int z = 0; z < rb->voxels_size.z; ++z)
        for (int y = 0; y < rb->voxels_size.y; ++y)
            for (int x = 0; x < rb->voxels_size.x; ++x)
                if (black_zone(x, y, z, mn, mx, rb)) rec_store(vol, v, or_voxel_address(x, y, z, rb), 0.f, 0);
    return 0;
}

/* clean_color_slice.cl:41-67 */
/* ---------------- colour integration (Integrate_Colors, opencl_wrappers.cpp:181-214; the kernel
 * integrate_color_volume is absent and is restated from KinectFusion's colour averaging).  Every
 * voxel is visited: its centre is projected into the frame; where the model surface point at that
 * pixel (the raycast vertex map, volume frame) lies closer than the truncation distance to the centre,
 * the voxel's colour becomes the weighted running mean of its colour and the pixel's, each channel
 * rounded to nearest (ties to even), and its weight grows by one up to max_weight. */
int or_integrate_colors(tde_color *col, const uint8_t *rgb, const float *vmap, float trunc, const float *Ri,
                        const float *t, const tde_intrinsics *in, const float *cell, const tde_round_buffer *rb,
                        int max_weight, uint64_t *updated) {
    const int W = in->cols, H = in->rows, Nx = rb->voxels_size.x, Ny = rb->voxels_size.y, Nz = rb->voxels_size.z;
    const int mw = imin(max_weight, 255);
    uint64_t n_up = 0;
#pragma omp parallel for schedule(static) reduction(+ : n_up)
    for (int y = 0; y < Ny; ++y)
        for (int x = 0; x < Nx; ++x) {
            const float ax = ((float)x + 0.5f) * cell[0], ay = ((float)y + 0.5f) * cell[1];
            const float gx = ax - t[0], gy = ay - t[1];
            for (int z = 0; z < Nz; ++z) {
                const float az = ((float)z + 0.5f) * cell[2];
                const float gz = az - t[2];
                float vx = 0.f; vx += Ri[0] * gx; vx += Ri[1] * gy; vx += Ri[2] * gz;
                float vy = 0.f; vy += Ri[3] * gx; vy += Ri[4] * gy; vy += Ri[5] * gz;
                float vz = 0.f; vz += Ri[6] * gx; vz += Ri[7] * gy; vz += Ri[8] * gz;
                if (!(vz > 0.f)) continue;
                int u = rint_sat(vx * in->fx / vz + in->cx);
                int w = rint_sat(vy * in->fy / vz + in->cy);
                if (u < 0 || u >= W || w < 0 || w >= H) continue;
                const float *pv = vmap + 3 * ((size_t)w * W + u);
                if (isnan(pv[0])) continue;
                const float dx = pv[0] - ax, dy = pv[1] - ay, dz = pv[2] - az;
                float d2 = 0.f; d2 += dx * dx; d2 += dy * dy; d2 += dz * dz;
                if (!(sqrtf(d2) < trunc)) continue;
                tde_color *c = &col[or_voxel_address(x, y, z, rb)];
                const uint8_t *src = rgb + 3 * ((size_t)w * W + u);
                const float fw = (float)c->w, fw1 = fw + 1.f;
                const int r = imax(0, imin(255, rint_sat(((float)c->r * fw + (float)src[0]) / fw1)));
                const int g = imax(0, imin(255, rint_sat(((float)c->g * fw + (float)src[1]) / fw1)));
                const int b = imax(0, imin(255, rint_sat(((float)c->b * fw + (float)src[2]) / fw1)));
                c->r = (uint8_t)r; c->g = (uint8_t)g; c->b = (uint8_t)b;
                c->w = (uint8_t)imin((int)c->w + 1, mw);
                ++n_up;
            }
        }
    if (updated) *updated = n_up;
    return 0;
}

int or_clean_color_slice(tde_color *col, const int *mn, const int *mx, const tde_round_buffer *rb) {
    for (int z = 0; z < rb->voxels_size.z; ++z)
        for (int y = 0; y < rb->voxels_size.y; ++y)
            for (int x = 0; x < rb->voxels_size.x; ++x)
                if (black_zone(x, y, z, mn, mx, rb)) {
                    tde_color z0 = {0, 0, 0, 0};
                    col[or_voxel_address(x, y, z, rb)] = z0;
                }
    return 0;
}

/* Generate_Image (common/src/opencl_wrappers.cpp:967-992; kernel
 * generate_image not in the reference): the published KinectFusion image
 * generator -- w = |dot(normalize(light - v), n)| (1 without a light, 0 with
 * the light on v), grey = clamp(trunc(205 w) + 50, 0, 255), black where the
 * vertex or normal is invalid.  Float operations in the kernel's order. */
void or_generate_image(const float *vmap, const float *nmap, int64_t npix, const float *light, int nlights,
                       uint8_t *image) {
    for (int64_t i = 0; i < npix; ++i) {
        const float *v = vmap + 3 * i, *n = nmap + 3 * i;
        int br = 0;
        if (!isnan(v[0]) && !isnan(n[0])) {
            float w = 1.f;
            if (nlights > 0) {
                float dx = light[0] - v[0], dy = light[1] - v[1], dz = light[2] - v[2];
                float d2 = dx * dx + dy * dy + dz * dz;
                if (d2 > 0.f) {
                    float inv = 1.f / sqrtf(d2);
                    dx *= inv; dy *= inv; dz *= inv;
                    w = fabsf(dx * n[0] + dy * n[1] + dz * n[2]);
                } else {
                    w = 0.f;
                }
            }
            if (isnan(w)) w = 0.f;  /* a NaN in y or z of an otherwise valid pixel */
            else if (w > 2.f) w = 2.f;  /* non-unit normals: 255 either way, no int overflow */
            br = (int)(205.f * w) + 50;
            br = br < 0 ? 0 : (br > 255 ? 255 : br);
        }
        image[3 * i] = image[3 * i + 1] = image[3 * i + 2] = (uint8_t)br;
    }
}
