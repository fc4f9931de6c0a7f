/* oracle_f64.c -- full-FP64 restatement of the model stages, for the storage
 * precision study (TEST INFRASTRUCTURE ONLY).
 *
 * The TSDF is kept as FP64 values with integer weights (no storage rounding)
 * and every stage computes in FP64: integration (the KinectFusion projective
 * update with the reference's conventions: encoding range [-1, 1], weight cap,
 * voxel centres at (i + 0.5) * cell), the raycast (GPU/opencl/raycast.cl:182-405:
 * 0.8 * trunc steps, sign-change test, secant refinement, central-difference
 * normals, trilinear interpolation raycast.cl:95-145), and the ICP terms
 * (projective association, point-to-plane rows, FP64 sums).  Addresses follow
 * calculate_address (raycast.cl:29-47) through or_voxel_address.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle.h"

#define QNAN_D (0.0 / 0.0)

typedef struct { double x, y, z; } d3;

static d3 mv(const double *M, d3 v) {
    d3 r = {M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
            M[6] * v.x + M[7] * v.y + M[8] * v.z};
    return r;
}
static double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static d3 cross(d3 a, d3 b) {
    d3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static d3 along(const double *o, d3 d, double t) {
    d3 r = {o[0] + d.x * t, o[1] + d.y * t, o[2] + d.z * t};
    return r;
}

/* depth along the ray in metres from uint16 mm (scale_depth in FP64) */
int or_scale_depth_f64(const uint16_t *depth, double *scaled, const tde_intrinsics *in) {
    for (int y = 0; y < in->rows; ++y)
        for (int x = 0; x < in->cols; ++x) {
            size_t o = (size_t)y * in->cols + x;
            double xl = ((double)x - in->cx) / in->fx, yl = ((double)y - in->cy) / in->fy;
            scaled[o] = (double)depth[o] * sqrt(xl * xl + yl * yl + 1.0) / 1000.0;
        }
    return 0;
}

int or_integrate_f64(const double *depth, double *tsdf, int32_t *weight, double trunc, const double *Ri,
                     const double *t, const tde_intrinsics *in, const double *cell, const tde_round_buffer *rb,
                     int max_weight) {
    const int W = in->cols, H = in->rows, Nx = rb->voxels_size.x, Ny = rb->voxels_size.y, Nz = rb->voxels_size.z;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < Ny; ++y)
        for (int x = 0; x < Nx; ++x) {
            const double gx = ((double)x + 0.5) * cell[0] - t[0];
            const double gy = ((double)y + 0.5) * cell[1] - t[1];
            for (int z = 0; z < Nz; ++z) {
                const double gz = ((double)z + 0.5) * cell[2] - t[2];
                d3 g = {gx, gy, gz};
                d3 v = mv(Ri, g);
                if (!(v.z > 0.0)) continue;
                const double uf = v.x * in->fx / v.z + in->cx, wf = v.y * in->fy / v.z + in->cy;
                if (!(uf > -1.0 && uf < W + 1.0 && wf > -1.0 && wf < H + 1.0)) continue;
                const int u = (int)nearbyint(uf), w = (int)nearbyint(wf);
                if (u < 0 || u >= W || w < 0 || w >= H) continue;
                const double Dp = depth[(size_t)w * W + u];
                if (Dp == 0.0) continue;
                const double sdf = Dp - sqrt(dot(g, g));
                if (!(sdf >= -trunc)) continue;
                const size_t idx = or_voxel_address(x, y, z, rb);
                const double f = sdf / trunc < 1.0 ? sdf / trunc : 1.0;
                const int wo = weight[idx];
                tsdf[idx] = (tsdf[idx] * wo + f) / (wo + 1.0);
                weight[idx] = wo + 1 < max_weight ? wo + 1 : max_weight;
            }
        }
    return 0;
}

typedef struct { const double *f; const tde_round_buffer *rb; const double *cell; } ctx64;

static double rd(const ctx64 *c, int x, int y, int z) { return c->f[or_voxel_address(x, y, z, c->rb)]; }

static double trilinear(const ctx64 *c, d3 p) {
    const tde_point3i N = c->rb->voxels_size;
    const double *cs = c->cell;
    int gx = (int)floor(p.x / cs[0]), gy = (int)floor(p.y / cs[1]), gz = (int)floor(p.z / cs[2]);
    if (gx <= 0 || gx >= N.x - 1 || gy <= 0 || gy >= N.y - 1 || gz <= 0 || gz >= N.z - 1) return QNAN_D;
    const double vx = (gx + 0.5) * cs[0], vy = (gy + 0.5) * cs[1], vz = (gz + 0.5) * cs[2];
    gx = p.x < vx ? gx - 1 : gx;
    gy = p.y < vy ? gy - 1 : gy;
    gz = p.z < vz ? gz - 1 : gz;
    double a = p.x / cs[0] - (gx + 0.5); if (a < 0) { gx--; a += 1.0; }
    double b = p.y / cs[1] - (gy + 0.5); if (b < 0) { gy--; b += 1.0; }
    double cc = p.z / cs[2] - (gz + 0.5); if (cc < 0) { gz--; cc += 1.0; }
    const double r000 = rd(c, gx, gy, gz), r001 = rd(c, gx, gy, gz + 1), r010 = rd(c, gx, gy + 1, gz),
                 r011 = rd(c, gx, gy + 1, gz + 1), r100 = rd(c, gx + 1, gy, gz), r101 = rd(c, gx + 1, gy, gz + 1),
                 r110 = rd(c, gx + 1, gy + 1, gz), r111 = rd(c, gx + 1, gy + 1, gz + 1);
    const double x0 = (1 - b) * (r000 * (1 - cc) + r001 * cc) + b * (r010 * (1 - cc) + r011 * cc);
    const double x1 = (1 - b) * (r100 * (1 - cc) + r101 * cc) + b * (r110 * (1 - cc) + r111 * cc);
    return (1 - a) * x0 + a * x1;
}

int or_raycast_f64(const double *tsdf, double *vmap, double *nmap, const double *t, const double *R, double trunc,
                   const tde_intrinsics *intr, const tde_round_buffer *rb, const double *cell) {
    ctx64 c = {tsdf, rb, cell};
    const int W = intr->cols, H = intr->rows;
    const double step = trunc * 0.8;
    const double V[3] = {rb->volume_size.x, rb->volume_size.y, rb->volume_size.z};
    const tde_point3i N = rb->voxels_size;
    const double max_time = 3.0 * (V[0] + V[1] + V[2]);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t pix = (size_t)W * y + x;
            double out[6] = {QNAN_D, QNAN_D, QNAN_D, QNAN_D, QNAN_D, QNAN_D};
            d3 ru = {((double)x - intr->cx) / intr->fx, ((double)y - intr->cy) / intr->fy, 1.0};
            d3 d = mv(R, ru);
            const double dn = sqrt(dot(d, d));
            d.x /= dn; d.y /= dn; d.z /= dn;
            d.x = d.x == 0.0 ? 1e-15 : d.x;
            d.y = d.y == 0.0 ? 1e-15 : d.y;
            d.z = d.z == 0.0 ? 1e-15 : d.z;
            const double dd[3] = {d.x, d.y, d.z};
            double ts = 0.0, te = 1e300;
            for (int k = 0; k < 3; ++k) {
                const double t0 = ((dd[k] > 0 ? 0.0 : V[k]) - t[k]) / dd[k];
                const double t1 = ((dd[k] > 0 ? V[k] : 0.0) - t[k]) / dd[k];
                ts = t0 > ts ? t0 : ts;
                te = t1 < te ? t1 : te;
            }
            if (!(ts >= te)) {
                double tc = ts;
                d3 pu = along(t, d, tc);
                int gx = (int)floor(pu.x / cell[0]), gy = (int)floor(pu.y / cell[1]), gz = (int)floor(pu.z / cell[2]);
                gx = gx < 0 ? 0 : gx >= N.x ? N.x - 1 : gx;
                gy = gy < 0 ? 0 : gy >= N.y ? N.y - 1 : gy;
                gz = gz < 0 ? 0 : gz >= N.z ? N.z - 1 : gz;
                double f = rd(&c, gx, gy, gz);
                for (; tc < max_time; tc += step) {
                    const double prev = f, ct = tc + step;
                    d3 q = along(t, d, ct);
                    const int sx = (int)floor(q.x / cell[0]), sy = (int)floor(q.y / cell[1]),
                              sz = (int)floor(q.z / cell[2]);
                    if (!(sx >= 0 && sy >= 0 && sz >= 0 && sx < N.x && sy < N.y && sz < N.z)) break;
                    f = rd(&c, sx, sy, sz);
                    if (prev < 0.0 && f > 0.0) break;
                    if (prev > 0.0 && f < 0.0) {
                        const double Ftdt = trilinear(&c, along(t, d, ct));
                        if (isnan(Ftdt)) break;
                        const double Ft = trilinear(&c, along(t, d, tc));
                        if (isnan(Ft)) break;
                        const double Ts = tc - step * Ft / (Ftdt - Ft);
                        d3 vf = along(t, d, Ts);
                        out[0] = vf.x; out[1] = vf.y; out[2] = vf.z;
                        d3 p3 = along(t, d, tc);
                        const int hx = (int)floor(p3.x / cell[0]), hy = (int)floor(p3.y / cell[1]),
                                  hz = (int)floor(p3.z / cell[2]);
                        if (hx > 1 && hy > 1 && hz > 1 && hx < N.x - 2 && hy < N.y - 2 && hz < N.z - 2) {
                            d3 tt;
                            tt = vf; tt.x += cell[0]; const double Fx1 = trilinear(&c, tt);
                            tt = vf; tt.x -= cell[0]; const double Fx2 = trilinear(&c, tt);
                            tt = vf; tt.y += cell[1]; const double Fy1 = trilinear(&c, tt);
                            tt = vf; tt.y -= cell[1]; const double Fy2 = trilinear(&c, tt);
                            tt = vf; tt.z += cell[2]; const double Fz1 = trilinear(&c, tt);
                            tt = vf; tt.z -= cell[2]; const double Fz2 = trilinear(&c, tt);
                            d3 nn = {Fx1 - Fx2, Fy1 - Fy2, Fz1 - Fz2};
                            const double l = sqrt(dot(nn, nn));
                            out[3] = nn.x / l; out[4] = nn.y / l; out[5] = nn.z / l;
                        }
                        break;
                    }
                }
            }
            memcpy(vmap + 3 * pix, out, 24);
            memcpy(nmap + 3 * pix, out + 3, 24);
        }
    return 0;
}

/* Projective association and point-to-plane terms in FP64 (27 + count). */
int or_icp_terms_f64(const float *vcur, const float *ncur, const double *vprev, const double *nprev,
                     const double *Rc, const double *tc, const double *Rpi, const double *tp,
                     const tde_intrinsics *in, double dist_thresh, double angle_thresh, double *sums) {
    const int W = in->cols, H = in->rows;
    for (int k = 0; k < 28; ++k) sums[k] = 0.0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * W + x;
            if (isnan(ncur[3 * i])) continue;
            d3 n = {ncur[3 * i], ncur[3 * i + 1], ncur[3 * i + 2]};
            d3 v = {vcur[3 * i], vcur[3 * i + 1], vcur[3 * i + 2]};
            d3 rv = mv(Rc, v);
            d3 vg = {rv.x + tc[0], rv.y + tc[1], rv.z + tc[2]};
            d3 dd = {vg.x - tp[0], vg.y - tp[1], vg.z - tp[2]};
            d3 vcp = mv(Rpi, dd);
            if (!(vcp.z > 0.0)) continue;
            const double uf = vcp.x * in->fx / vcp.z + in->cx, wf = vcp.y * in->fy / vcp.z + in->cy;
            if (!(uf > -1.0 && uf < W + 1.0 && wf > -1.0 && wf < H + 1.0)) continue;
            const int u = (int)nearbyint(uf), w = (int)nearbyint(wf);
            if (u < 0 || w < 0 || u >= W || w >= H) continue;
            const size_t j = (size_t)w * W + u;
            if (isnan(nprev[3 * j])) continue;
            d3 np = {nprev[3 * j], nprev[3 * j + 1], nprev[3 * j + 2]};
            d3 vp = {vprev[3 * j], vprev[3 * j + 1], vprev[3 * j + 2]};
            d3 dv = {vp.x - vg.x, vp.y - vg.y, vp.z - vg.z};
            if (sqrt(dot(dv, dv)) > dist_thresh) continue;
            d3 ng = mv(Rc, n);
            d3 cr = cross(ng, np);
            if (sqrt(dot(cr, cr)) >= angle_thresh) continue;
            d3 c = cross(vg, np);
            const double row[7] = {c.x, c.y, c.z, np.x, np.y, np.z, dot(np, dv)};
            int s = 0;
            for (int a = 0; a < 6; ++a)
                for (int b = a; b < 7; ++b) sums[s++] += row[a] * row[b];
            sums[27] += 1.0;
        }
    return 0;
}
