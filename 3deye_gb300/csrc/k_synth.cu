// k_synth.cu -- synthetic depth sensor: ray-casts the seeded procedural scene
// (plane / sphere / axis-aligned box primitives) and applies the Kinect noise
// model.  It produces benchmark and test inputs; it is not part of the
// per-frame pipeline.  Every operation is IEEE exact or correctly rounded and
// the unit is compiled without contraction, so its frames equal the CPU
// sensor's bit for bit (the CPU arm of the benchmark renders the same ones).
#include "tde_common.cuh"

namespace tde {
namespace {

__device__ double hit_prim(const double *P, const double o[3], const double d[3]) {
    const double inf = 1e300;
    const int type = (int)P[0];
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
        double Cc = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - a[3] * a[3];
        double disc = B * B - A * Cc;
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
            tmin = fmax(tmin, t1);
            tmax = fmin(tmax, t2);
        }
        if (tmax < tmin) return inf;
        if (tmin > 1e-9) return tmin;
        if (tmax > 1e-9) return tmax;
        return inf;
    }
    return inf;
}

// lowbias32 integer hash (C. Wellons, public domain); same as the CPU sensor.
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float u01(uint32_t h) { return ((float)(h >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// Standard normal deviate as the Irwin-Hall sum of 12 uniforms minus 6 (mean
// 0, variance 1): twelve 16-bit uniforms from six hashes; the numerator is an
// integer below 2^19 and the scale a power of two, so the result is exact and
// equal to the CPU sensor's.
__device__ __forceinline__ float gauss12(uint32_t key) {
    const uint32_t salt[6] = {0x02e5be93U, 0x967a889bU, 0x1b873593U, 0xcc9e2d51U, 0x85ebca6bU, 0xc2b2ae35U};
    int32_t sum = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const uint32_t h = hash32(key ^ salt[k]);
        sum += (int32_t)(h & 0xFFFFu) + (int32_t)(h >> 16);
    }
    return (float)(sum + 6 - 6 * 65536) * (1.0f / 65536.0f);
}

struct SynthParams {
    double R[9], t[3];
    tde_intrinsics intr;
    int nprim;
    uint32_t seed, frame;
    float max_range, dropout;
};

__global__ void synth_kernel(const double *__restrict__ scene, const SynthParams p, uint16_t *__restrict__ out_mm,
                             float *__restrict__ out_m) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= p.intr.cols || v >= p.intr.rows) return;
    extern __shared__ double s_scene[];
    (void)s_scene;
    double dc[3] = {((double)u - p.intr.cx) / p.intr.fx, ((double)v - p.intr.cy) / p.intr.fy, 1.0};
    double d[3] = {p.R[0] * dc[0] + p.R[1] * dc[1] + p.R[2] * dc[2], p.R[3] * dc[0] + p.R[4] * dc[1] + p.R[5] * dc[2],
                   p.R[6] * dc[0] + p.R[7] * dc[1] + p.R[8] * dc[2]};
    double best = 1e300;
    for (int k = 0; k < p.nprim; ++k) best = fmin(best, hit_prim(scene + 8 * k, p.t, d));
    const float z = best < 1e299 ? (float)best : 0.f;
    const int i = v * p.intr.cols + u;
    if (out_m) out_m[i] = z;
    if (out_mm) {
        uint32_t key = hash32(p.seed ^ hash32(p.frame * 0x9e3779b9U ^ hash32((uint32_t)i)));
        float ud = u01(hash32(key ^ 0x68bc21ebU));
        uint16_t o = 0;
        if (z > 0.f && z <= p.max_range && ud >= p.dropout) {
            float g = gauss12(key);
            float s = 0.0012f + 0.0019f * (z - 0.4f) * (z - 0.4f);
            float mm = nearbyintf((z + s * g) * 1000.f);
            if (mm > 0.f && mm <= p.max_range * 1000.f && mm < 65535.f) o = (uint16_t)mm;
        }
        out_mm[i] = o;
    }
}

// Procedural colour of a surface point: triangle waves of its coordinates
// (exact or correctly rounded operations; the CPU sensor's texture).
__device__ __forceinline__ double tri(double a) { return fabs(a - floor(a) - 0.5); }

__global__ void synth_rgb_kernel(const double *__restrict__ scene, const SynthParams p, uint8_t *__restrict__ rgb) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= p.intr.cols || v >= p.intr.rows) return;
    double dc[3] = {((double)u - p.intr.cx) / p.intr.fx, ((double)v - p.intr.cy) / p.intr.fy, 1.0};
    double d[3] = {p.R[0] * dc[0] + p.R[1] * dc[1] + p.R[2] * dc[2], p.R[3] * dc[0] + p.R[4] * dc[1] + p.R[5] * dc[2],
                   p.R[6] * dc[0] + p.R[7] * dc[1] + p.R[8] * dc[2]};
    double best = 1e300;
    for (int k = 0; k < p.nprim; ++k) best = fmin(best, hit_prim(scene + 8 * k, p.t, d));
    uint8_t *o = rgb + 3 * ((size_t)v * p.intr.cols + u);
    if (best < 1e299) {
        const double X[3] = {p.t[0] + best * d[0], p.t[1] + best * d[1], p.t[2] + best * d[2]};
        const double a = tri(X[0] * 7.0 + X[1] * 3.0), b = tri(X[1] * 9.0 - X[2] * 5.0),
                     c = tri(X[2] * 11.0 + X[0] * 4.0), e = tri((X[0] + X[1] + X[2]) * 23.0);
        o[0] = (uint8_t)(40.0 + 400.0 * a * 0.5 + 200.0 * e * 0.5);
        o[1] = (uint8_t)(40.0 + 400.0 * b * 0.5 + 200.0 * e * 0.5);
        o[2] = (uint8_t)(40.0 + 400.0 * c * 0.5 + 200.0 * e * 0.5);
    } else {
        o[0] = o[1] = o[2] = 0;
    }
}

}  // namespace
}  // namespace tde

using namespace tde;

extern "C" {

// Synthetic sensor: renders `scene` (device, nprim x 8 doubles) from pose12
// (host: R camera->world row-major, t) and writes noisy uint16 depth in mm
// (out_mm) and/or the noise-free depth in metres (out_m), both device.
int tde_synth_depth(const double *scene, int nprim, const double *pose12, const tde_intrinsics *intr, uint32_t seed,
                    uint32_t frame, float max_range_m, float dropout, uint16_t *out_mm, float *out_m, void *stream) {
    if (!scene || nprim <= 0 || !pose12 || !intr || (!out_mm && !out_m) || intr->cols <= 0 || intr->rows <= 0)
        return set_error(TDE_ERR_INVALID_ARG, "synth_depth: bad arguments");
    SynthParams p;
    for (int k = 0; k < 9; ++k) p.R[k] = pose12[k];
    for (int k = 0; k < 3; ++k) p.t[k] = pose12[9 + k];
    p.intr = *intr; p.nprim = nprim; p.seed = seed; p.frame = frame; p.max_range = max_range_m; p.dropout = dropout;
    dim3 block(32, 8), grid(div_up(intr->cols, 32), div_up(intr->rows, 8));
    synth_kernel<<<grid, block, 0, as_stream(stream)>>>(scene, p, out_mm, out_m);
    return check_launch("synth_depth");
}

// Synthetic colour camera: the scene's procedural texture at each pixel's
// nearest hit from pose12 (host), black without a hit; rgb: device, 3 bytes
// a pixel.  Same ray and camera as tde_synth_depth.
int tde_synth_rgb(const double *scene, int nprim, const double *pose12, const tde_intrinsics *intr, uint8_t *rgb,
                  void *stream) {
    if (!scene || nprim <= 0 || !pose12 || !intr || !rgb || intr->cols <= 0 || intr->rows <= 0)
        return set_error(TDE_ERR_INVALID_ARG, "synth_rgb: bad arguments");
    SynthParams p = {};
    for (int k = 0; k < 9; ++k) p.R[k] = pose12[k];
    for (int k = 0; k < 3; ++k) p.t[k] = pose12[9 + k];
    p.intr = *intr;
    p.nprim = nprim;
    dim3 block(32, 8), grid(div_up(intr->cols, 32), div_up(intr->rows, 8));
    synth_rgb_kernel<<<grid, block, 0, as_stream(stream)>>>(scene, p, rgb);
    return check_launch("synth_rgb");
}

}  // extern "C"
