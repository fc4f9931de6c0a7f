// k_integrate.cu -- projective TSDF integration (Integrate_Tsdf_Data,
// common/src/opencl_wrappers.cpp:21-64; the reference kernel
// integrate_tsdf_volume is absent, this follows the KinectFusion update).
//
// Work is organised in 8^3-voxel bricks.  A first kernel tests each brick
// against the frame: the brick's voxel-centre box is projected (8 corners)
// and, if it lies entirely behind the camera, outside the image, or farther
// from the camera than the largest observed depth over the pixels it covers
// plus the truncation distance, none of its voxels can pass the per-voxel
// test, so the brick is dropped.  A second kernel sweeps the surviving bricks,
// one warp per brick, and applies the per-voxel update --
// the same IEEE float operations, in the same order, as the CPU oracle, which
// visits every voxel (fused multiply-adds and correctly rounded reciprocals
// written out on both sides, no divisions).  Culling only removes voxels the exact test rejects, so
// volumes are bit-identical.
//
// The maximum (and smallest non-zero) observed depth per screen tile comes
// from a 5-level pyramid (16..256-pixel tiles) built by depth_max_kernel each
// frame.  With saturation flags, a brick whose every voxel already holds f = 1
// at the maximum weight, and which lies entirely more than the truncation
// distance in front of the smallest depth it projects to, is not swept either:
// each of its voxels would get tsdf = 1 and keep f = 1, w = max, bit for bit.
//
// Built with -fmad=false (no contraction beyond the explicit __fmaf_rn) so every
// voxel decision and value equals the oracle's.
#include "tde_common.cuh"
#include "tde_integrate.cuh"

#include <algorithm>

namespace tde {
namespace {

constexpr int kBrick = 8;
constexpr float kNoDepth = 3.3961514e38f;  // bytes 0x7f7f7f7f: "no non-zero depth in the tile"

// ---------------------------------------------------------------------------
// Max scaled depth per 16x16 tile (level 0) and per 32..256 tiles (levels 1-4,
// by atomicMax on the bit pattern: non-negative floats order like ints).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) depth_max_kernel(const float *__restrict__ depth, int W, int H,
                                                        DepthMaxPyramid pyr) {
    __shared__ float red[8], red_min[8];
    const int tx = blockIdx.x, ty = blockIdx.y;
    const int x = tx * 16 + (threadIdx.x & 15), y = ty * 16 + (threadIdx.x >> 4);
    float m = 0.f, mn = kNoDepth;
    if (x < W && y < H) {
        const float d = depth[(size_t)y * W + x];
        m = fmaxf(0.f, d);
        if (d > 0.f) mn = d;
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = m; red_min[threadIdx.x >> 5] = mn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < 8; ++i) { m = fmaxf(m, red[i]); mn = fminf(mn, red_min[i]); }
        pyr.level[0][ty * pyr.tiles_x[0] + tx] = m;
        pyr.level_min[0][ty * pyr.tiles_x[0] + tx] = mn;
        // non-negative floats order like their bit patterns
        for (int l = 1; l < kDepthMaxLevels; ++l) {
            const int i = (ty >> l) * pyr.tiles_x[l] + (tx >> l);
            atomicMax(reinterpret_cast<int *>(&pyr.level[l][i]), __float_as_int(m));
            atomicMin(reinterpret_cast<int *>(&pyr.level_min[l][i]), __float_as_int(mn));
        }
    }
}

// Largest observed depth over pixel rectangle [u0,u1]x[v0,v1] (inclusive,
// inside the image); the level is chosen so the rectangle meets <= 2x2 tiles.
__device__ __forceinline__ float rect_max_depth(const DepthMaxPyramid &pyr, int u0, int v0, int u1, int v1) {
    const int ext = max(u1 - u0, v1 - v0) + 1;
    int l = 0;
    while (l < kDepthMaxLevels - 1 && (16 << l) < ext) ++l;
    if ((16 << l) < ext) return 3.0e38f;  // larger than the coarsest tile: never cull on depth
    const int s = 4 + l;  // log2 tile size
    float m = 0.f;
    for (int ty = v0 >> s; ty <= (v1 >> s); ++ty)
        for (int tx = u0 >> s; tx <= (u1 >> s); ++tx) m = fmaxf(m, pyr.level[l][ty * pyr.tiles_x[l] + tx]);
    return m;
}

// Smallest non-zero observed depth over the same rectangle; 0 (nothing
// provable) when the rectangle is larger than the coarsest tile.
__device__ __forceinline__ float rect_min_depth(const DepthMaxPyramid &pyr, int u0, int v0, int u1, int v1) {
    const int ext = max(u1 - u0, v1 - v0) + 1;
    int l = 0;
    while (l < kDepthMaxLevels - 1 && (16 << l) < ext) ++l;
    if ((16 << l) < ext) return 0.f;
    const int s = 4 + l;
    float m = kNoDepth;
    for (int ty = v0 >> s; ty <= (v1 >> s); ++ty)
        for (int tx = u0 >> s; tx <= (u1 >> s); ++tx) m = fminf(m, pyr.level_min[l][ty * pyr.tiles_x[l] + tx]);
    return m;
}

struct Pose {
    float Ri[9];
    float t[3];
};

// True when no voxel of brick (bx,by,bz) can pass the per-voxel test, or
// (saturated: every voxel holds f = 1 at the maximum weight) when every voxel
// that passes would get tsdf = 1 and so stay as it is.
// COLOR: the pyramid holds the model surface's distances from the camera
// instead, and a voxel can only be updated within the truncation distance of
// the model point at its pixel, so the brick must also reach past the
// smallest of those distances minus the truncation (triangle inequality).
template <bool COLOR = false>
__device__ __forceinline__ bool brick_culled(const IntegrateParams &P, const Pose &q, const DepthMaxPyramid &pyr, int bx,
                                             int by, int bz, bool saturated) {
    const tde_point3i &Nv = P.rb.voxels_size;
    const int x0 = bx * kBrick, y0 = by * kBrick, z0 = bz * kBrick;
    const int x1 = min(x0 + kBrick, Nv.x) - 1, y1 = min(y0 + kBrick, Nv.y) - 1, z1 = min(z0 + kBrick, Nv.z) - 1;
    // voxel-centre box, camera-relative
    const float lo[3] = {((float)x0 + 0.5f) * P.cell.x - q.t[0], ((float)y0 + 0.5f) * P.cell.y - q.t[1],
                         ((float)z0 + 0.5f) * P.cell.z - q.t[2]};
    const float hi[3] = {((float)x1 + 0.5f) * P.cell.x - q.t[0], ((float)y1 + 0.5f) * P.cell.y - q.t[1],
                         ((float)z1 + 0.5f) * P.cell.z - q.t[2]};
    float umin = 3e38f, umax = -3e38f, vmin = 3e38f, vmax = -3e38f;
    int behind = 0;
    bool near_plane = false;
    #pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float gx = (c & 1) ? hi[0] : lo[0], gy = (c & 2) ? hi[1] : lo[1], gz = (c & 4) ? hi[2] : lo[2];
        const float vx = q.Ri[0] * gx + q.Ri[1] * gy + q.Ri[2] * gz;
        const float vy = q.Ri[3] * gx + q.Ri[4] * gy + q.Ri[5] * gz;
        const float vz = q.Ri[6] * gx + q.Ri[7] * gy + q.Ri[8] * gz;
        if (vz <= 0.f) ++behind;
        if (vz < 1e-4f) { near_plane = true; continue; }
        const float iz = 1.f / vz;
        const float u = P.intr.fx * vx * iz + P.intr.cx, v = P.intr.fy * vy * iz + P.intr.cy;
        umin = fminf(umin, u); umax = fmaxf(umax, u); vmin = fminf(vmin, v); vmax = fmaxf(vmax, v);
    }
    if (behind == 8) return true;  // convex hull behind the camera plane
    if (near_plane) return false;  // projection unbounded: keep
    const int W = P.intr.cols, H = P.intr.rows;
    if (umax < -1.f || vmax < -1.f || umin > (float)W || vmin > (float)H) return true;  // outside the image
    const int u0 = max(0, (int)floorf(umin) - 1), u1 = min(W - 1, (int)ceilf(umax) + 1);
    const int v0 = max(0, (int)floorf(vmin) - 1), v1 = min(H - 1, (int)ceilf(vmax) + 1);
    if (u0 > u1 || v0 > v1) return true;
    const float dmax = rect_max_depth(pyr, u0, v0, u1, v1);
    // nearest distance from the camera centre to the box
    float d2 = 0.f;
    #pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float d = fmaxf(0.f, fmaxf(lo[a], -hi[a]));
        d2 += d * d;
    }
    if (sqrtf(d2) > dmax + P.trunc + 1e-3f + 1e-4f * dmax) return true;
    if (!saturated && !COLOR) return false;
    // farthest voxel centre: every voxel that projects onto a non-zero depth
    // Dp >= dmin has sdf = Dp - dist > trunc (margins far above float error)
    float dmin;
    if ((u1 >> 4) - (u0 >> 4) < 8 && (v1 >> 4) - (v0 >> 4) < 8) {
        dmin = kNoDepth;  // the 16-pixel tiles over the footprint
        for (int ty = v0 >> 4; ty <= (v1 >> 4); ++ty)
            for (int tx = u0 >> 4; tx <= (u1 >> 4); ++tx) dmin = fminf(dmin, pyr.level_min[0][ty * pyr.tiles_x[0] + tx]);
    } else {
        dmin = rect_min_depth(pyr, u0, v0, u1, v1);
    }
    float f2 = 0.f;
    #pragma unroll
    for (int a = 0; a < 3; ++a) f2 += fmaxf(lo[a] * lo[a], hi[a] * hi[a]);
    return dmin - sqrtf(f2) > P.trunc + 1e-3f + 1e-4f * dmin;  // COLOR: every voxel closer than every model point - trunc
}

// One thread per brick: surviving bricks are appended to a global list (its
// order varies run to run; every brick owns disjoint voxels, so the result
// does not depend on it).
template <bool COLOR = false>
__global__ void __launch_bounds__(256) cull_bricks_kernel(const IntegrateParams P,
                                                          const __grid_constant__ DepthMaxPyramid pyr,
                                                          int *__restrict__ list, int *__restrict__ count,
                                                          const uint8_t *__restrict__ sat) {
    __shared__ Pose q;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < 12) {
        float v;
        if (P.dpose) v = tid < 9 ? P.dpose->R_inv[tid] : P.dpose->t[tid - 9];
        else v = tid < 9 ? P.R_inv[tid] : P.t[tid - 9];
        if (tid < 9) q.Ri[tid] = v; else q.t[tid - 9] = v;
    }
    __syncthreads();
    const tde_point3i &Nv = P.rb.voxels_size;
    const int nbx = (Nv.x + kBrick - 1) / kBrick, nby = (Nv.y + kBrick - 1) / kBrick, nbz = (Nv.z + kBrick - 1) / kBrick;
    const int b = blockIdx.x * blockDim.x + tid;
    bool keep = false;
    if (b < nbx * nby * nbz)
        keep = !brick_culled<COLOR>(P, q, pyr, b % nbx, (b / nbx) % nby, b / (nbx * nby), sat && sat[b] != 0);
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) list[base + __popc(m & ((1u << lane) - 1u))] = b;
}

// Voxels a lane projects and loads together, and the blocks per SM the
// registers are sized for.
constexpr int kIntGroup = 4;
constexpr int kIntBlocksPerSM = 4;

// One warp per surviving brick (16 voxels per lane), grid-strided over the
// list so the work spreads over every SM whatever the scene's layout.
template <int FMT>
__global__ void __launch_bounds__(256, kIntBlocksPerSM) integrate_bricks_kernel(const float *__restrict__ depth, void *__restrict__ vol,
                                                               const IntegrateParams P, const int *__restrict__ list,
                                                               const int *__restrict__ count,
                                                               uint8_t *__restrict__ neg_flags,
                                                               unsigned long long *__restrict__ stats,
                                                               uint8_t *__restrict__ sat) {
    __shared__ Pose q;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < 12) {
        float v;
        if (P.dpose) v = tid < 9 ? P.dpose->R_inv[tid] : P.dpose->t[tid - 9];
        else v = tid < 9 ? P.R_inv[tid] : P.t[tid - 9];
        if (tid < 9) q.Ri[tid] = v; else q.t[tid - 9] = v;
    }
    __syncthreads();
    const tde_point3i &Nv = P.rb.voxels_size;
    const int nbx = (Nv.x + kBrick - 1) / kBrick, nby = (Nv.y + kBrick - 1) / kBrick;
    const size_t nbricks_all = (size_t)nbx * nby * ((Nv.z + kBrick - 1) / kBrick);
    typedef TsdfStore<FMT> S;
    const float ntrunc = -P.trunc, itrunc = __frcp_rn(P.trunc);
    const int W = P.intr.cols, H = P.intr.rows;
    const float fx = P.intr.fx, fy = P.intr.fy, ccx = P.intr.cx, ccy = P.intr.cy;
    const int n_list = *count;
    const int gwarp = (blockIdx.x * blockDim.x + tid) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned n_read = 0, n_written = 0;
    const int NxNy = Nv.x * Nv.y;
    const typename S::Raw sat_raw = S::encode(1.f, P.max_weight);  // f = 1 at the maximum weight
    for (int i = gwarp; i < n_list; i += nwarps) {
        const int b = list[i];
        const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
        const int x = bx * kBrick + (lane & 7);
        const float gx = ((float)x + 0.5f) * P.cell.x - q.t[0];
        // A lane's 16 voxels share x and take two y values: the x and y parts
        // of the projection sums, of the squared distance and of the address
        // are formed once, as the leading terms of the same left-to-right
        // sums (identical bits).
        float pvx[2], pvy[2], pvz[2], pn2[2];
        int pxy[2], py_[2];
        const int px = wrap_mod(x + P.rb.origin_GRID.x, Nv.x);
        #pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int y = by * kBrick + (lane >> 3) + 4 * h;
            const float gy = ((float)y + 0.5f) * P.cell.y - q.t[1];
            pvx[h] = __fmaf_rn(q.Ri[1], gy, __fmul_rn(q.Ri[0], gx));
            pvy[h] = __fmaf_rn(q.Ri[4], gy, __fmul_rn(q.Ri[3], gx));
            pvz[h] = __fmaf_rn(q.Ri[7], gy, __fmul_rn(q.Ri[6], gx));
            pn2[h] = __fmaf_rn(gy, gy, __fmul_rn(gx, gx));
            py_[h] = y;
            pxy[h] = Nv.x * wrap_mod(y + P.rb.origin_GRID.y, Nv.y) + px;
        }
        bool all_sat = true;    // every voxel this lane updated was left saturated
        unsigned taken = 0u;    // bit j: voxel j of this lane was updated; bit 16 + j: written negative
        #pragma unroll 1
        for (int j0 = 0; j0 < 16; j0 += kIntGroup) {
            size_t idx[kIntGroup];
            float sdfv[kIntGroup];
            bool take[kIntGroup];

            #pragma unroll
            for (int k = 0; k < kIntGroup; ++k) {
                const int j = j0 + k;
                const int h = j & 1;
                const int y = py_[h];
                const int z = bz * kBrick + (j >> 1);
                take[k] = false; sdfv[k] = 0.f; idx[k] = 0;
                if (x >= Nv.x || y >= Nv.y || z >= Nv.z) continue;
                const float gz = ((float)z + 0.5f) * P.cell.z - q.t[2];
                const float vx = __fmaf_rn(q.Ri[2], gz, pvx[h]);
                const float vy = __fmaf_rn(q.Ri[5], gz, pvy[h]);
                const float vz = __fmaf_rn(q.Ri[8], gz, pvz[h]);
                if (!(vz > 0.f)) continue;
                const float iz = __frcp_rn(vz);
                const int u = __float2int_rn(__fmaf_rn(vx, __fmul_rn(fx, iz), ccx));
                const int v = __float2int_rn(__fmaf_rn(vy, __fmul_rn(fy, iz), ccy));
                if (u < 0 || u >= W || v < 0 || v >= H) continue;
                const float Dp = __ldg(depth + (size_t)v * W + u);
                if (Dp == 0.f) continue;
                const float sdf = Dp - __fsqrt_rn(__fmaf_rn(gz, gz, pn2[h]));
                if (!(sdf >= ntrunc)) continue;
                take[k] = true;
                sdfv[k] = sdf;
                // voxel_address with the x and y parts above
                size_t a = (size_t)(long)(NxNy * wrap_mod(z + P.rb.origin_GRID.z, Nv.z) + pxy[h]);
                a += (size_t)(long)P.rb.start_index;
                if (a > (size_t)(long)P.rb.buffer_length) a %= (size_t)(long)P.rb.buffer_length;
                idx[k] = a;
            }
            typename S::Raw raw[kIntGroup];
            #pragma unroll
            for (int k = 0; k < kIntGroup; ++k)
                if (take[k]) raw[k] = S::load_raw(vol, idx[k], P.n);
            #pragma unroll
            for (int k = 0; k < kIntGroup; ++k) {
                if (!take[k]) continue;
                taken |= 1u << (j0 + k);
                ++n_read;
                float fo;
                int wo;
                S::decode(raw[k], fo, wo);
                const float tsdf = fminf(1.f, __fmul_rn(sdfv[k], itrunc));
                const float fw = (float)wo;
                // running mean as an increment: f = tsdf (free space at 1) is a fixed point
                const float fnew = __fmaf_rn(tsdf - fo, __frcp_rn(fw + 1.f), fo);
                const int wnew = min(wo + 1, P.max_weight);
                const typename S::Raw rn = S::encode(fnew, wnew);
                all_sat = all_sat && S::same(rn, sat_raw);
                if (!S::same(rn, raw[k])) {
                    S::store_raw(vol, idx[k], P.n, rn);
                    ++n_written;
                    if (neg_flags) {
                        float fs;
                        int ws;
                        S::decode(rn, fs, ws);
                        if (fs < 0.f) taken |= 1u << (16 + j0 + k);
                    }
                }
            }
        }
        if (unsigned negm = taken >> 16) {
            // brick / super-brick flags of the negative writes: the brick's
            // voxels fall in at most two physical bricks per axis, so each flag
            // is stored once (physical_brick / physical_superbrick in 32 bits)
            unsigned last_pb = ~0u, last_ps = ~0u;
            do {
                const int j = __ffs(negm) - 1;
                negm &= negm - 1u;
                const unsigned py = wrap_mod(py_[j & 1] + P.rb.origin_GRID.y, Nv.y);
                const unsigned pz = wrap_mod(bz * kBrick + (j >> 1) + P.rb.origin_GRID.z, Nv.z);
                const unsigned pb = ((unsigned)px >> 3) + ((unsigned)(Nv.x + 7) >> 3) *
                                    ((py >> 3) + ((unsigned)(Nv.y + 7) >> 3) * (pz >> 3));
                const unsigned ps = ((unsigned)px >> 5) + ((unsigned)(Nv.x + 31) >> 5) *
                                    ((py >> 5) + ((unsigned)(Nv.y + 31) >> 5) * (pz >> 5));
                if (pb != last_pb) { neg_flags[pb] = 1; last_pb = pb; }
                if (ps != last_ps) { neg_flags[nbricks_all + ps] = 1; last_ps = ps; }
            } while (negm);
        }
        if (sat) {
            // Saturated brick: every voxel at f = 1, maximum weight.  Only when
            // all updated voxels are, the others (depth dropouts, outside the
            // image) are read to check them too.
            bool brick_sat = __all_sync(0xffffffffu, all_sat);
            if (brick_sat) {
                bool rest = true;
                #pragma unroll 1
                for (int j = 0; j < 16; ++j) {
                    if (taken & (1u << j)) continue;
                    const int h = j & 1, z = bz * kBrick + (j >> 1);
                    if (x >= Nv.x || py_[h] >= Nv.y || z >= Nv.z) { rest = false; break; }
                    size_t a = (size_t)(long)(NxNy * wrap_mod(z + P.rb.origin_GRID.z, Nv.z) + pxy[h]);
                    a += (size_t)(long)P.rb.start_index;
                    if (a > (size_t)(long)P.rb.buffer_length) a %= (size_t)(long)P.rb.buffer_length;
                    if (!S::same(S::load_raw(vol, a, P.n), sat_raw)) { rest = false; break; }
                }
                brick_sat = __all_sync(0xffffffffu, rest);
            }
            if (lane == 0) sat[b] = brick_sat ? 1 : 0;
        }
    }
    if (stats) {
        unsigned r = n_read, w = n_written;
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r += __shfl_down_sync(0xffffffffu, r, off);
            w += __shfl_down_sync(0xffffffffu, w, off);
        }
        if (lane == 0 && (r | w)) {
            atomicAdd(stats, (unsigned long long)r);
            atomicAdd(stats + 1, (unsigned long long)w);
        }
        if (blockIdx.x == 0 && tid == 0) atomicAdd(stats + 2, (unsigned long long)n_list);
    }
}

// Distance of each model surface point (raycast vertex map, volume frame)
// from the camera centre; 0 where the map holds no point.
__global__ void model_dist_kernel(const float *__restrict__ vmap, int n, const IntegrateParams P,
                                  float *__restrict__ dist) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float tx = P.dpose ? P.dpose->t[0] : P.t[0], ty = P.dpose ? P.dpose->t[1] : P.t[1],
                tz = P.dpose ? P.dpose->t[2] : P.t[2];
    const float x = vmap[3 * i], y = vmap[3 * i + 1], z = vmap[3 * i + 2];
    float d = 0.f;
    if (!isnan(x)) d = sqrtf((x - tx) * (x - tx) + (y - ty) * (y - ty) + (z - tz) * (z - tz));
    dist[i] = d;
}

// Colour integration of the surviving bricks, one warp per brick: the same
// voxel test and running mean, in the same IEEE operations, as the oracle.
__global__ void __launch_bounds__(256) integrate_colors_kernel(const uint8_t *__restrict__ rgb,
                                                               const float *__restrict__ vmap,
                                                               tde_color *__restrict__ col, const IntegrateParams P,
                                                               const int *__restrict__ list,
                                                               const int *__restrict__ count,
                                                               unsigned long long *__restrict__ updated) {
    __shared__ Pose q;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < 12) {
        float v;
        if (P.dpose) v = tid < 9 ? P.dpose->R_inv[tid] : P.dpose->t[tid - 9];
        else v = tid < 9 ? P.R_inv[tid] : P.t[tid - 9];
        if (tid < 9) q.Ri[tid] = v; else q.t[tid - 9] = v;
    }
    __syncthreads();
    const tde_point3i &Nv = P.rb.voxels_size;
    const int nbx = (Nv.x + kBrick - 1) / kBrick, nby = (Nv.y + kBrick - 1) / kBrick;
    const int W = P.intr.cols, H = P.intr.rows;
    const int mw = min(P.max_weight, 255);
    const int n_list = *count;
    const int gwarp = (blockIdx.x * blockDim.x + tid) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned n_up = 0;
    for (int i = gwarp; i < n_list; i += nwarps) {
        const int b = list[i];
        const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
        const int x = bx * kBrick + (lane & 7);
        const float ax = ((float)x + 0.5f) * P.cell.x;
        const float gx = ax - q.t[0];
        #pragma unroll 2
        for (int j = 0; j < 16; ++j) {
            const int y = by * kBrick + (lane >> 3) + 4 * (j & 1);
            const int z = bz * kBrick + (j >> 1);
            if (x >= Nv.x || y >= Nv.y || z >= Nv.z) continue;
            const float ay = ((float)y + 0.5f) * P.cell.y, az = ((float)z + 0.5f) * P.cell.z;
            const float gy = ay - q.t[1], gz = az - q.t[2];
            float vx = 0.f; vx += q.Ri[0] * gx; vx += q.Ri[1] * gy; vx += q.Ri[2] * gz;
            float vy = 0.f; vy += q.Ri[3] * gx; vy += q.Ri[4] * gy; vy += q.Ri[5] * gz;
            float vz = 0.f; vz += q.Ri[6] * gx; vz += q.Ri[7] * gy; vz += q.Ri[8] * gz;
            if (!(vz > 0.f)) continue;
            const int u = __float2int_rn(vx * P.intr.fx / vz + P.intr.cx);
            const int v = __float2int_rn(vy * P.intr.fy / vz + P.intr.cy);
            if (u < 0 || u >= W || v < 0 || v >= H) continue;
            const size_t pix = (size_t)v * W + u;
            const float px = __ldg(vmap + 3 * pix);
            if (isnan(px)) continue;
            const float dx = px - ax, dy = __ldg(vmap + 3 * pix + 1) - ay, dz = __ldg(vmap + 3 * pix + 2) - az;
            float d2 = 0.f; d2 += dx * dx; d2 += dy * dy; d2 += dz * dz;
            if (!(sqrtf(d2) < P.trunc)) continue;
            tde_color *c = col + voxel_address(x, y, z, P.rb);
            const tde_color o = *c;
            const uint8_t *src = rgb + 3 * pix;
            const float fw = (float)o.w, fw1 = fw + 1.f;
            tde_color nc;
            nc.r = (uint8_t)max(0, min(255, __float2int_rn(((float)o.r * fw + (float)__ldg(src)) / fw1)));
            nc.g = (uint8_t)max(0, min(255, __float2int_rn(((float)o.g * fw + (float)__ldg(src + 1)) / fw1)));
            nc.b = (uint8_t)max(0, min(255, __float2int_rn(((float)o.b * fw + (float)__ldg(src + 2)) / fw1)));
            nc.w = (uint8_t)min((int)o.w + 1, mw);
            *c = nc;
            ++n_up;
        }
    }
    if (updated) {
        for (int off = 16; off > 0; off >>= 1) n_up += __shfl_down_sync(0xffffffffu, n_up, off);
        if (lane == 0 && n_up) atomicAdd(updated, (unsigned long long)n_up);
    }
}

}  // namespace

size_t depth_max_floats(int W, int H) {
    size_t n = 0;
    for (int l = 0; l < kDepthMaxLevels; ++l) {
        const int t = 16 << l;
        n += (size_t)((W + t - 1) / t) * ((H + t - 1) / t);
    }
    return n;
}

// The max pyramid, then the min pyramid (same layout).
DepthMaxPyramid depth_max_layout(float *base, int W, int H) {
    DepthMaxPyramid p;
    const size_t n = depth_max_floats(W, H);
    size_t off = 0;
    for (int l = 0; l < kDepthMaxLevels; ++l) {
        const int t = 16 << l;
        p.tiles_x[l] = (W + t - 1) / t;
        p.level[l] = base + off;
        p.level_min[l] = base + n + off;
        off += (size_t)p.tiles_x[l] * ((H + t - 1) / t);
    }
    return p;
}

int launch_depth_max(const float *depth_scaled, int W, int H, float *scratch, cudaStream_t stream) {
    DepthMaxPyramid pyr = depth_max_layout(scratch, W, H);
    // levels >= 1 are atomicMax / atomicMin targets: start them at +0 / kNoDepth
    const size_t l0 = (size_t)pyr.tiles_x[0] * ((H + 15) / 16), n = depth_max_floats(W, H);
    cudaError_t e = cudaMemsetAsync(scratch + l0, 0, (n - l0) * sizeof(float), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + n + l0, 0x7f, (n - l0) * sizeof(float), stream);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "depth_max: %s", cudaGetErrorString(e));
    dim3 grid(div_up(W, 16), div_up(H, 16));
    depth_max_kernel<<<grid, 256, 0, stream>>>(depth_scaled, W, H, pyr);
    return check_launch("depth_max");
}

size_t brick_count(const tde_round_buffer &rb) {
    return (size_t)((rb.voxels_size.x + kBrick - 1) / kBrick) * ((rb.voxels_size.y + kBrick - 1) / kBrick) *
           ((rb.voxels_size.z + kBrick - 1) / kBrick);
}

size_t superbrick_count(const tde_round_buffer &rb) {
    return (size_t)((rb.voxels_size.x + 31) / 32) * ((rb.voxels_size.y + 31) / 32) * ((rb.voxels_size.z + 31) / 32);
}

size_t integrate_scratch_bytes(int W, int H, const tde_round_buffer &rb) {
    // depth max and min pyramids, then (aligned) the brick counter and the brick list
    const size_t dm = ((2 * depth_max_floats(W, H) * sizeof(float)) + 255) & ~size_t(255);
    return dm + 256 + brick_count(rb) * sizeof(int);
}

int launch_integrate(const float *depth_scaled, void *volume, int format, const IntegrateParams &P, void *scratch,
                     uint8_t *neg_flags, unsigned long long *stats, cudaStream_t stream, uint8_t *sat_flags) {
    const int W = P.intr.cols, H = P.intr.rows;
    float *dmax = static_cast<float *>(scratch);
    const size_t dm = ((2 * depth_max_floats(W, H) * sizeof(float)) + 255) & ~size_t(255);
    int *count = reinterpret_cast<int *>(static_cast<char *>(scratch) + dm);
    int *list = reinterpret_cast<int *>(static_cast<char *>(scratch) + dm + 256);
    const DepthMaxPyramid pyr = depth_max_layout(dmax, W, H);
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), stream);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "integrate: %s", cudaGetErrorString(e));
    const unsigned nb = (unsigned)brick_count(P.rb);
    cull_bricks_kernel<<<div_up(nb, 256u), 256, 0, stream>>>(P, pyr, list, count, sat_flags);
    int st = check_launch("integrate/cull");
    if (st) return st;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one resident wave (measured at 640x480 / 512^3: 4 blocks per SM
    // 0.0655 ms, 6: 0.0696, 8: 0.0658, 12: 0.0658)
    const unsigned blocks = std::min(div_up(nb, 8u), (unsigned)(sms * kIntBlocksPerSM));
    return dispatch_format(format, [&](auto F) {
        integrate_bricks_kernel<decltype(F)::value><<<blocks, 256, 0, stream>>>(depth_scaled, volume, P, list, count,
                                                                               neg_flags, stats, sat_flags);
        return check_launch("integrate_tsdf");
    });
}

size_t integrate_colors_scratch_bytes(int W, int H, const tde_round_buffer &rb) {
    return (((size_t)W * H * sizeof(float) + 255) & ~size_t(255)) + integrate_scratch_bytes(W, H, rb);
}

int launch_integrate_colors(tde_color *col, const uint8_t *rgb, const float *vmap, const IntegrateParams &P,
                            void *scratch, unsigned long long *updated, cudaStream_t stream) {
    const int W = P.intr.cols, H = P.intr.rows, n = W * H;
    float *dist = static_cast<float *>(scratch);
    char *iscratch = static_cast<char *>(scratch) + (((size_t)n * sizeof(float) + 255) & ~size_t(255));
    model_dist_kernel<<<div_up(n, 256), 256, 0, stream>>>(vmap, n, P, dist);
    int st = check_launch("integrate_colors/model distances");
    if (st) return st;
    if ((st = launch_depth_max(dist, W, H, reinterpret_cast<float *>(iscratch), stream))) return st;
    const size_t dm = ((2 * depth_max_floats(W, H) * sizeof(float)) + 255) & ~size_t(255);
    int *count = reinterpret_cast<int *>(iscratch + dm);
    int *list = reinterpret_cast<int *>(iscratch + dm + 256);
    const DepthMaxPyramid pyr = depth_max_layout(reinterpret_cast<float *>(iscratch), W, H);
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), stream);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "integrate_colors: %s", cudaGetErrorString(e));
    const unsigned nb = (unsigned)brick_count(P.rb);
    cull_bricks_kernel<true><<<div_up(nb, 256u), 256, 0, stream>>>(P, pyr, list, count, nullptr);
    if ((st = check_launch("integrate_colors/cull"))) return st;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned blocks = std::min(div_up(nb, 8u), (unsigned)sms * 8u);
    integrate_colors_kernel<<<blocks, 256, 0, stream>>>(rgb, vmap, col, P, list, count, updated);
    return check_launch("integrate_colors");
}

}  // namespace tde
