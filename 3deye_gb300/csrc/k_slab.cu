// k_slab.cu -- cyclic-volume slab extraction and slab cleaning.
//
// Extract_Slice (common/src/opencl_wrappers.cpp:856-964) runs, per z chunk, a
// predicate scan (scan_slice_of_both_volumes.cl:76-208), an exclusive prefix
// sum and a scatter (extract_slice_as_cloud.cl:72-201).  The output order is
// therefore: chunk, then plane (+x, +y, +z, colour), then (z, y, x) raster.
//
// Here the same order is produced in three launches over "tiles" -- TY rows
// of one z slice, contiguous in raster order:
//   1. count:   per tile and plane, the number of set predicates;
//   2. scan:    one exclusive scan over counts laid out (chunk, plane, tile);
//   3. scatter: predicates recomputed, ranked inside the tile with warp
//               ballots, and written at offset + rank.
// Tiles that cannot intersect the black zone exit at once, so the cost
// follows the slab, not the volume.  All indexing is integer: the output is
// bit-identical to the reference on the scan's predicate set.
#include "tde_common.cuh"
#include "tde_slab.cuh"

namespace tde {
namespace {

constexpr int kSlabThreads = 256;

struct SlabParams {
    const void *vol;
    const tde_color *color;
    tde_round_buffer rb;
    tde_point3i mn, mx;
    size_t n;
    int step;            // chunk depth
    int ty;              // rows per tile
    int tiles_per_z;     // ceil(H / ty)
    int tiles_per_chunk; // step * tiles_per_z
    int metric;          // points as metric voxel centres (x + 0.5) * cell
    tde_point3f cell;
};

__device__ __forceinline__ bool color_set(tde_color c) { return (c.r | c.g | c.b | c.w) != 0; }

// F != 1 and W != 0 test of the reference (raw float compare after decode).
template <int FMT>
__device__ __forceinline__ void fetch(const SlabParams &p, int x, int y, int z, float &f, int &w) {
    typedef TsdfStore<FMT> S;
    S::decode(S::load_raw(p.vol, voxel_address(x, y, z, p.rb), p.n), f, w);
}
__device__ __forceinline__ bool crossing(float F, float Fn, int Wn) {
    return (Wn != 0 && Fn != 1.f) && ((F > 0 && Fn < 0) || (F < 0 && Fn > 0));
}

// Predicate bits of one voxel: bit0 +x, bit1 +y, bit2 +z, bit3 colour.
template <int FMT>
__device__ __forceinline__ unsigned predicates(const SlabParams &p, int x, int y, int z, int z_end) {
    if (!in_black_zone(x, y, z, p.mn, p.mx, p.rb)) return 0u;
    unsigned bits = 0;
    const int Wd = p.rb.voxels_size.x, Hd = p.rb.voxels_size.y;
    float F; int Wt;
    fetch<FMT>(p, x, y, z, F, Wt);
    if (Wt != 0 && F != 1.f) {
        float Fn; int Wn;
        if (x + 1 < Wd) { fetch<FMT>(p, x + 1, y, z, Fn, Wn); if (crossing(F, Fn, Wn)) bits |= 1u; }
        if (y + 1 < Hd) { fetch<FMT>(p, x, y + 1, z, Fn, Wn); if (crossing(F, Fn, Wn)) bits |= 2u; }
        if (z + 1 < z_end) { fetch<FMT>(p, x, y, z + 1, Fn, Wn); if (crossing(F, Fn, Wn)) bits |= 4u; }
    }
    if (p.color && color_set(p.color[voxel_address(x, y, z, p.rb)])) bits |= 8u;
    return bits;
}

// Tile -> (chunk, z, y0); returns false when the tile cannot touch the zone.
__device__ __forceinline__ bool tile_coords(const SlabParams &p, int tile, int &chunk, int &z, int &y0, int &y1) {
    chunk = tile / p.tiles_per_chunk;
    int r = tile - chunk * p.tiles_per_chunk;
    int zl = r / p.tiles_per_z;
    int ti = r - zl * p.tiles_per_z;
    z = chunk * p.step + zl;
    y0 = ti * p.ty;
    y1 = min(y0 + p.ty, p.rb.voxels_size.y);
    const tde_round_buffer &rb = p.rb;
    int ix0 = rb.origin_GRID.x, ix1 = rb.origin_GRID.x + rb.voxels_size.x - 1;
    int iy0 = y0 + rb.origin_GRID.y, iy1 = y1 - 1 + rb.origin_GRID.y;
    int iz = z + rb.origin_GRID.z;
    bool hx = !(ix1 < p.mn.x || ix0 > p.mx.x);
    bool hy = !(iy1 < p.mn.y || iy0 > p.mx.y);
    bool hz = iz >= p.mn.z && iz <= p.mx.z;
    return hx || hy || hz;
}

template <int FMT>
__global__ void __launch_bounds__(kSlabThreads) slab_count_kernel(const SlabParams p, uint32_t *__restrict__ counts) {
    __shared__ unsigned s_cnt[4];
    const int tile = blockIdx.x;
    int chunk, z, y0, y1;
    const bool live = tile_coords(p, tile, chunk, z, y0, y1);
    const int W = p.rb.voxels_size.x;
    const int z_end = (chunk + 1) * p.step;
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    unsigned c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    if (live) {
        const int nvox = (y1 - y0) * W;
        for (int r = threadIdx.x; r < nvox; r += kSlabThreads) {
            int y = y0 + r / W, x = r - (r / W) * W;
            unsigned b = predicates<FMT>(p, x, y, z, z_end);
            c0 += b & 1u; c1 += (b >> 1) & 1u; c2 += (b >> 2) & 1u; c3 += (b >> 3) & 1u;
        }
    }
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        c0 += __shfl_down_sync(0xffffffffu, c0, off);
        c1 += __shfl_down_sync(0xffffffffu, c1, off);
        c2 += __shfl_down_sync(0xffffffffu, c2, off);
        c3 += __shfl_down_sync(0xffffffffu, c3, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c0) atomicAdd(&s_cnt[0], c0);
        if (c1) atomicAdd(&s_cnt[1], c1);
        if (c2) atomicAdd(&s_cnt[2], c2);
        if (c3) atomicAdd(&s_cnt[3], c3);
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int tin = tile - chunk * p.tiles_per_chunk;
        counts[(size_t)(chunk * 4 + threadIdx.x) * p.tiles_per_chunk + tin] = s_cnt[threadIdx.x];
    }
}

// Exclusive scan of n counts in place (one block of 1024 threads); the total
// goes to *total.
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(uint32_t *__restrict__ a, int n,
                                                              uint32_t *__restrict__ total) {
    __shared__ uint32_t warp_sums[32];
    const int tid = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int b = tid * per, e = min(n, b + per);
    uint32_t s = 0;
    for (int i = b; i < e; ++i) s += a[i];
    // block exclusive scan of s
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t v = s;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += o;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t o = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += o;
        }
        warp_sums[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    uint32_t base = (warp ? warp_sums[warp - 1] : 0u) + v - s;
    for (int i = b; i < e; ++i) { uint32_t c = a[i]; a[i] = base; base += c; }
    if (tid == 1023) *total = warp_sums[31];
}

template <int FMT>
__global__ void __launch_bounds__(kSlabThreads) slab_scatter_kernel(const SlabParams p, const uint32_t *__restrict__ offs,
                                                                   tde_xyzi *__restrict__ pts, tde_color *__restrict__ cols,
                                                                   float *__restrict__ wts, uint32_t capacity) {
    __shared__ unsigned s_warp[4][kSlabThreads / 32];
    __shared__ unsigned s_base[4];
    const int tile = blockIdx.x;
    int chunk, z, y0, y1;
    if (!tile_coords(p, tile, chunk, z, y0, y1)) return;
    const int W = p.rb.voxels_size.x;
    const int z_end = (chunk + 1) * p.step;
    const int tin = tile - chunk * p.tiles_per_chunk;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < 4) s_base[threadIdx.x] = offs[(size_t)(chunk * 4 + threadIdx.x) * p.tiles_per_chunk + tin];
    __syncthreads();
    const int nvox = (y1 - y0) * W;
    const unsigned lt = (1u << lane) - 1u;
    for (int r0 = 0; r0 < nvox; r0 += kSlabThreads) {
        const int r = r0 + threadIdx.x;
        unsigned bits = 0;
        int x = 0, y = 0;
        if (r < nvox) {
            y = y0 + r / W; x = r - (r / W) * W;
            bits = predicates<FMT>(p, x, y, z, z_end);
        }
        unsigned m[4], rank[4];
        #pragma unroll
        for (int q = 0; q < 4; ++q) {
            m[q] = __ballot_sync(0xffffffffu, (bits >> q) & 1u);
            rank[q] = __popc(m[q] & lt);
            if (lane == 0) s_warp[q][warp] = __popc(m[q]);
        }
        __syncthreads();
        #pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (!((bits >> q) & 1u)) continue;
            unsigned before = 0;
            for (int w2 = 0; w2 < warp; ++w2) before += s_warp[q][w2];
            const uint32_t slot = s_base[q] + before + rank[q];
            if (slot >= capacity) continue;
            const int dx = q == 0, dy = q == 1, dz = q == 2;
            const int nx = x + dx, ny = y + dy, nz = z + dz;
            float px = (float)nx, py = (float)ny, pz = (float)nz;
            if (p.metric) {
                px = __fmul_rn(__fadd_rn(px, 0.5f), p.cell.x);
                py = __fmul_rn(__fadd_rn(py, 0.5f), p.cell.y);
                pz = __fmul_rn(__fadd_rn(pz, 0.5f), p.cell.z);
            }
            pts[slot] = tde_xyzi{px, py, pz, 1.0f};
            const size_t a = voxel_address(nx, ny, nz, p.rb);
            if (cols) cols[slot] = p.color ? p.color[a] : tde_color{0, 0, 0, 0};
            if (wts) {
                float f; int w;
                TsdfStore<FMT>::decode(TsdfStore<FMT>::load_raw(p.vol, a, p.n), f, w);
                wts[slot] = (float)w;
            }
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            unsigned tot = 0;
            for (int w2 = 0; w2 < kSlabThreads / 32; ++w2) tot += s_warp[threadIdx.x][w2];
            s_base[threadIdx.x] += tot;
        }
        __syncthreads();
    }
}

template <int FMT>
__global__ void clean_tsdf_kernel(void *__restrict__ vol, const tde_point3i mn, const tde_point3i mx,
                                  const tde_round_buffer rb, size_t n) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= rb.voxels_size.x || y >= rb.voxels_size.y) return;
    const int ix = x + rb.origin_GRID.x, iy = y + rb.origin_GRID.y;
    const bool whole = (ix >= mn.x && ix <= mx.x) || (iy >= mn.y && iy <= mx.y);
    int z0 = 0, z1 = rb.voxels_size.z - 1;
    if (!whole) { z0 = max(z0, mn.z - rb.origin_GRID.z); z1 = min(z1, mx.z - rb.origin_GRID.z); }
    for (int z = z0; z <= z1; ++z) TsdfStore<FMT>::clear(vol, voxel_address(x, y, z, rb), n);
}

// clean_color_slice.cl:41-67
__global__ void clean_color_kernel(tde_color *__restrict__ col, const tde_point3i mn, const tde_point3i mx,
                                   const tde_round_buffer rb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= rb.voxels_size.x || y >= rb.voxels_size.y) return;
    const int ix = x + rb.origin_GRID.x, iy = y + rb.origin_GRID.y;
    const bool whole = (ix >= mn.x && ix <= mx.x) || (iy >= mn.y && iy <= mx.y);
    int z0 = 0, z1 = rb.voxels_size.z - 1;
    if (!whole) { z0 = max(z0, mn.z - rb.origin_GRID.z); z1 = min(z1, mx.z - rb.origin_GRID.z); }
    for (int z = z0; z <= z1; ++z) col[voxel_address(x, y, z, rb)] = tde_color{0, 0, 0, 0};
}

// Extract_Color_Volume (opencl_wrappers.cpp:545-581, kernel extract_colors
// absent): the voxel holding a metric point is floor(p / cell) per axis
// (correctly rounded division); points outside the volume get zero colour.
__global__ void gather_colors_kernel(const tde_color *__restrict__ color, const tde_round_buffer rb,
                                     const tde_xyzi *__restrict__ pts, uint32_t n, tde_point3f cell,
                                     tde_color *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const tde_xyzi q = pts[i];
    const float fx = floorf(__fdiv_rn(q.x, cell.x)), fy = floorf(__fdiv_rn(q.y, cell.y)),
                fz = floorf(__fdiv_rn(q.z, cell.z));
    tde_color c = {0, 0, 0, 0};
    // NaN fails every comparison
    if (fx >= 0.f && fy >= 0.f && fz >= 0.f && fx < (float)rb.voxels_size.x && fy < (float)rb.voxels_size.y &&
        fz < (float)rb.voxels_size.z)
        c = color[voxel_address((int)fx, (int)fy, (int)fz, rb)];
    out[i] = c;
}

void slab_geometry(const tde_round_buffer &rb, SlabParams &p) {
    const int W = rb.voxels_size.x, H = rb.voxels_size.y;
    p.ty = max(1, min(H, 8192 / max(1, W)));
    p.tiles_per_z = (H + p.ty - 1) / p.ty;
    p.tiles_per_chunk = p.step * p.tiles_per_z;
}

}  // namespace

int slab_chunk_depth(int depth, int divisor) {
    unsigned step = 0, n = 0;
    if (tde_determine_extract_step((unsigned)depth, divisor, &step, &n) == TDE_OK) return (int)step;
    // depths outside the reference's table: 64-voxel chunks when they divide it
    if (depth % 64 == 0) return 64;
    return depth;
}

// chunks * 4 planes * (step * tiles_per_z) counts = 4 * depth * tiles_per_z:
// the same for every chunk depth that divides the volume depth.
size_t slab_scratch_bytes(const tde_round_buffer &rb) {
    SlabParams p;
    p.step = slab_chunk_depth(rb.voxels_size.z, 4);
    slab_geometry(rb, p);
    const size_t chunks = (size_t)rb.voxels_size.z / p.step;
    return (chunks * 4 * (size_t)p.tiles_per_chunk + 64) * sizeof(uint32_t);
}

int launch_extract_slice(const void *vol, int fmt, const tde_color *color, tde_point3i mn, tde_point3i mx,
                         const tde_round_buffer &rb, void *scratch, size_t scratch_bytes, tde_xyzi *pts,
                         tde_color *cols, float *wts, uint32_t capacity, uint32_t *count, int step,
                         const tde_point3f *cell, cudaStream_t stream) {
    SlabParams p;
    p.vol = vol; p.color = color; p.rb = rb; p.mn = mn; p.mx = mx; p.n = voxel_count(rb);
    p.metric = cell != nullptr;
    p.cell = cell ? *cell : tde_point3f{1.f, 1.f, 1.f};
    p.step = step > 0 ? step : slab_chunk_depth(rb.voxels_size.z, 4);
    if (rb.voxels_size.z % p.step)
        return set_error(TDE_ERR_INVALID_ARG, "extract_slice: chunk depth %d does not divide %d", p.step,
                         rb.voxels_size.z);
    slab_geometry(rb, p);
    const int chunks = rb.voxels_size.z / p.step;
    const int ntiles = chunks * p.tiles_per_chunk;
    const int ncounts = ntiles * 4;
    if (scratch_bytes < slab_scratch_bytes(rb))
        return set_error(TDE_ERR_INVALID_ARG, "extract_slice: scratch %zu < %zu bytes", scratch_bytes,
                         slab_scratch_bytes(rb));
    uint32_t *counts = reinterpret_cast<uint32_t *>(scratch);
    return dispatch_format(fmt, [&](auto F) {
        constexpr int FMT = decltype(F)::value;
        slab_count_kernel<FMT><<<ntiles, kSlabThreads, 0, stream>>>(p, counts);
        int st = check_launch("extract_slice/count");
        if (st) return st;
        exclusive_scan_kernel<<<1, 1024, 0, stream>>>(counts, ncounts, count);
        st = check_launch("extract_slice/scan");
        if (st) return st;
        slab_scatter_kernel<FMT><<<ntiles, kSlabThreads, 0, stream>>>(p, counts, pts, cols, wts, capacity);
        return check_launch("extract_slice/scatter");
    });
}

int launch_gather_colors(const tde_color *color, const tde_round_buffer &rb, const tde_xyzi *pts, uint32_t n,
                         tde_point3f cell, tde_color *out, cudaStream_t stream) {
    if (!n) return TDE_OK;
    gather_colors_kernel<<<div_up(n, 256u), 256, 0, stream>>>(color, rb, pts, n, cell, out);
    return check_launch("extract_color_volume");
}

int launch_clean_tsdf_slice(void *vol, int fmt, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                            cudaStream_t stream) {
    dim3 block(32, 8), grid(div_up(rb.voxels_size.x, 32), div_up(rb.voxels_size.y, 8));
    return dispatch_format(fmt, [&](auto F) {
        clean_tsdf_kernel<decltype(F)::value><<<grid, block, 0, stream>>>(vol, mn, mx, rb, voxel_count(rb));
        return check_launch("clean_tsdf_slice");
    });
}

int launch_clean_color_slice(tde_color *col, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                             cudaStream_t stream) {
    dim3 block(32, 8), grid(div_up(rb.voxels_size.x, 32), div_up(rb.voxels_size.y, 8));
    clean_color_kernel<<<grid, block, 0, stream>>>(col, mn, mx, rb);
    return check_launch("clean_color_slice");
}

}  // namespace tde
