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
//   3. scatter: points ranked inside the tile and written at offset + rank.
// Two forms: the row kernels (rows of whole 4-voxel groups: 16-byte loads,
// the count pass stores each group's predicate bits for the scatter, ranks
// from one block scan) and the scalar kernels (any row length: predicates
// recomputed in the scatter, ranked with warp ballots).  Tiles that cannot
// intersect the black zone exit at once, so the cost follows the slab, not
// the volume; Extract_Tsdf_Volume is the same scan with the whole volume as
// the zone.  All indexing is integer: the output is bit-identical to the
// reference on the scan's predicate set.
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
    uint16_t *gbits;     // row kernels: predicate bits per 4-voxel group, kTileGroups per tile
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
// goes to *total.  Segments of 8192 counts are staged through shared memory
// with coalesced loads and stores; each thread scans 8 adjacent counts.
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(uint32_t *__restrict__ a, int n,
                                                              uint32_t *__restrict__ total) {
    constexpr int kPer = 8, kSeg = 1024 * kPer;
    __shared__ uint32_t buf[kSeg];
    __shared__ uint32_t warp_sums[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t carry = 0;
    for (int base = 0; base < n; base += kSeg) {
        const int m = min(kSeg, n - base);
        for (int i = tid; i < kSeg; i += 1024) buf[i] = i < m ? a[base + i] : 0u;
        __syncthreads();
        uint32_t v[kPer], s = 0;
        #pragma unroll
        for (int k = 0; k < kPer; ++k) { v[k] = buf[tid * kPer + k]; s += v[k]; }
        uint32_t x = s;
        #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += o;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane];
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += o;
            }
            warp_sums[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        uint32_t run = carry + (warp ? warp_sums[warp - 1] : 0u) + x - s;
        #pragma unroll
        for (int k = 0; k < kPer; ++k) { buf[tid * kPer + k] = run; run += v[k]; }
        carry += warp_sums[31];
        __syncthreads();
        for (int i = tid; i < m; i += 1024) a[base + i] = buf[i];
        __syncthreads();
    }
    if (tid == 0) *total = carry;
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

// ---------------------------------------------------------------------------
// Row-vector form of the same count and scatter (volumes with W % 4 == 0,
// 32 <= W, 16-byte aligned buffers).  A thread takes a group of 4 voxels
// that are adjacent in memory -- physical x' = 4k..4k+3 of one row -- with
// one 16-byte load; the +y / +z neighbour groups are loaded only when one of
// the 4 voxels can emit (w != 0, f != 1), the +x neighbour of the last voxel
// only when it can.  Physical order within a row is the logical order
// rotated by origin_GRID.x, so the logical raster rank of a point is its
// physical-order rank rotated about the row's count before x' = ox.  Same
// predicate set, same output order, same bits as the kernels above.
// ---------------------------------------------------------------------------
constexpr int kGroupsPerThread = 8;  // tile = ty * W / 4 <= 2048 groups
constexpr int kTileGroups = kSlabThreads * kGroupsPerThread;

struct Rec4 { float f[4]; int w[4]; };

// Four adjacent records as loaded (one or two vector loads), then decoded.
template <int FMT> struct Raw4 { uint4 v; };
template <> struct Raw4<TDE_TSDF_F32> { float4 f; ushort4 w; };

template <int FMT> __device__ __forceinline__ Raw4<FMT> load_raw4(const void *vol, uint32_t a, size_t) {
    Raw4<FMT> r;
    r.v = __ldg(reinterpret_cast<const uint4 *>(vol) + (a >> 2));
    return r;
}
template <>
__device__ __forceinline__ Raw4<TDE_TSDF_F32> load_raw4<TDE_TSDF_F32>(const void *vol, uint32_t a, size_t n) {
    Raw4<TDE_TSDF_F32> r;
    r.f = __ldg(reinterpret_cast<const float4 *>(vol) + (a >> 2));
    r.w = __ldg(reinterpret_cast<const ushort4 *>(TsdfStore<TDE_TSDF_F32>::wplane(vol, n)) + (a >> 2));
    return r;
}
template <int FMT> __device__ __forceinline__ void decode4(const Raw4<FMT> &r, Rec4 &c) {
    const uint32_t u[4] = {r.v.x, r.v.y, r.v.z, r.v.w};
    #pragma unroll
    for (int i = 0; i < 4; ++i) TsdfStore<FMT>::decode(u[i], c.f[i], c.w[i]);
}
template <> __device__ __forceinline__ void decode4<TDE_TSDF_F32>(const Raw4<TDE_TSDF_F32> &r, Rec4 &c) {
    c.f[0] = r.f.x; c.f[1] = r.f.y; c.f[2] = r.f.z; c.f[3] = r.f.w;
    c.w[0] = r.w.x; c.w[1] = r.w.y; c.w[2] = r.w.z; c.w[3] = r.w.w;
}
template <int FMT> __device__ __forceinline__ void load4(const void *vol, uint32_t a, size_t n, Rec4 &c) {
    decode4<FMT>(load_raw4<FMT>(vol, a, n), c);
}

// 4-bit mask of the group's voxels with w != 0 and f != 1, read from the
// record bits: I16 f == 1 only for v == 32767 (v / 32767 is correctly
// rounded), F16 only for the half 0x3c00; F32 compares the float.
template <int FMT> __device__ __forceinline__ unsigned live_mask(const Raw4<FMT> &r, uint32_t one) {
    const uint32_t u[4] = {r.v.x, r.v.y, r.v.z, r.v.w};
    unsigned m = 0;
    #pragma unroll
    for (int i = 0; i < 4; ++i) m |= (unsigned)((u[i] >> 16) != 0u && (u[i] & 0xffffu) != one) << i;
    return m;
}
template <>
__device__ __forceinline__ unsigned live_mask<TDE_TSDF_F32>(const Raw4<TDE_TSDF_F32> &r, uint32_t) {
    return (unsigned)(r.w.x != 0 && r.f.x != 1.f) | ((unsigned)(r.w.y != 0 && r.f.y != 1.f) << 1) |
           ((unsigned)(r.w.z != 0 && r.f.z != 1.f) << 2) | ((unsigned)(r.w.w != 0 && r.f.w != 1.f) << 3);
}
template <int FMT> struct OneBits { static constexpr uint32_t value = 0x7fffu; };  // I16: v = 32767
template <> struct OneBits<TDE_TSDF_F16> { static constexpr uint32_t value = 0x3c00u; };  // half 1.0
template <> struct OneBits<TDE_TSDF_F32> { static constexpr uint32_t value = 0u; };       // unused

// Per-launch constants of the row kernels.
struct RowGeom {
    uint32_t g_magic;  // ceil(2^32 / G): g / G = umulhi(g, g_magic) for g < 2^16
    int G;             // groups per row, W / 4
    int xlast;         // physical x' of logical x = W - 1 (no +x neighbour)
    int row_stride_z;  // W * H
};

// Group g of a tile starting at logical row y0 of slice z: its row r, group
// k (physical x' = 4k) and the address of its first record.  The volume
// holds fewer than 2^31 voxels, so addresses are 32-bit.
struct GroupAt {
    int r, k;
    int py, pz;   // physical row and slice
    uint32_t a;
};
__device__ __forceinline__ int wrap1(int v, int n) { return v >= n ? v - n : v; }  // v in [0, 2n)
__device__ __forceinline__ GroupAt group_at(const SlabParams &p, const RowGeom &rg, int g, int y0, int z) {
    GroupAt at;
    at.r = (int)__umulhi((unsigned)g, rg.g_magic);
    at.k = g - at.r * rg.G;
    at.py = wrap1(y0 + at.r + p.rb.origin_GRID.y, p.rb.voxels_size.y);
    at.pz = wrap1(z + p.rb.origin_GRID.z, p.rb.voxels_size.z);
    at.a = (uint32_t)(at.pz * rg.row_stride_z + at.py * p.rb.voxels_size.x + 4 * at.k);
    return at;
}

__device__ __forceinline__ unsigned plane_count(unsigned bits, int q) { return __popc(bits & (0x1111u << q)); }

// Predicate bits of the 4 voxels of a group of logical row y, slice z (its
// records and colours already loaded): bit 4*i + q for voxel i (physical
// x' = 4k + i) and plane q.  ZONE = false: every voxel is in the zone.
template <int FMT, bool ZONE, bool COLOR>
__device__ __forceinline__ unsigned group_bits(const SlabParams &p, const RowGeom &rg, const GroupAt &at, int y, int z,
                                               int z_end, const Raw4<FMT> &raw, const uint4 &colour, unsigned lmask) {
    const int W = p.rb.voxels_size.x, H = p.rb.voxels_size.y, D = p.rb.voxels_size.z;
    const int x0 = 4 * at.k;
    bool zone[4] = {true, true, true, true};
    if (ZONE) {
        const int iy = y + p.rb.origin_GRID.y, iz = z + p.rb.origin_GRID.z;
        const bool yz = (iy >= p.mn.y && iy <= p.mx.y) || (iz >= p.mn.z && iz <= p.mx.z);
        int lx0 = x0 - p.rb.origin_GRID.x;
        if (lx0 < 0) lx0 += W;
        #pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int lx = lx0 + i >= W ? lx0 + i - W : lx0 + i;
            const int ix = lx + p.rb.origin_GRID.x;
            zone[i] = yz || (ix >= p.mn.x && ix <= p.mx.x);
        }
    }
    bool live[4], any = false;
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        live[i] = zone[i] && ((lmask >> i) & 1u);
        any |= live[i];
    }
    unsigned bits = 0;
    if (any) {
        Rec4 c;
        decode4<FMT>(raw, c);
        Rec4 ny, nz;
        const bool has_y = y + 1 < H, has_z = z + 1 < z_end;
        const uint32_t row = at.a - (uint32_t)x0;
        if (has_y) load4<FMT>(p.vol, (uint32_t)(at.pz * rg.row_stride_z + wrap1(at.py + 1, H) * W + x0), p.n, ny);
        if (has_z) load4<FMT>(p.vol, (uint32_t)(wrap1(at.pz + 1, D) * rg.row_stride_z + at.py * W + x0), p.n, nz);
        float fx3 = 0.f;
        int wx3 = 0;
        if (live[3] && x0 + 3 != rg.xlast) {
            const int xn = x0 + 4 == W ? 0 : x0 + 4;
            TsdfStore<FMT>::decode(TsdfStore<FMT>::load_raw(p.vol, row + xn, p.n), fx3, wx3);
        }
        #pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (!live[i]) continue;
            if (x0 + i != rg.xlast) {
                const float fn = i < 3 ? c.f[i < 3 ? i + 1 : 3] : fx3;
                const int wn = i < 3 ? c.w[i < 3 ? i + 1 : 3] : wx3;
                if (crossing(c.f[i], fn, wn)) bits |= 1u << (4 * i);
            }
            if (has_y && crossing(c.f[i], ny.f[i], ny.w[i])) bits |= 2u << (4 * i);
            if (has_z && crossing(c.f[i], nz.f[i], nz.w[i])) bits |= 4u << (4 * i);
        }
    }
    if (COLOR) {
        const uint32_t cc[4] = {colour.x, colour.y, colour.z, colour.w};
        #pragma unroll
        for (int i = 0; i < 4; ++i)
            if (zone[i] && cc[i] != 0u) bits |= 8u << (4 * i);
    }
    return bits;
}

// Bits of the groups g = g0 + stride * j (j < kGroupsPerThread) of a tile;
// every record (and colour) load is issued before any is used, and group
// coordinates are recomputed rather than held, to keep registers for loads
// in flight.
template <int FMT, bool ZONE, bool COLOR>
__device__ __forceinline__ void tile_bits(const SlabParams &p, const RowGeom &rg, int y0, int z, int z_end,
                                          int ngroups, int g0, int stride, unsigned (&bits)[kGroupsPerThread]) {
    Raw4<FMT> raw[kGroupsPerThread];
    uint4 colour[COLOR ? kGroupsPerThread : 1];
    #pragma unroll
    for (int j = 0; j < kGroupsPerThread; ++j) {
        const int g = g0 + stride * j;
        if (g < ngroups) {
            const uint32_t a = group_at(p, rg, g, y0, z).a;
            raw[j] = load_raw4<FMT>(p.vol, a, p.n);
            if (COLOR) colour[COLOR ? j : 0] = __ldg(reinterpret_cast<const uint4 *>(p.color) + (a >> 2));
        }
    }
    #pragma unroll
    for (int j = 0; j < kGroupsPerThread; ++j) {
        const int g = g0 + stride * j;
        bits[j] = 0;
        if (g < ngroups) {
            // most groups hold nothing that can emit: no coordinates, no decode
            const unsigned lmask = live_mask<FMT>(raw[j], OneBits<FMT>::value);
            const bool colour_any = COLOR && (colour[COLOR ? j : 0].x | colour[COLOR ? j : 0].y |
                                              colour[COLOR ? j : 0].z | colour[COLOR ? j : 0].w) != 0u;
            if (lmask || colour_any) {
                const GroupAt at = group_at(p, rg, g, y0, z);
                bits[j] = group_bits<FMT, ZONE, COLOR>(p, rg, at, y0 + at.r, z, z_end, raw[j],
                                                       COLOR ? colour[COLOR ? j : 0] : make_uint4(0u, 0u, 0u, 0u),
                                                       lmask);
            }
        }
    }
}

template <int FMT, bool ZONE, bool COLOR>
__global__ void __launch_bounds__(kSlabThreads, 4) row_count_kernel(const SlabParams p, const RowGeom rg,
                                                                uint32_t *__restrict__ counts) {
    __shared__ unsigned s_cnt[4];
    const int tile = blockIdx.x;
    int chunk, z, y0, y1;
    const bool live = tile_coords(p, tile, chunk, z, y0, y1);
    const int z_end = (chunk + 1) * p.step;
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    unsigned c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    if (live) {
        unsigned bits[kGroupsPerThread];
        // coalesced: a warp's j-th loads cover 512 contiguous bytes
        tile_bits<FMT, ZONE, COLOR>(p, rg, y0, z, z_end, (y1 - y0) * rg.G, threadIdx.x, kSlabThreads, bits);
        // the scatter reads these instead of the volume
        uint16_t *tb = p.gbits + (size_t)tile * kTileGroups;
        #pragma unroll
        for (int j = 0; j < kGroupsPerThread; ++j) {
            const unsigned b = bits[j];
            tb[threadIdx.x + kSlabThreads * j] = (uint16_t)b;
            c0 += plane_count(b, 0); c1 += plane_count(b, 1); c2 += plane_count(b, 2); c3 += plane_count(b, 3);
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

// Packed per-plane counts: 16 bits per plane (a tile holds <= 8192 voxels).
__device__ __forceinline__ unsigned long long packed_counts(unsigned bits) {
    return (unsigned long long)plane_count(bits, 0) | ((unsigned long long)plane_count(bits, 1) << 16) |
           ((unsigned long long)plane_count(bits, 2) << 32) | ((unsigned long long)plane_count(bits, 3) << 48);
}
__device__ __forceinline__ int field(unsigned long long v, int q) { return (int)((v >> (16 * q)) & 0xffffu); }

template <int FMT, bool ZONE, bool COLOR>
__global__ void __launch_bounds__(kSlabThreads, 4) row_scatter_kernel(const SlabParams p, const RowGeom rg,
                                                                  const uint32_t *__restrict__ offs,
                                                                  tde_xyzi *__restrict__ pts, tde_color *__restrict__ cols,
                                                                  float *__restrict__ wts, uint32_t capacity) {
    constexpr int kMaxRows = 256;                       // ty <= 8192 / W, W >= 32
    __shared__ unsigned long long s_row[kMaxRows + 1];  // tile-flat exclusive prefix at each row start
    __shared__ unsigned long long s_ox[kMaxRows];       // ... at physical x' = ox of each row
    __shared__ unsigned long long s_warp[kSlabThreads / 32];
    __shared__ unsigned s_base[4];
    const int tile = blockIdx.x;
    int chunk, z, y0, y1;
    if (!tile_coords(p, tile, chunk, z, y0, y1)) return;
    const int W = p.rb.voxels_size.x;
    const int ox = p.rb.origin_GRID.x, kx = ox >> 2, ix = ox & 3;
    const int z_end = (chunk + 1) * p.step;
    const int rows = y1 - y0, ngroups = rows * rg.G;
    const int tin = tile - chunk * p.tiles_per_chunk;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < 4) s_base[threadIdx.x] = offs[(size_t)(chunk * 4 + threadIdx.x) * p.tiles_per_chunk + tin];

    // phase 1: the predicate bits of the thread's 8 consecutive groups
    // g = 8 t + j, as the count kernel stored them (zero past the tile's end)
    unsigned bits[kGroupsPerThread];
    const int g0 = kGroupsPerThread * threadIdx.x;
    {
        const uint4 v = *reinterpret_cast<const uint4 *>(p.gbits + (size_t)tile * kTileGroups + g0);
        const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
        #pragma unroll
        for (int j = 0; j < kGroupsPerThread; ++j) bits[j] = (w4[j >> 1] >> (16 * (j & 1))) & 0xffffu;
    }
    // phase 2: one block scan of the per-thread packed counts; serial within the thread
    unsigned long long tsum = 0;
    #pragma unroll
    for (int j = 0; j < kGroupsPerThread; ++j) tsum += packed_counts(bits[j]);
    unsigned long long v = tsum;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long o = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += o;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    unsigned long long run = v - tsum;
    for (int w2 = 0; w2 < warp; ++w2) run += s_warp[w2];
    unsigned long long excl[kGroupsPerThread];
    #pragma unroll
    for (int j = 0; j < kGroupsPerThread; ++j) {
        excl[j] = run;
        const int g = g0 + j;
        if (g < ngroups) {
            const int r = (int)__umulhi((unsigned)g, rg.g_magic), k = g - r * rg.G;
            if (k == 0) s_row[r] = run;
            // count before physical x' = ox: the groups before, and voxels i < ix of this group
            if (k == kx) s_ox[r] = run + packed_counts(bits[j] & ((1u << (4 * ix)) - 1u));
        }
        run += packed_counts(bits[j]);
    }
    if (threadIdx.x == kSlabThreads - 1) s_row[rows] = run;  // the tile total
    __syncthreads();

    // phase 3: logical raster rank = physical rank rotated about x' = ox
    #pragma unroll
    for (int j = 0; j < kGroupsPerThread; ++j) {
        unsigned b = bits[j];
        if (!b) continue;
        const int g = g0 + j;
        const int r = (int)__umulhi((unsigned)g, rg.g_magic), k = g - r * rg.G, y = y0 + r;
        const unsigned long long rs = s_row[r], re = s_row[r + 1], ro = s_ox[r];
        while (b) {
            const int bit = __ffs(b) - 1;
            b &= b - 1;
            const int i = bit >> 2, q = bit & 3;
            const int xp = 4 * k + i;
            // physical prefix within the row for plane q
            const int P = field(excl[j], q) - field(rs, q) + plane_count(bits[j] & ((1u << (4 * i)) - 1u), q);
            const int A = field(ro, q) - field(rs, q), T = field(re, q) - field(rs, q);
            const int rank = xp >= ox ? P - A : P + (T - A);
            const uint32_t slot = s_base[q] + (uint32_t)(field(rs, q)) + (uint32_t)rank;
            if (slot >= capacity) continue;
            int lxv = xp - ox;
            if (lxv < 0) lxv += W;
            const int nx = lxv + (q == 0), ny = y + (q == 1), nz = z + (q == 2);
            float px = (float)nx, py = (float)ny, pz = (float)nz;
            if (p.metric) {
                px = __fmul_rn(__fadd_rn(px, 0.5f), p.cell.x);
                py = __fmul_rn(__fadd_rn(py, 0.5f), p.cell.y);
                pz = __fmul_rn(__fadd_rn(pz, 0.5f), p.cell.z);
            }
            pts[slot] = tde_xyzi{px, py, pz, 1.0f};
            if (cols || wts) {
                const size_t a = voxel_address(nx, ny, nz, p.rb);
                if (cols) cols[slot] = COLOR ? p.color[a] : tde_color{0, 0, 0, 0};
                if (wts) {
                    float f; int w;
                    TsdfStore<FMT>::decode(TsdfStore<FMT>::load_raw(p.vol, a, p.n), f, w);
                    wts[slot] = (float)w;
                }
            }
        }
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

// Extract_Color_Slice (opencl_wrappers.cpp:687-782; its kernels
// scan_slice_of_color_volume and extract_color_slice_as_cloud are absent):
// the colour plane alone -- voxels of the black zone whose colour is set
// (Color_Point_Is_Set, scan_slice_of_both_volumes.cl:53-58), in (z, y, x)
// raster order of logical voxels (the order chunking in z keeps for one
// plane).  Tiles as above, one count per tile.
__global__ void __launch_bounds__(kSlabThreads) color_count_kernel(const SlabParams p, uint32_t *__restrict__ counts) {
    __shared__ unsigned s_cnt;
    const int tile = blockIdx.x;
    int chunk, z, y0, y1;
    const bool live = tile_coords(p, tile, chunk, z, y0, y1);
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    unsigned c = 0;
    if (live) {
        const int W = p.rb.voxels_size.x, nvox = (y1 - y0) * W;
        for (int r = threadIdx.x; r < nvox; r += kSlabThreads) {
            const int y = y0 + r / W, x = r - (r / W) * W;
            c += in_black_zone(x, y, z, p.mn, p.mx, p.rb) && color_set(p.color[voxel_address(x, y, z, p.rb)]);
        }
    }
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_cnt, c);
    __syncthreads();
    if (threadIdx.x == 0) counts[tile] = s_cnt;
}

__global__ void __launch_bounds__(kSlabThreads) color_scatter_kernel(const SlabParams p, const uint32_t *__restrict__ offs,
                                                                    tde_color *__restrict__ cols, uint32_t capacity) {
    __shared__ unsigned s_warp[kSlabThreads / 32];
    __shared__ unsigned s_base;
    const int tile = blockIdx.x;
    int chunk, z, y0, y1;
    if (!tile_coords(p, tile, chunk, z, y0, y1)) return;
    const int W = p.rb.voxels_size.x, nvox = (y1 - y0) * W;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_base = offs[tile];
    __syncthreads();
    for (int r0 = 0; r0 < nvox; r0 += kSlabThreads) {
        const int r = r0 + threadIdx.x;
        bool set = false;
        tde_color c = {0, 0, 0, 0};
        if (r < nvox) {
            const int y = y0 + r / W, x = r - (r / W) * W;
            if (in_black_zone(x, y, z, p.mn, p.mx, p.rb)) {
                c = p.color[voxel_address(x, y, z, p.rb)];
                set = color_set(c);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, set);
        if (lane == 0) s_warp[warp] = __popc(m);
        __syncthreads();
        if (set) {
            unsigned before = 0;
            for (int w2 = 0; w2 < warp; ++w2) before += s_warp[w2];
            const uint32_t slot = s_base + before + __popc(m & ((1u << lane) - 1u));
            if (slot < capacity) cols[slot] = c;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (int w2 = 0; w2 < kSlabThreads / 32; ++w2) tot += s_warp[w2];
            s_base += tot;
        }
        __syncthreads();
    }
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
// Scratch: the (chunk, plane, tile) counts, then -- when the volume's rows
// suit the row kernels -- kTileGroups 16-bit predicate words per tile.
static bool row_geometry(const tde_round_buffer &rb, const SlabParams &p) {
    const int W = rb.voxels_size.x;
    return W % 4 == 0 && W >= 32 && p.ty * (W / 4) <= kTileGroups && p.ty <= 256;
}
static size_t counts_bytes(const tde_round_buffer &rb, const SlabParams &p) {
    const size_t tiles = (size_t)rb.voxels_size.z * p.tiles_per_z;
    return ((tiles * 4 + 64) * sizeof(uint32_t) + 15) & ~(size_t)15;
}
size_t slab_scratch_bytes(const tde_round_buffer &rb) {
    SlabParams p;
    p.step = slab_chunk_depth(rb.voxels_size.z, 4);
    slab_geometry(rb, p);
    const size_t tiles = (size_t)rb.voxels_size.z * p.tiles_per_z;
    return counts_bytes(rb, p) + (row_geometry(rb, p) ? tiles * kTileGroups * sizeof(uint16_t) : 0);
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
    // the row-vector kernels need whole 4-voxel groups, 16-byte aligned
    // buffers and at most 2048 groups / 256 rows per tile
    const bool vec = row_geometry(rb, p) && reinterpret_cast<uintptr_t>(vol) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(color) % 16 == 0 && reinterpret_cast<uintptr_t>(scratch) % 16 == 0;
    p.gbits = vec ? reinterpret_cast<uint16_t *>(static_cast<char *>(scratch) + counts_bytes(rb, p)) : nullptr;
    const bool scalar = !vec;
    // a zone covering every voxel (whole-volume export) skips the zone tests
    const tde_point3i &o = rb.origin_GRID, &N = rb.voxels_size;
    const bool whole = mn.x <= o.x && mx.x >= o.x + N.x - 1;  // every logical x is in the zone
    RowGeom rg;
    rg.G = rb.voxels_size.x / 4;
    rg.g_magic = (uint32_t)((0x100000000ull + (unsigned long long)rg.G - 1) / (unsigned long long)rg.G);
    rg.xlast = o.x == 0 ? N.x - 1 : o.x - 1;
    rg.row_stride_z = N.x * N.y;
    return dispatch_format(fmt, [&](auto F) {
        constexpr int FMT = decltype(F)::value;
        if (scalar) slab_count_kernel<FMT><<<ntiles, kSlabThreads, 0, stream>>>(p, counts);
        else if (whole && !color) row_count_kernel<FMT, false, false><<<ntiles, kSlabThreads, 0, stream>>>(p, rg, counts);
        else if (!color) row_count_kernel<FMT, true, false><<<ntiles, kSlabThreads, 0, stream>>>(p, rg, counts);
        else row_count_kernel<FMT, true, true><<<ntiles, kSlabThreads, 0, stream>>>(p, rg, counts);
        int st = check_launch("extract_slice/count");
        if (st) return st;
        exclusive_scan_kernel<<<1, 1024, 0, stream>>>(counts, ncounts, count);
        st = check_launch("extract_slice/scan");
        if (st) return st;
        if (scalar)
            slab_scatter_kernel<FMT><<<ntiles, kSlabThreads, 0, stream>>>(p, counts, pts, cols, wts, capacity);
        else if (whole && !color)
            row_scatter_kernel<FMT, false, false>
                <<<ntiles, kSlabThreads, 0, stream>>>(p, rg, counts, pts, cols, wts, capacity);
        else if (!color)
            row_scatter_kernel<FMT, true, false>
                <<<ntiles, kSlabThreads, 0, stream>>>(p, rg, counts, pts, cols, wts, capacity);
        else
            row_scatter_kernel<FMT, true, true>
                <<<ntiles, kSlabThreads, 0, stream>>>(p, rg, counts, pts, cols, wts, capacity);
        return check_launch("extract_slice/scatter");
    });
}

int launch_extract_color_slice(const tde_color *color, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                               void *scratch, size_t scratch_bytes, tde_color *cols, uint32_t capacity,
                               uint32_t *count, cudaStream_t stream) {
    SlabParams p;
    p.vol = nullptr; p.color = color; p.rb = rb; p.mn = mn; p.mx = mx; p.n = voxel_count(rb);
    p.metric = 0; p.cell = tde_point3f{1.f, 1.f, 1.f}; p.gbits = nullptr;
    // one plane: the whole depth as one chunk gives the same raster order
    p.step = rb.voxels_size.z;
    slab_geometry(rb, p);
    const int ntiles = p.tiles_per_chunk;
    if (scratch_bytes < slab_scratch_bytes(rb) || (size_t)ntiles * sizeof(uint32_t) > scratch_bytes)
        return set_error(TDE_ERR_INVALID_ARG, "extract_color_slice: scratch %zu < %zu bytes", scratch_bytes,
                         slab_scratch_bytes(rb));
    uint32_t *counts = reinterpret_cast<uint32_t *>(scratch);
    color_count_kernel<<<ntiles, kSlabThreads, 0, stream>>>(p, counts);
    int st = check_launch("extract_color_slice/count");
    if (st) return st;
    exclusive_scan_kernel<<<1, 1024, 0, stream>>>(counts, ntiles, count);
    if ((st = check_launch("extract_color_slice/scan"))) return st;
    color_scatter_kernel<<<ntiles, kSlabThreads, 0, stream>>>(p, counts, cols, capacity);
    return check_launch("extract_color_slice/scatter");
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
