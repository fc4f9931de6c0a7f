// k_refiner.cu -- kernels of the learned depth refiner.
//
// The convolutions are implicit GEMMs on the 5th-generation tensor cores:
// bf16 operands in shared memory, FP32 accumulators in tensor memory, issued
// by one thread with tcgen05.mma.  Activations are NHWC bf16, so the 16-byte
// "core matrix" rows the tensor core reads are 8 consecutive channels of one
// pixel.
//
// Forward / input gradient (conv3x3_tc_kernel): M = 128 output pixels of one
// image row, N = output channels, K = 9 taps x input channels.  The block
// stages the 3 x 130-pixel input halo once, as planes of 8-channel chunks
// (plane (row, chunk) holds the chunk of every halo pixel, 16 B apart).  In
// that layout the A operand of tap (dy, dx) is the same planes started dx
// pixels later, so each of the 9 taps is a descriptor offset -- no im2col
// copy.  The input gradient is the same kernel run on the output gradient
// with the transposed, tap-flipped weights.
//
// Weight gradient (wgrad_tc_kernel): M = 128 rows of (tap, input channel),
// N = output channels, K = pixels.  Both operands are transposed into
// K-major core matrices in shared memory (K = 64 pixels per step); a row of
// ones gives the bias gradient.  Each block accumulates its share of the
// pixels for all row tiles in tensor memory and writes one partial; a
// reduction kernel sums the partials in a fixed order (deterministic).
#include <cuda_bf16.h>

#include "tde_common.cuh"
#include "tde_refiner.cuh"
#include "tde_tc.cuh"

namespace tde {
namespace refiner {
namespace {

constexpr int kTileM = 128;             // output pixels per MMA tile
constexpr int kHaloW = kTileM + 2;      // halo pixels per row
constexpr int kConvThreads = 128;       // 4 warps: one TMEM lane quarter each
constexpr int kWgK = 64;                // pixels per weight-gradient K step
constexpr int kWgHalo = kWgK + 2;
constexpr int kWgThreads = 256;
constexpr uint32_t kSmemPerSM = 228 * 1024;

__host__ __device__ inline uint32_t tmem_cols(int n) {
    uint32_t c = 32;
    while (c < (uint32_t)n) c <<= 1;
    return c;
}

__device__ __forceinline__ uint4 ldg16(const bf16 *p) { return __ldg(reinterpret_cast<const uint4 *>(p)); }

__device__ __forceinline__ uint32_t bmax2(uint32_t a, uint32_t b) {
    __nv_bfloat162 x = *reinterpret_cast<__nv_bfloat162 *>(&a), y = *reinterpret_cast<__nv_bfloat162 *>(&b);
    __nv_bfloat162 r = __hmax2(x, y);
    return *reinterpret_cast<uint32_t *>(&r);
}
__device__ __forceinline__ uint4 bmax4(uint4 a, uint4 b) {
    return make_uint4(bmax2(a.x, b.x), bmax2(a.y, b.y), bmax2(a.z, b.z), bmax2(a.w, b.w));
}

__device__ __forceinline__ float bf_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }
__device__ __forceinline__ void unpack8(uint4 q, float *f) {
    f[0] = bf_lo(q.x); f[1] = bf_hi(q.x); f[2] = bf_lo(q.y); f[3] = bf_hi(q.y);
    f[4] = bf_lo(q.z); f[5] = bf_hi(q.z); f[6] = bf_lo(q.w); f[7] = bf_hi(q.w);
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 r = __floats2bfloat162_rn(a, b);  // .x = a (low half)
    return *reinterpret_cast<uint32_t *>(&r);
}
__device__ __forceinline__ uint4 pack8(const float *f) {
    return make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
}

// Chunk c (channels 8c..8c+7) of the concatenated convolution input at
// (img, y, x); zero outside the image.  ca and cb are multiples of 8.
template <typename Args>
__device__ __forceinline__ uint4 load_input_chunk(const Args &A, int img, int y, int x, int c) {
    if (y < 0 || y >= A.h || x < 0 || x >= A.w) return make_uint4(0u, 0u, 0u, 0u);
    const int cca = A.ca >> 3;
    if (c < cca) {
        if (A.mode_a == SRC_DIRECT) return ldg16(A.a + (((size_t)img * A.h + y) * A.w + x) * A.ca + 8 * c);
        if (A.mode_a == SRC_UP) {
            const int hh = A.h >> 1, ww = A.w >> 1;
            return ldg16(A.a + (((size_t)img * hh + (y >> 1)) * ww + (x >> 1)) * A.ca + 8 * c);
        }
        const int W2 = A.w * 2;
        const bf16 *p = A.a + (((size_t)img * (A.h * 2) + 2 * y) * W2 + 2 * x) * A.ca + 8 * c;
        const size_t row = (size_t)W2 * A.ca;
        return bmax4(bmax4(ldg16(p), ldg16(p + A.ca)), bmax4(ldg16(p + row), ldg16(p + row + A.ca)));
    }
    return ldg16(A.b + (((size_t)img * A.h + y) * A.w + x) * A.cb + 8 * (c - cca));
}

// ---------------------------------------------------------------------------
// Forward / input-gradient convolution
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kConvThreads) conv3x3_tc_kernel(const ConvArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int cin = A.ca + A.cb, cc = cin >> 3;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned char *halo = smem;
    unsigned char *wsm = smem + (size_t)3 * cc * kHaloW * 16;
    const uint32_t ncols = tmem_cols(A.cout);

    if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    // weights: global [co][t][ci] -> planes (t, chunk) of cout rows x 16 B
    const int nw = A.cout * 9 * cc;
    for (int i = tid; i < nw; i += kConvThreads) {
        const int c = i % cc, t = (i / cc) % 9, co = i / (9 * cc);
        *reinterpret_cast<uint4 *>(wsm + ((size_t)(t * cc + c) * A.cout + co) * 16) = ldg16(A.wgt + (size_t)i * 8);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t halo_s = tc::smem_u32(halo), w_s = tc::smem_u32(wsm);
    const uint32_t idesc = tc::idesc_bf16(kTileM, A.cout);
    const int tiles_x = (A.w + kTileM - 1) / kTileM;
    const int ntiles = A.n * A.h * tiles_x;
    const int nh = 3 * kHaloW * cc;
    uint32_t parity = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int xt = tile % tiles_x, rowi = tile / tiles_x;
        const int y = rowi % A.h, img = rowi / A.h;
        const int x0 = xt * kTileM;
        for (int i = tid; i < nh; i += kConvThreads) {
            const int c = i % cc, px = (i / cc) % kHaloW, dy = i / (cc * kHaloW);
            *reinterpret_cast<uint4 *>(halo + ((size_t)(dy * cc + c) * kHaloW + px) * 16) =
                load_input_chunk(A, img, y + dy - 1, x0 + px - 1, c);
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            uint32_t acc = 0;
            for (int t = 0; t < 9; ++t) {
                const int dy = t / 3, dx = t % 3;
                for (int kc = 0; kc < cc; kc += 2) {
                    const uint64_t ad = tc::desc(halo_s + (uint32_t)(((dy * cc + kc) * kHaloW + dx) * 16), kHaloW * 16, 128);
                    const uint64_t bd = tc::desc(w_s + (uint32_t)((t * cc + kc) * A.cout * 16), A.cout * 16, 128);
                    tc::mma_bf16(tmem, ad, bd, idesc, acc);
                    acc = 1;
                }
            }
            tc::commit(&mbar);
        }
        const bool done = tc::mbar_wait(&mbar, parity);
        parity ^= 1u;
        if (__syncthreads_or(!done)) {
            failed = true;
            break;
        }
        tc::fence_after_sync();

        // epilogue: warp w owns TMEM lanes (pixels) 32w..32w+31
        const int m = warp * 32 + lane;
        const int x = x0 + m;
        const bool valid = x < A.w;
        const size_t pix = ((size_t)img * A.h + y) * A.w + (valid ? x : 0);
        float r = 0.f;
        for (int j = 0; j < A.cout; j += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j, v);
            if (!valid) continue;
            if (A.bias) {
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] += __ldg(A.bias + j + k);
            }
            if (A.relu) {
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] = v[k] > 0.f ? v[k] : 0.f;
            }
            if (A.mask) {
                float mk[16];
                unpack8(ldg16(A.mask + pix * A.cout + j), mk);
                unpack8(ldg16(A.mask + pix * A.cout + j + 8), mk + 8);
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] = mk[k] > 0.f ? v[k] : 0.f;
            }
            const uint4 q0 = pack8(v), q1 = pack8(v + 8);
            uint4 *o = reinterpret_cast<uint4 *>(A.out + pix * A.cout + j);
            o[0] = q0;
            o[1] = q1;
            if (A.head_w) {
                float f[16];
                unpack8(q0, f);
                unpack8(q1, f + 8);
#pragma unroll
                for (int k = 0; k < 16; ++k) r = fmaf(__ldg(A.head_w + j + k), f[k], r);
            }
        }
        if (valid && A.head_w) {
            const float d = A.depth_in[pix];
            const float o = d > 0.f ? d + 0.01f * (r + __ldg(A.head_b)) : 0.f;  // residual in cm
            if (A.depth_out) A.depth_out[pix] = o;
            if (A.depth_mm) {
                const float mm = fminf(fmaxf(rintf(o * 1000.f), 0.f), (float)TDE_MAX_DEPTH_VALUE);
                A.depth_mm[pix] = (uint16_t)mm;
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) atomicExch(A.err, 1);
        // give the MMAs in flight a second bounded chance to finish before
        // the tensor memory they write is released
        tc::mbar_wait(&mbar, parity ^ 1u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Weight gradient
// ---------------------------------------------------------------------------
struct WgLayout {
    int cin, cc, rows, mtiles;
    uint32_t x_off, z_off, bt_off, a_off, total;
};
__host__ __device__ inline WgLayout wg_layout(int cin, int cout) {
    WgLayout L;
    L.cin = cin;
    L.cc = cin / 8;
    L.rows = 9 * cin + 1;
    L.mtiles = (L.rows + 127) / 128;
    L.x_off = 0;                                               // X halo, planes (row, chunk) x 66 px x 16 B
    L.z_off = L.x_off + (uint32_t)(3 * L.cc * kWgHalo * 16);   // dZ rows [px][cout]
    L.bt_off = L.z_off + (uint32_t)(kWgK * cout * 2);          // B: dZ^T core matrices
    L.a_off = L.bt_off + (uint32_t)(kWgK * cout * 2);          // A: 2 buffers of 128 x 64 bf16
    L.a_off = (L.a_off + 127u) & ~127u;
    L.total = L.a_off + 2u * 128u * kWgK * 2u;
    return L;
}

__global__ void __launch_bounds__(kWgThreads) wgrad_tc_kernel(const WgradArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    const int cin = A.ca + A.cb, cout = A.cout;
    const WgLayout L = wg_layout(cin, cout);
    const int cc = L.cc;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols = tmem_cols(L.mtiles * cout);
    unsigned char *xs = smem + L.x_off;
    const bf16 *xsb = reinterpret_cast<const bf16 *>(xs);
    bf16 *zs = reinterpret_cast<bf16 *>(smem + L.z_off);
    unsigned char *bt = smem + L.bt_off;
    unsigned char *as = smem + L.a_off;

    if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t a_s = tc::smem_u32(as), b_s = tc::smem_u32(bt);
    const uint32_t idesc = tc::idesc_bf16(128, cout);
    const int tiles_x = (A.w + kWgK - 1) / kWgK;
    const int ntiles = A.n * A.h * tiles_x;
    uint32_t issued[2] = {0u, 0u}, waited[2] = {0u, 0u};
    bool first = true, failed = false;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int xt = tile % tiles_x, rowi = tile / tiles_x;
        const int y = rowi % A.h, img = rowi / A.h;
        const int x0 = xt * kWgK;
        // every MMA reading B (and the A buffers) must be done before restaging
        bool ok = true;
        for (int b = 0; b < 2; ++b)
            if (issued[b] > waited[b]) {
                ok &= tc::mbar_wait(&mbar[b], waited[b] & 1u);
                waited[b]++;
            }
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        // stage X halo (3 rows x 66 px x cin) and the dZ row segment (64 px x cout)
        for (int i = tid; i < 3 * kWgHalo * cc; i += kWgThreads) {
            const int c = i % cc, px = (i / cc) % kWgHalo, dy = i / (cc * kWgHalo);
            *reinterpret_cast<uint4 *>(xs + ((size_t)(dy * cc + c) * kWgHalo + px) * 16) =
                load_input_chunk(A, img, y + dy - 1, x0 + px - 1, c);
        }
        const int zc = cout / 8;
        for (int i = tid; i < kWgK * zc; i += kWgThreads) {
            const int c = i % zc, px = i / zc;
            const int x = x0 + px;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (x < A.w) v = ldg16(A.dz + (((size_t)img * A.h + y) * A.w + x) * cout + 8 * c);
            *reinterpret_cast<uint4 *>(zs + (size_t)px * cout + 8 * c) = v;
        }
        __syncthreads();
        // B = dZ^T: row co, K = pixel; core matrix (k chunk g, row group co/8)
        for (int i = tid; i < cout * (kWgK / 8); i += kWgThreads) {
            const int co = i % cout, g = i / cout;
            float f[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) f[j] = __bfloat162float(zs[(size_t)(8 * g + j) * cout + co]);
            *reinterpret_cast<uint4 *>(bt + ((size_t)(g * (cout / 8) + co / 8) * 128 + (co % 8) * 16)) = pack8(f);
        }
        for (int mt = 0; mt < L.mtiles; ++mt) {
            const int buf = (int)((issued[0] + issued[1]) & 1u);
            ok = true;
            if (issued[buf] > waited[buf]) {
                ok = tc::mbar_wait(&mbar[buf], waited[buf] & 1u);
                waited[buf]++;
            }
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            unsigned char *ab = as + (size_t)buf * 128 * kWgK * 2;
            // A rows r = mt*128 + i: (tap, channel) of the shifted input, or ones (bias), or zero
            for (int it = tid; it < 128 * (kWgK / 8); it += kWgThreads) {
                const int i = it % 128, g = it / 128;
                const int r = mt * 128 + i;
                float f[8];
                if (r < 9 * cin) {
                    const int t = r / cin, ci = r % cin;
                    const int dy = t / 3, dx = t % 3;
                    const bf16 *src = xsb + ((size_t)(dy * cc + ci / 8) * kWgHalo) * 8 + (ci % 8);
#pragma unroll
                    for (int j = 0; j < 8; ++j) f[j] = __bfloat162float(src[(size_t)(8 * g + j + dx) * 8]);
                } else {
                    const float one = r == 9 * cin ? 1.f : 0.f;
#pragma unroll
                    for (int j = 0; j < 8; ++j) f[j] = (x0 + 8 * g + j < A.w) ? one : 0.f;
                }
                *reinterpret_cast<uint4 *>(ab + ((size_t)g * 2048 + (i / 8) * 128 + (i % 8) * 16)) = pack8(f);
            }
            tc::fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t abase = a_s + (uint32_t)buf * 128u * kWgK * 2u;
                for (int kk = 0; kk < kWgK / 16; ++kk) {
                    const uint64_t ad = tc::desc(abase + (uint32_t)(2 * kk * 2048), 2048, 128);
                    const uint64_t bd = tc::desc(b_s + (uint32_t)(2 * kk * (cout / 8) * 128), cout * 16, 128);
                    tc::mma_bf16(tmem + (uint32_t)(mt * cout), ad, bd, idesc, (first && kk == 0) ? 0u : 1u);
                }
                tc::commit(&mbar[buf]);
            }
            issued[buf]++;
        }
        first = false;
    }
    // drain
    bool ok = true;
    for (int b = 0; b < 2; ++b)
        if (issued[b] > waited[b]) {
            ok &= tc::mbar_wait(&mbar[b], waited[b] & 1u);
            waited[b]++;
        }
    failed |= __syncthreads_or(!ok) != 0;
    tc::fence_after_sync();
    if (failed) {
        if (tid == 0) atomicExch(A.err, 1);
    } else {
        // epilogue: warps w and w+4 share TMEM lane quarter w; they split the row tiles
        const int q = warp & 3;
        const size_t rows_pad = (size_t)L.mtiles * 128;
        float *dst = A.partial + (size_t)blockIdx.x * rows_pad * cout;
        for (int mt = 0; mt < L.mtiles; ++mt) {
            const bool mine = ((mt & 1) == (warp >> 2));
            for (int j = 0; j < cout; j += 16) {
                float v[16];
                if (mine) {
                    tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(mt * cout + j), v);
                    if (first) {  // this block visited no pixels
#pragma unroll
                        for (int k = 0; k < 16; ++k) v[k] = 0.f;
                    }
                    const size_t r = (size_t)mt * 128 + q * 32 + lane;
                    float4 *o = reinterpret_cast<float4 *>(dst + r * cout + j);
#pragma unroll
                    for (int k = 0; k < 4; ++k) o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

__global__ void wgrad_reduce_kernel(const float *__restrict__ partial, int blocks, int cin, int cout, size_t rows_pad,
                                    float *__restrict__ dw, float *__restrict__ db) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = r * cout + co
    const int nr = 9 * cin + 1;
    if (i >= nr * cout) return;
    const int r = i / cout, co = i % cout;
    float s = 0.f;
    for (int b = 0; b < blocks; ++b) s += partial[((size_t)b * rows_pad + r) * cout + co];
    if (r == 9 * cin) db[co] = s;
    else dw[((size_t)co * 9 + r / cin) * cin + r % cin] = s;
}

// ---------------------------------------------------------------------------
// First convolution (2 -> 16, FP32) and its weight gradient
// ---------------------------------------------------------------------------
// Input features of tap t (3x3 window around the pixel, t = 3*dy + dx):
// [100 (d_t - d_c) if both valid else 0, valid_t, d_t], d in metres (0 where
// invalid).  Differences in centimetres keep millimetre noise representable
// once the first layer's output is stored as bf16.
constexpr int kInCh = 3, kInK = 9 * kInCh;
__device__ __forceinline__ void input_features(const float (&d)[9], float (&in)[kInK]) {
    const float dc = d[4];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const bool vt = d[t] > 0.f;
        in[3 * t] = (vt && dc > 0.f) ? (d[t] - dc) * 100.f : 0.f;
        in[3 * t + 1] = vt ? 1.f : 0.f;
        in[3 * t + 2] = d[t];
    }
}

__global__ void __launch_bounds__(256) conv_in_kernel(const uint16_t *__restrict__ raw, float *__restrict__ depth_m,
                                                      const float *__restrict__ w1, const float *__restrict__ b1,
                                                      bf16 *__restrict__ e0a, int n, int h, int w) {
    __shared__ float sw[16 * kInK + 16];
    for (int i = threadIdx.x; i < 16 * kInK; i += blockDim.x) sw[i] = w1[i];
    if (threadIdx.x < 16) sw[16 * kInK + threadIdx.x] = b1[threadIdx.x];
    __syncthreads();
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (size_t)n * h * w) return;
    const int x = (int)(p % w), y = (int)((p / w) % h), img = (int)(p / ((size_t)w * h));
    float d[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
        d[t] = 0.f;
        if (yy >= 0 && yy < h && xx >= 0 && xx < w) d[t] = (float)raw[((size_t)img * h + yy) * w + xx] * 0.001f;
    }
    float in[kInK];
    input_features(d, in);
    depth_m[p] = d[4];
    float o[16];
#pragma unroll
    for (int co = 0; co < 16; ++co) {
        float s = sw[16 * kInK + co];
#pragma unroll
        for (int k = 0; k < kInK; ++k) s = fmaf(sw[co * kInK + k], in[k], s);
        o[co] = s > 0.f ? s : 0.f;
    }
    uint4 *dst = reinterpret_cast<uint4 *>(e0a + p * 16);
    dst[0] = pack8(o);
    dst[1] = pack8(o + 8);
}

// Block = 16 output channels x 16 pixel lanes; each block covers whole image
// rows and writes 16 x 28 partial sums (27 weights + bias per channel).
constexpr int kInRowsPerBlock = 4;
constexpr int kInPartial = 16 * (kInK + 1);
__global__ void __launch_bounds__(256) conv_in_wgrad_kernel(const float *__restrict__ depth_m,
                                                            const bf16 *__restrict__ dz1, int n, int h, int w,
                                                            float *__restrict__ partial) {
    __shared__ float red[16][16][kInK + 1];
    const int co = threadIdx.x & 15, pl = threadIdx.x >> 4;
    float s[kInK + 1];
#pragma unroll
    for (int k = 0; k <= kInK; ++k) s[k] = 0.f;
    const int row0 = blockIdx.x * kInRowsPerBlock;
    for (int rr = 0; rr < kInRowsPerBlock; ++rr) {
        const int rowi = row0 + rr;
        if (rowi >= n * h) break;
        const int y = rowi % h, img = rowi / h;
        for (int x = pl; x < w; x += 16) {
            const size_t p = ((size_t)img * h + y) * w + x;
            const float g = __bfloat162float(dz1[p * 16 + co]);
            if (g == 0.f) continue;
            float d[9];
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
                d[t] = (yy >= 0 && yy < h && xx >= 0 && xx < w) ? depth_m[((size_t)img * h + yy) * w + xx] : 0.f;
            }
            float in[kInK];
            input_features(d, in);
#pragma unroll
            for (int k = 0; k < kInK; ++k) s[k] = fmaf(g, in[k], s[k]);
            s[kInK] += g;
        }
    }
#pragma unroll
    for (int k = 0; k <= kInK; ++k) red[pl][co][k] = s[k];
    __syncthreads();
    for (int i = threadIdx.x; i < kInPartial; i += blockDim.x) {
        const int c = i / (kInK + 1), k = i % (kInK + 1);
        float t = 0.f;
        for (int l = 0; l < 16; ++l) t += red[l][c][k];
        partial[(size_t)blockIdx.x * kInPartial + i] = t;
    }
}

__global__ void conv_in_wgrad_reduce_kernel(const float *__restrict__ partial, int blocks, float *__restrict__ dw1,
                                            float *__restrict__ db1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // c * 28 + k
    if (i >= kInPartial) return;
    float t = 0.f;
    for (int b = 0; b < blocks; ++b) t += partial[(size_t)b * kInPartial + i];
    const int c = i / (kInK + 1), k = i % (kInK + 1);
    if (k == kInK) db1[c] = t;
    else dw1[c * kInK + k] = t;
}

// ---------------------------------------------------------------------------
// Loss, head gradient and the gradient entering the last convolution
// ---------------------------------------------------------------------------
constexpr int kLossThreads = 256;
__global__ void __launch_bounds__(kLossThreads) loss_kernel(const float *__restrict__ out_m,
                                                            const float *__restrict__ depth_m,
                                                            const uint16_t *__restrict__ target,
                                                            const bf16 *__restrict__ d0,
                                                            const float *__restrict__ head_w, size_t npix, float inv,
                                                            bf16 *__restrict__ dz11, float *__restrict__ partial) {
    // per thread: loss, count, 16 head-weight sums, head-bias sum
    float acc[19];
#pragma unroll
    for (int k = 0; k < 19; ++k) acc[k] = 0.f;
    float hw[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) hw[c] = __ldg(head_w + c);
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        const float t = (float)target[p] * 0.001f;
        const bool m = depth_m[p] > 0.f && target[p] != 0;
        const float diff = out_m[p] - t;
        float dr = 0.f;
        if (m) {
            acc[0] += fabsf(diff) * inv;
            acc[1] += 1.f;
            // gradient with respect to the head output r (out = d + 0.01 r)
            dr = 0.01f * (diff > 0.f ? inv : diff < 0.f ? -inv : 0.f);
        }
        float f[16];
        unpack8(ldg16(d0 + p * 16), f);
        unpack8(ldg16(d0 + p * 16 + 8), f + 8);
        float g[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            acc[2 + c] = fmaf(dr, f[c], acc[2 + c]);
            g[c] = f[c] > 0.f ? dr * hw[c] : 0.f;
        }
        acc[18] += dr;
        uint4 *o = reinterpret_cast<uint4 *>(dz11 + p * 16);
        o[0] = pack8(g);
        o[1] = pack8(g + 8);
    }
    __shared__ float red[kLossThreads / 32][19];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 19; ++k) {
        float v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 19) {
        float v = 0.f;
        for (int w = 0; w < kLossThreads / 32; ++w) v += red[w][threadIdx.x];
        partial[(size_t)blockIdx.x * 19 + threadIdx.x] = v;
    }
}

__global__ void loss_reduce_kernel(const float *__restrict__ partial, int blocks, float *__restrict__ dhead_w,
                                   float *__restrict__ dhead_b, double *__restrict__ loss2) {
    const int k = threadIdx.x;
    if (k >= 19) return;
    double t = 0.0;
    for (int b = 0; b < blocks; ++b) t += (double)partial[(size_t)b * 19 + k];
    if (k < 2) loss2[k] = t;
    else if (k < 18) dhead_w[k - 2] = (float)t;
    else dhead_b[0] = (float)t;
}

// ---------------------------------------------------------------------------
// Gradient routing through upsampling, pooling and skips
// ---------------------------------------------------------------------------
__global__ void up_back_kernel(const bf16 *__restrict__ g, int cu, int ca, const bf16 *__restrict__ y_low,
                               bf16 *__restrict__ dz, int n, int h, int w) {
    const int hl = h >> 1, wl = w >> 1, cch = ca >> 3;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * hl * wl * cch) return;
    const int c = (int)(i % cch);
    const size_t q = i / cch;
    const int xl = (int)(q % wl), yl = (int)((q / wl) % hl), img = (int)(q / ((size_t)wl * hl));
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int y = 2 * yl + (k >> 1), x = 2 * xl + (k & 1);
        float f[8];
        unpack8(ldg16(g + (((size_t)img * h + y) * w + x) * cu + 8 * c), f);
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] += f[j];
    }
    float mk[8];
    unpack8(ldg16(y_low + q * ca + 8 * c), mk);
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] = mk[j] > 0.f ? s[j] : 0.f;
    *reinterpret_cast<uint4 *>(dz + q * ca + 8 * c) = pack8(s);
}

__global__ void pool_back_add_kernel(const bf16 *__restrict__ e, const bf16 *__restrict__ gp,
                                     const bf16 *__restrict__ skip, int cu, int off, int ch, bf16 *__restrict__ dz,
                                     int n, int h, int w) {
    const int hl = h >> 1, wl = w >> 1, cch = ch >> 3;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * hl * wl * cch) return;
    const int c = (int)(i % cch);
    const size_t q = i / cch;
    const int xl = (int)(q % wl), yl = (int)((q / wl) % hl), img = (int)(q / ((size_t)wl * hl));
    float ev[4][8], mx[8];
    size_t pix[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        pix[k] = ((size_t)img * h + 2 * yl + (k >> 1)) * w + 2 * xl + (k & 1);
        unpack8(ldg16(e + pix[k] * ch + 8 * c), ev[k]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) mx[j] = fmaxf(fmaxf(ev[0][j], ev[1][j]), fmaxf(ev[2][j], ev[3][j]));
    float gv[8];
    unpack8(ldg16(gp + q * ch + 8 * c), gv);
    int first[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) first[j] = ev[0][j] == mx[j] ? 0 : ev[1][j] == mx[j] ? 1 : ev[2][j] == mx[j] ? 2 : 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float s[8];
        unpack8(ldg16(skip + pix[k] * cu + off + 8 * c), s);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float v = s[j] + (first[j] == k ? gv[j] : 0.f);
            s[j] = ev[k][j] > 0.f ? v : 0.f;
        }
        *reinterpret_cast<uint4 *>(dz + pix[k] * ch + 8 * c) = pack8(s);
    }
}

// ---------------------------------------------------------------------------
// Optimiser and weight packing
// ---------------------------------------------------------------------------
__global__ void adamw_kernel(float *__restrict__ theta, const float *__restrict__ grad, float *__restrict__ m,
                             float *__restrict__ v, const uint8_t *__restrict__ decay, size_t count, float lr,
                             float b1, float b2, float eps, float wd, float bc1, float bc2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float upd = (mi / bc1) / (sqrtf(vi / bc2) + eps);
    const float th = theta[i];
    theta[i] = th - lr * (upd + (decay[i] ? wd : 0.f) * th);
}

__global__ void pack_weights_kernel(const float *__restrict__ w, int cout, int cin, bf16 *__restrict__ wq,
                                    bf16 *__restrict__ wt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = (co * 9 + t) * cin + ci
    if (i >= cout * 9 * cin) return;
    const int ci = i % cin, t = (i / cin) % 9, co = i / (9 * cin);
    const bf16 q = __float2bfloat16_rn(w[i]);
    wq[i] = q;
    wt[((size_t)ci * 9 + (8 - t)) * cout + co] = q;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
static uint32_t smem_floor_for_tmem(uint32_t ncols) {
    // at most 512 / ncols blocks per SM may hold TMEM at once; a block asks
    // for enough shared memory that no more than that fit
    const uint32_t kmax = 512u / ncols;
    return kSmemPerSM / (kmax + 1) - 1024u + 16u;
}

// Raises the kernel's dynamic shared-memory limit to `bytes` when needed.
static int allow_smem(const void *fn, size_t bytes, const char *what) {
    cudaFuncAttributes fa;
    TDE_CUDA(cudaFuncGetAttributes(&fa, fn), what);
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return TDE_OK;
    if (bytes + fa.sharedSizeBytes > 227 * 1024)
        return set_error(TDE_ERR_UNSUPPORTED, "%s: %zu B of shared memory", what, bytes);
    TDE_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes), what);
    return TDE_OK;
}

size_t conv_smem_bytes(int cin, int cout) {
    const int cc = cin / 8;
    size_t s = (size_t)3 * cc * kHaloW * 16 + (size_t)9 * cc * cout * 16;
    return s > smem_floor_for_tmem(tmem_cols(cout)) ? s : smem_floor_for_tmem(tmem_cols(cout));
}

int launch_conv(const ConvArgs &a, int num_sms, cudaStream_t s) {
    const int cin = a.ca + a.cb;
    if (cin % 16 || a.ca % 8 || a.cout % 16 || a.cout < 16 || a.cout > 256 || a.w <= 0 || a.h <= 0 || a.n <= 0 ||
        (a.head_w && a.cout != 16) || (a.mode_a == SRC_UP && (a.h % 2 || a.w % 2)))
        return set_error(TDE_ERR_INVALID_ARG, "refiner conv: unsupported shape cin=%d cout=%d", cin, a.cout);
    const size_t smem = conv_smem_bytes(cin, a.cout);
    if (smem > 227 * 1024) return set_error(TDE_ERR_UNSUPPORTED, "refiner conv: %zu B of shared memory", smem);
    TDE_TRY(allow_smem((const void *)conv3x3_tc_kernel, smem, "refiner conv"));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv3x3_tc_kernel, kConvThreads, smem);
    if (per_sm < 1) per_sm = 1;
    const int tiles = a.n * a.h * ((a.w + kTileM - 1) / kTileM);
    int grid = num_sms * per_sm;
    if (grid > tiles) grid = tiles;
    conv3x3_tc_kernel<<<grid, kConvThreads, smem, s>>>(a);
    return check_launch("refiner conv");
}

int wgrad_blocks(int num_sms, int cin, int cout) {
    (void)cin;
    (void)cout;
    return num_sms;
}

size_t wgrad_partial_floats(int blocks, int cin, int cout) {
    const WgLayout L = wg_layout(cin, cout);
    return (size_t)blocks * L.mtiles * 128 * cout;
}

int launch_wgrad(const WgradArgs &a, int blocks, cudaStream_t s) {
    const int cin = a.ca + a.cb;
    const WgLayout L = wg_layout(cin, a.cout);
    if (cin % 8 || a.cout % 16 || a.cout < 16 || L.mtiles * a.cout > 512)
        return set_error(TDE_ERR_INVALID_ARG, "refiner wgrad: unsupported shape cin=%d cout=%d", cin, a.cout);
    size_t smem = L.total;
    const size_t fl = smem_floor_for_tmem(tmem_cols(L.mtiles * a.cout));
    if (smem < fl) smem = fl;
    if (smem > 227 * 1024) return set_error(TDE_ERR_UNSUPPORTED, "refiner wgrad: %zu B of shared memory", smem);
    TDE_TRY(allow_smem((const void *)wgrad_tc_kernel, smem, "refiner wgrad"));
    wgrad_tc_kernel<<<blocks, kWgThreads, smem, s>>>(a);
    return check_launch("refiner wgrad");
}

int launch_wgrad_reduce(const float *partial, int blocks, int cin, int cout, float *dw, float *db, cudaStream_t s) {
    const WgLayout L = wg_layout(cin, cout);
    const int n = (9 * cin + 1) * cout;
    wgrad_reduce_kernel<<<div_up(n, 256), 256, 0, s>>>(partial, blocks, cin, cout, (size_t)L.mtiles * 128, dw, db);
    return check_launch("refiner wgrad reduce");
}

int launch_conv_in(const uint16_t *raw, float *depth_m, const float *w1, const float *b1, bf16 *e0a, int n, int h,
                   int w, cudaStream_t s) {
    const size_t np = (size_t)n * h * w;
    conv_in_kernel<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(raw, depth_m, w1, b1, e0a, n, h, w);
    return check_launch("refiner conv_in");
}

int conv_in_wgrad_blocks(int n, int h) { return div_up(n * h, kInRowsPerBlock); }

int launch_conv_in_wgrad(const float *depth_m, const bf16 *dz1, int n, int h, int w, float *partial, int blocks,
                         float *dw1, float *db1, cudaStream_t s) {
    conv_in_wgrad_kernel<<<blocks, 256, 0, s>>>(depth_m, dz1, n, h, w, partial);
    TDE_TRY(check_launch("refiner conv_in wgrad"));
    conv_in_wgrad_reduce_kernel<<<div_up(kInPartial, 128), 128, 0, s>>>(partial, blocks, dw1, db1);
    return check_launch("refiner conv_in wgrad reduce");
}

int loss_blocks(int n, int h, int w) {
    const size_t np = (size_t)n * h * w;
    size_t b = (np + kLossThreads * 8 - 1) / (kLossThreads * 8);
    return (int)(b < 1 ? 1 : b > 4096 ? 4096 : b);
}

int launch_loss(const float *out_m, const float *depth_m, const uint16_t *target, const bf16 *d0, const float *head_w,
                int n, int h, int w, bf16 *dz11, float *partial, int blocks, float *dhead_w, float *dhead_b,
                double *loss2, cudaStream_t s) {
    const size_t np = (size_t)n * h * w;
    loss_kernel<<<blocks, kLossThreads, 0, s>>>(out_m, depth_m, target, d0, head_w, np, 1.f / (float)np, dz11,
                                                partial);
    TDE_TRY(check_launch("refiner loss"));
    loss_reduce_kernel<<<1, 32, 0, s>>>(partial, blocks, dhead_w, dhead_b, loss2);
    return check_launch("refiner loss reduce");
}

int launch_up_back(const bf16 *g, int cu, int ca, const bf16 *y_low, bf16 *dz, int n, int h, int w, cudaStream_t s) {
    const size_t items = (size_t)n * (h / 2) * (w / 2) * (ca / 8);
    up_back_kernel<<<(unsigned)((items + 255) / 256), 256, 0, s>>>(g, cu, ca, y_low, dz, n, h, w);
    return check_launch("refiner up_back");
}

int launch_pool_back_add(const bf16 *e, const bf16 *gp, const bf16 *skip, int cu, int off, int c, bf16 *dz, int n,
                         int h, int w, cudaStream_t s) {
    const size_t items = (size_t)n * (h / 2) * (w / 2) * (c / 8);
    pool_back_add_kernel<<<(unsigned)((items + 255) / 256), 256, 0, s>>>(e, gp, skip, cu, off, c, dz, n, h, w);
    return check_launch("refiner pool_back_add");
}

int launch_adamw(float *theta, const float *grad, float *m, float *v, const uint8_t *decay_mask, size_t count,
                 float lr, float beta1, float beta2, float eps, float wd, float bc1, float bc2, cudaStream_t s) {
    adamw_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(theta, grad, m, v, decay_mask, count, lr, beta1,
                                                                 beta2, eps, wd, bc1, bc2);
    return check_launch("refiner adamw");
}

int launch_pack_weights(const float *w, int cout, int cin, bf16 *wq, bf16 *wt, cudaStream_t s) {
    const int n = cout * 9 * cin;
    pack_weights_kernel<<<div_up(n, 256), 256, 0, s>>>(w, cout, cin, wq, wt);
    return check_launch("refiner pack weights");
}

}  // namespace refiner
}  // namespace tde
