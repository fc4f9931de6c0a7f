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
// Weight gradient (wgrad_tc_kernel): M = 128 rows of (tap row, input
// channel), N = output channels, K = pixels, with MN-major operands read from
// the staged NHWC data; an all-ones operand gives the bias gradient.  Each
// block accumulates its share of the pixels in tensor memory and writes one
// partial; a reduction kernel sums the partials in a fixed order
// (deterministic).
#include <cuda_bf16.h>

#include <vector>

#include "tde_common.cuh"
#include "tde_refiner.cuh"
#include "tde_tc.cuh"

namespace tde {
namespace refiner {
namespace {

constexpr int kTileM = 128;             // output pixels per MMA tile
constexpr int kHaloW = kTileM + 2;      // halo pixels per row
constexpr int kWgK = 64;                // pixels per weight-gradient K step
constexpr int kWgHalo = kWgK + 2;
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
template <int MODE, typename Args>
__device__ __forceinline__ uint4 load_input_chunk(const Args &A, int img, int y, int x, int c) {
    if (y < 0 || y >= A.h || x < 0 || x >= A.w) return make_uint4(0u, 0u, 0u, 0u);
    const int cca = A.ca >> 3;
    if (c < cca) {
        if (MODE == SRC_DIRECT) return ldg16(A.a + (((size_t)img * A.h + y) * A.w + x) * A.ca + 8 * c);
        if (MODE == SRC_UP) {
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
template <typename Args>
__device__ __forceinline__ uint4 load_input_chunk(const Args &A, int img, int y, int x, int c) {
    if (A.mode_a == SRC_POOL) return load_input_chunk<SRC_POOL>(A, img, y, x, c);
    if (A.mode_a == SRC_UP) return load_input_chunk<SRC_UP>(A, img, y, x, c);
    return load_input_chunk<SRC_DIRECT>(A, img, y, x, c);
}

// ---------------------------------------------------------------------------
// Forward / input-gradient convolution: a warp-specialised pipeline.
//
// A block owns strips of consecutive output rows of one 128-pixel column
// tile.  Its warps have fixed roles, connected by mbarriers (no block-wide
// barrier in the steady state):
//   warps 4-7 (producers): input row j goes to warp 4 + (j & 3), which loads
//     the halo row (pixels x0-1 .. x0+128, every 8-channel chunk, as planes)
//     into ring slot j % S once the tensor core has released that slot, and
//     marks it full -- four rows in flight, one per warp;
//   warp 8, one lane (MMA issuer): output row r waits for its three input
//     rows and for a free accumulator (one of kConvAcc in tensor memory),
//     issues 9 taps x CC/2 MMAs (M = 128 pixels, N = cout, K = 16), and
//     commits them to the accumulator's "full" barrier and to the "empty"
//     barrier of the input row no later output row reads;
//   warps 0-3 (epilogue): TMEM lane quarter q of warp q, one pixel per
//     thread -- wait for the accumulator, read it (tcgen05.ld), apply bias,
//     ReLU, mask or the fused head, store bf16 NHWC, release the accumulator.
// Input rows are loaded once per strip; loads, MMAs and epilogues of
// different rows overlap.  Every wait is bounded: on a timeout the block
// raises A.err, all roles leave their loops, the issuer waits (bounded) for
// its MMAs in flight, and the tensor memory is freed.
// ---------------------------------------------------------------------------
constexpr int kConvEpiWarps = 4, kConvProdWarps = 4;
constexpr int kConvThreads = 32 * (kConvEpiWarps + kConvProdWarps + 1);  // + the MMA warp
constexpr int kConvMmaWarp = kConvEpiWarps + kConvProdWarps;
constexpr int kConvAcc = 4;       // accumulators in tensor memory
constexpr int kConvMaxSlots = 8;  // input-row ring
constexpr int kConvMinSlots = 4;
constexpr int kStripRowsOneWave = 8;   // longest strip of a one-wave launch
constexpr int kStripRowsBalanced = 16;  // strip length when the work is larger
constexpr uint64_t kConvWaitNs = 2000000000ull;

struct ConvPipe {
    uint64_t full[kConvMaxSlots], empty[kConvMaxSlots];
    uint64_t acc_full[kConvAcc], acc_empty[kConvAcc];
    uint64_t drain;
    uint32_t tmem;
    int abort;
};

// Bounded wait on an mbarrier phase; false when the block aborted (here or
// in another role).
__device__ __forceinline__ bool pipe_wait(uint64_t *bar, uint32_t parity, volatile int *abort, int *err,
                                          uint64_t limit_ns = kConvWaitNs) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = tc::globaltimer_ns();
    // sleeping waits (up to 20 us each) leave the issue slots to the working warps
    while (!tc::mbar_try_wait_sleep(bar, parity, 20000u)) {
        if (*abort) return false;
        if (tc::globaltimer_ns() - t0 > limit_ns) {
            *abort = 1;
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}
// The bounded wait on its own: one lane waits for a phase that nothing
// completes; after limit_ns it gives up, raises the error flag and the block
// returns normally.  out[0] = the flag, out[1] = nanoseconds waited.
__global__ void wait_selftest_kernel(uint64_t limit_ns, unsigned long long *out) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    __shared__ int err;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        abort_flag = 0;
        err = 0;
        const uint64_t t0 = tc::globaltimer_ns();
        const bool ok = pipe_wait(&bar, 0u, &abort_flag, &err, limit_ns);
        out[0] = ok ? 0ull : (unsigned long long)err;
        out[1] = tc::globaltimer_ns() - t0;
    }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

// Strip `item` of the block's sequence: image, column start, rows [y0, y1).
struct Strip { int img, x0, y0, y1; };
__device__ __forceinline__ Strip strip_of(const ConvArgs &A, int item, int rows_per_item) {
    const int tiles_x = (A.w + kTileM - 1) / kTileM;
    const int chunks = (A.h + rows_per_item - 1) / rows_per_item;
    Strip s;
    s.x0 = (item % tiles_x) * kTileM;
    s.y0 = ((item / tiles_x) % chunks) * rows_per_item;
    s.img = item / (tiles_x * chunks);
    s.y1 = min(A.h, s.y0 + rows_per_item);
    return s;
}

// One warp starts the copies of input row y (halo pixels x0-1 .. x0+128) into
// a slot as planes: CCA chunks of source A (read directly, or through the
// nearest 2x upsample of an h/2 x w/2 tensor), then CCB chunks of source B;
// 16-byte cp.async, zero outside the image; one commit group per row.
// Consecutive lanes copy consecutive 16-byte pieces of a source row.
template <int CP, bool UPS, int HALO = kHaloW>
__device__ __forceinline__ void warp_copy_part(const bf16 *row, int px_elems, int w, int x_start, int plane0, bool row_in,
                                               unsigned char *slot, const bf16 *dummy, int lane) {
    for (int i = lane; i < HALO * CP; i += 32) {
        const int px = i / CP, c = i - px * CP;
        const int x = x_start + px;
        const bool in = row_in && (unsigned)x < (unsigned)w;
        const bf16 *src = in ? row + (size_t)(UPS ? (x >> 1) : x) * px_elems + 8 * c : dummy;
        const uint32_t dst = tc::smem_u32(slot + ((size_t)(plane0 + c) * HALO + px) * 16);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(in ? 16 : 0)
                     : "memory");
    }
}
template <int MODE, int CCA, int CCB>
__device__ __forceinline__ void warp_issue_row(const ConvArgs &A, unsigned char *slot, int img, int y, int x0, int lane) {
    const bool row_in = y >= 0 && y < A.h;
    const int yc = row_in ? y : 0;
    if (MODE == SRC_UP) {
        const bf16 *ra = A.a + (((size_t)img * (A.h >> 1) + (yc >> 1)) * (A.w >> 1)) * A.ca;
        warp_copy_part<CCA, true>(ra, A.ca, A.w, x0 - 1, 0, row_in, slot, A.a, lane);
    } else {
        const bf16 *ra = A.a + (((size_t)img * A.h + yc) * A.w) * A.ca;
        warp_copy_part<CCA, false>(ra, A.ca, A.w, x0 - 1, 0, row_in, slot, A.a, lane);
    }
    if (CCB > 0) {
        const bf16 *rb = A.b + (((size_t)img * A.h + yc) * A.w) * A.cb;
        warp_copy_part<CCB, false>(rb, A.cb, A.w, x0 - 1, CCA, row_in, slot, A.a, lane);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Epilogue of one output row for one pixel (TMEM lane quarter of this warp).
// With a pooled output, `keep` holds the row's bf16 results when y is even;
// at the odd row below it the 2x2 maximum (the row pair in registers, the
// pixel pair across lanes x and x ^ 1) goes to pool_out -- the same bits as
// a max pool of the stored rows.
constexpr int kPoolMaxChunks = 8;  // pooled outputs have at most 64 channels
__device__ __forceinline__ void conv_epilogue(const ConvArgs &A, uint32_t tacc, int quarter, int lane, int img, int y,
                                              int x0, float depth_in, uint4 (&keep)[kPoolMaxChunks],
                                              const float *s_bias, const float *s_head) {
    const int m = quarter * 32 + lane;
    const int x = x0 + m;
    const bool valid = x < A.w;
    const size_t pix = ((size_t)img * A.h + y) * A.w + (valid ? x : 0);
    const bool pool_row = A.pool_out && (y & 1);
    const size_t ppix = ((size_t)img * (A.h >> 1) + (y >> 1)) * (A.w >> 1) + (valid ? (x >> 1) : 0);
    float r = 0.f;
    for (int j = 0; j < A.cout; j += 16) {
        float v[16];
        tc::tmem_ld16(tacc + ((uint32_t)(quarter * 32) << 16) + (uint32_t)j, v);
        if (A.bias) {
#pragma unroll
            for (int k = 0; k < 16; ++k) v[k] += s_bias[j + k];
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
        if (valid) {
            uint4 *o = reinterpret_cast<uint4 *>(A.out + pix * A.cout + j);
            o[0] = q0;
            o[1] = q1;
        }
        if (A.pool_out) {
            const int c = j >> 3;
            if (!pool_row) {
                keep[c] = q0;
                keep[c + 1] = q1;
            } else {
                uint4 p0 = bmax4(keep[c], q0), p1 = bmax4(keep[c + 1], q1);
                uint4 n0, n1;
                n0.x = __shfl_xor_sync(0xffffffffu, p0.x, 1); n0.y = __shfl_xor_sync(0xffffffffu, p0.y, 1);
                n0.z = __shfl_xor_sync(0xffffffffu, p0.z, 1); n0.w = __shfl_xor_sync(0xffffffffu, p0.w, 1);
                n1.x = __shfl_xor_sync(0xffffffffu, p1.x, 1); n1.y = __shfl_xor_sync(0xffffffffu, p1.y, 1);
                n1.z = __shfl_xor_sync(0xffffffffu, p1.z, 1); n1.w = __shfl_xor_sync(0xffffffffu, p1.w, 1);
                if (valid && !(x & 1)) {
                    uint4 *o = reinterpret_cast<uint4 *>(A.pool_out + ppix * A.cout + j);
                    o[0] = bmax4(p0, n0);
                    o[1] = bmax4(p1, n1);
                }
            }
        }
        if (A.head_w && valid) {
            float f[16];
            unpack8(q0, f);
            unpack8(q1, f + 8);
#pragma unroll
            for (int k = 0; k < 16; ++k) r = fmaf(s_head[k], f[k], r);
        }
    }
    if (valid && A.head_w) {
        const float o = depth_in > 0.f ? depth_in + 0.01f * (r + s_head[16]) : 0.f;  // residual in cm
        if (A.depth_out) A.depth_out[pix] = o;
        if (A.depth_mm) {
            const float mm = fminf(fmaxf(rintf(o * 1000.f), 0.f), (float)TDE_MAX_DEPTH_VALUE);
            A.depth_mm[pix] = (uint16_t)mm;
        }
    }
}

template <int MODE, int CCA, int CCB>
__global__ void __launch_bounds__(kConvThreads) conv3x3_tc_kernel(const ConvArgs A, int rows_per_item, int S) {
    constexpr int CC = CCA + CCB;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ ConvPipe pp;
    __shared__ float s_bias[128], s_head[17];  // bias; head weights and head bias
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr uint32_t slot_bytes = (uint32_t)CC * kHaloW * 16;
    unsigned char *halo = smem;
    unsigned char *wsm = smem + (size_t)S * slot_bytes;
    const uint32_t ncols = tmem_cols(A.cout);
    const uint32_t tcols = kConvAcc * ncols;
    volatile int *abort = &pp.abort;

    // the next layer may start its prologue; it waits for this grid before
    // reading anything this one writes
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (warp == kConvMmaWarp) tc::tmem_alloc(&pp.tmem, tcols);
    if (tid == 0) {
        for (int s = 0; s < kConvMaxSlots; ++s) {
            tc::mbar_init(&pp.full[s], 1);
            tc::mbar_init(&pp.empty[s], 1);
        }
        for (int a = 0; a < kConvAcc; ++a) {
            tc::mbar_init(&pp.acc_full[a], 1);
            tc::mbar_init(&pp.acc_empty[a], kConvEpiWarps);
        }
        tc::mbar_init(&pp.drain, 1);
        pp.abort = 0;
    }
    if (A.bias && tid < A.cout) s_bias[tid] = A.bias[tid];
    if (A.head_w && tid < 17) s_head[tid] = tid < 16 ? A.head_w[tid] : A.head_b[0];
    // weights: global [co][t][ci] -> planes (t, chunk) of cout rows x 16 B.
    // No kernel launched right before a convolution writes weights, so they
    // are fetched before waiting for the previous grid.
    {
        const int nw = A.cout * 9 * CC;
        for (int i = tid; i < nw; i += kConvThreads) {
            const int c = i % CC, t = (i / CC) % 9, co = i / (9 * CC);
            const uint32_t dst = tc::smem_u32(wsm + ((size_t)(t * CC + c) * A.cout + co) * 16);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(A.wgt + (size_t)i * 8) : "memory");
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = pp.tmem;
    const int tiles_x = (A.w + kTileM - 1) / kTileM;
    const int items = A.n * tiles_x * ((A.h + rows_per_item - 1) / rows_per_item);

    if (warp >= kConvEpiWarps && warp < kConvMmaWarp) {
        // ---- producers: warp pw loads the input rows j = pw (mod 4), two in
        // flight; a row is marked full once its copies have landed ----
        const int pw = warp - kConvEpiWarps;
        uint32_t j = 0;                  // this block's input-row sequence
        int pending = -1;                // slot of the row issued before the current one
        bool ok = true;
        auto publish = [&](int wait_groups) {
            if (pending < 0) return;
            if (wait_groups) asm volatile("cp.async.wait_group 1;" ::: "memory");
            else asm volatile("cp.async.wait_group 0;" ::: "memory");
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&pp.full[pending]);
            pending = -1;
        };
        for (int item = blockIdx.x; item < items && ok && !*abort; item += gridDim.x) {
            const Strip st = strip_of(A, item, rows_per_item);
            const int nin = st.y1 - st.y0 + 2;
            for (int i = 0; i < nin; ++i, ++j) {
                if ((int)(j & 3u) != pw) continue;
                const uint32_t s = j % (uint32_t)S, k = j / (uint32_t)S;
                if (k > 0) {
                    // the MMA that frees this slot reads input rows up to
                    // j - S + 2; when that reaches this warp's previous row
                    // (j - 4, S <= 6), publish it before waiting
                    if (S <= 6) publish(0);
                    if (!(ok = pipe_wait(&pp.empty[s], (k - 1) & 1u, abort, A.err))) break;
                }
                warp_issue_row<MODE, CCA, CCB>(A, halo + (size_t)s * slot_bytes, st.img, st.y0 - 1 + i, st.x0, lane);
                publish(1);  // the previous row of this warp, while this one is in flight
                pending = (int)s;
            }
        }
        publish(0);
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else if (warp == kConvMmaWarp) {
        // ---- MMA issuer ----
        if (lane == 0) {
            const uint32_t halo_s = tc::smem_u32(halo), w_s = tc::smem_u32(wsm);
            const uint32_t idesc = tc::idesc_bf16(kTileM, A.cout);
            // descriptor bases: A at a slot's first plane (LBO = plane stride),
            // B at the first weight plane; an MMA adds its byte offset >> 4
            const uint64_t a_desc0 = tc::desc(halo_s, kHaloW * 16, 128);
            const uint64_t b_desc0 = tc::desc(w_s, A.cout * 16, 128);
            const uint32_t b_plane = (uint32_t)A.cout * 16;
            uint32_t jin = 0, waited = 0, q = 0;  // input rows of earlier strips, rows known full, output rows
            bool ok = true;
            for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
                const Strip st = strip_of(A, item, rows_per_item);
                const int R = st.y1 - st.y0;
                for (int o = 0; o < R && ok; ++o, ++q) {
                    // its input rows jin + o .. jin + o + 2
                    for (; waited <= jin + o + 2 && ok; ++waited)
                        ok = pipe_wait(&pp.full[waited % (uint32_t)S], (waited / (uint32_t)S) & 1u, abort, A.err);
                    const uint32_t a = q % kConvAcc, ka = q / kConvAcc;
                    if (ok && ka > 0) ok = pipe_wait(&pp.acc_empty[a], (ka - 1) & 1u, abort, A.err);
                    if (!ok) break;
                    tc::fence_after_sync();
                    const uint32_t dacc = tmem + a * ncols;
#pragma unroll
                    for (int t = 0; t < 9; ++t) {
                        const int dy = t / 3, dx = t % 3;
                        const uint32_t a_off = ((jin + o + dy) % (uint32_t)S) * slot_bytes + dx * 16;
#pragma unroll
                        for (int kc = 0; kc < CC; kc += 2) {
                            const uint64_t ad = a_desc0 + ((a_off + (uint32_t)kc * kHaloW * 16) >> 4);
                            const uint64_t bd = b_desc0 + (((uint32_t)(t * CC + kc) * b_plane) >> 4);
                            tc::mma_bf16(dacc, ad, bd, idesc, (t | kc) ? 1u : 0u);
                        }
                    }
                    tc::commit(&pp.acc_full[a]);
                    // input row o is read by no later output row of the strip;
                    // after the last output row, neither are the two below it
                    tc::commit(&pp.empty[(jin + o) % (uint32_t)S]);
                    if (o == R - 1) {
                        tc::commit(&pp.empty[(jin + o + 1) % (uint32_t)S]);
                        tc::commit(&pp.empty[(jin + o + 2) % (uint32_t)S]);
                    }
                }
                jin += (uint32_t)(R + 2);
            }
            // every MMA issued has finished before the tensor memory is freed
            tc::commit(&pp.drain);
            tc::mbar_wait(&pp.drain, 0u, kConvWaitNs);
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp q drains TMEM lanes 32q .. 32q + 31 ----
        uint32_t q = 0;
        uint4 keep[kPoolMaxChunks];
        for (int item = blockIdx.x; item < items && !*abort; item += gridDim.x) {
            const Strip st = strip_of(A, item, rows_per_item);
            bool ok = true;
            for (int y = st.y0; y < st.y1; ++y, ++q) {
                const int x = st.x0 + warp * 32 + lane;
                float din = 0.f;  // the head's input depth, fetched before the wait
                if (A.head_w && x < A.w) din = __ldg(A.depth_in + ((size_t)st.img * A.h + y) * A.w + x);
                const uint32_t a = q % kConvAcc, ka = q / kConvAcc;
                if (!(ok = pipe_wait(&pp.acc_full[a], ka & 1u, abort, A.err))) break;
                tc::fence_after_sync();
                conv_epilogue(A, tmem + a * ncols, warp, lane, st.img, y, st.x0, din, keep, s_bias, s_head);
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(&pp.acc_empty[a]);
            }
            if (!ok) break;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == kConvMmaWarp) tc::tmem_dealloc(tmem, tcols);
}

// (mode, input chunks) pairs the network uses: forward c2..c11 (the encoder's
// pooled inputs come precomputed from the epilogue of the layer before) and
// the input gradients of c2..c11 (direct sources with cout/8 chunks)
#define TDE_CONV_VARIANTS(X) \
    X(SRC_DIRECT, 2, 0) X(SRC_DIRECT, 4, 0) X(SRC_DIRECT, 6, 0) X(SRC_DIRECT, 8, 0) \
    X(SRC_UP, 4, 2) X(SRC_UP, 6, 4) X(SRC_UP, 8, 6)

// The kernel for a source mode and the input chunks of sources A and B.
const void *conv_kernel_fn(int mode, int cca, int ccb) {
#define TDE_CONV_FN(M, A, B) \
    if (mode == M && cca == A && ccb == B) return (const void *)conv3x3_tc_kernel<M, A, B>;
    TDE_CONV_VARIANTS(TDE_CONV_FN)
#undef TDE_CONV_FN
    return nullptr;
}

// ---------------------------------------------------------------------------
// Weight gradient
//
// dW[co][t][ci] = sum_p dZ[p][co] X[p + s_t][ci] as D = A B with K = pixels,
// both operands MN-major: the tensor core reads the staged NHWC data as it
// lies.  X is staged per 64-pixel step as planes of 8-channel chunks (3 rows
// x 66 halo pixels, 16 B per pixel); for horizontal tap offset dx, the rows
// (dy, ci) of A are the planes in order (a uniform chunk stride) and the
// pixel window starts dx pixels later (16 * dx bytes).  dZ is staged the same
// way (planes of 8 output channels).  The bias gradient is the same MMA with
// a constant all-ones A.  Without swizzling, a descriptor's LBO is the stride
// between 8-element groups along K and its SBO the stride along M (or N), for
// MN-major operands as for K-major ones.
// ---------------------------------------------------------------------------
constexpr int kWgPlaneX = kWgHalo * 16;   // 1056 B: one 8-channel plane of X
constexpr int kWgPlaneZ = kWgK * 16;      // 1024 B: one 8-channel plane of dZ

struct WgLayout {
    int cin, cc, mtiles, xplanes, zplanes;
    uint32_t x_bytes, z_bytes, tcols;
};
__host__ __device__ inline WgLayout wg_layout(int cin, int cout) {
    WgLayout L;
    L.cin = cin;
    L.cc = cin / 8;
    L.mtiles = (3 * cin + 127) / 128;                 // rows (dy, ci) per horizontal offset
    L.xplanes = max(3 * L.cc, 16 * L.mtiles);         // MMAs read whole 16-chunk row tiles
    L.zplanes = cout / 8;
    L.x_bytes = (uint32_t)(L.xplanes * kWgPlaneX);
    L.z_bytes = (uint32_t)(L.zplanes * kWgPlaneZ);
    L.tcols = (uint32_t)(3 * L.mtiles * cout + cout);  // 3 dx x row tiles, + bias
    return L;
}

// MN-major kind::f16 instruction descriptor (bits 15, 16 = 1).
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N) {
    return tc::idesc_bf16(M, N) | (1u << 15) | (1u << 16);
}

// Pipelined form: a block owns K steps k = blockIdx.x, + gridDim.x, ... (one
// 64-pixel segment of one row each).  Up to 8 producer warps stage step k --
// X over 3 rows x 66 halo pixels and dZ over 64 pixels, as planes, with
// cp.async -- into ring stage k % S once the tensor core has released it
// (step k - S done), warp k % min(S, 8) taking step k; warp 8, one lane, issues each
// step's MMAs into the block's accumulators (3 dx x row tiles + the bias
// column block), which stay in tensor memory across all the block's steps,
// and commits them to the stage's "empty" barrier.  At the end every warp
// drains the accumulators into the block's partial.  Bounded waits as in the
// convolution: a timeout raises A.err and the block leaves cleanly.
constexpr int kWgProdWarps = 8;
constexpr int kWgThreadsP = 32 * (kWgProdWarps + 1);
constexpr int kWgMaxStages = 8;
struct WgPipe {
    uint64_t full[kWgMaxStages], empty[kWgMaxStages], drain;
    uint32_t tmem;
    int abort;
};

template <int MODE, int CCA, int CCB>
__global__ void __launch_bounds__(kWgThreadsP) wgrad_tc_kernel(const WgradArgs A, int S) {
    constexpr int CC = CCA + CCB;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ WgPipe pp;
    const int cin = A.ca + A.cb, cout = A.cout;
    const WgLayout L = wg_layout(cin, cout);
    const int zc = cout / 8;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols = tmem_cols((int)L.tcols);
    const uint32_t stage_bytes = L.x_bytes + L.z_bytes;
    unsigned char *ones = smem + (size_t)S * stage_bytes;
    volatile int *abort = &pp.abort;

    if (warp == kWgProdWarps) tc::tmem_alloc(&pp.tmem, ncols);
    if (tid == 0) {
        for (int s = 0; s < kWgMaxStages; ++s) {
            tc::mbar_init(&pp.full[s], 1);
            tc::mbar_init(&pp.empty[s], 1);
        }
        tc::mbar_init(&pp.drain, 1);
        pp.abort = 0;
    }
    {
        const uint4 one8 = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);  // eight bf16 1.0
        for (int i = tid; i < 256; i += kWgThreadsP) *reinterpret_cast<uint4 *>(ones + (size_t)i * 16) = one8;
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = pp.tmem;
    const int tiles_x = (A.w + kWgK - 1) / kWgK;
    const int ntiles = A.n * A.h * tiles_x;
    // this block's steps: k-th step is tile blockIdx.x + k * gridDim.x
    const int nsteps = blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    // Producer warps: no more than the ring has stages, so that the stage a
    // warp waits for was released one phase ago at most (a parity wait cannot
    // tell phase f - 1 from f - 3): steps are released in order, and a warp's
    // previous wait already covered step k - np - S >= k - 2S.
    const int np = S < kWgProdWarps ? S : kWgProdWarps;
    if (warp < np) {
        // ---- producers ----
        for (int k = warp; k < nsteps && !*abort; k += np) {
            const uint32_t s = (uint32_t)k % (uint32_t)S, f = (uint32_t)k / (uint32_t)S;
            if (f > 0 && !pipe_wait(&pp.empty[s], (f - 1) & 1u, abort, A.err)) break;
            const int tile = blockIdx.x + k * gridDim.x;
            const int xt = tile % tiles_x, rowi = tile / tiles_x;
            const int y = rowi % A.h, img = rowi / A.h;
            const int x0 = xt * kWgK;
            unsigned char *xs = smem + (size_t)s * stage_bytes;
            unsigned char *zs = xs + L.x_bytes;
            // X: planes (dy, c) of 66 halo pixels; consecutive lanes take
            // consecutive 16-byte pieces of a source pixel row
#pragma unroll 1
            for (int dy = 0; dy < 3; ++dy) {
                const int yy = y + dy - 1;
                const bool row_in = yy >= 0 && yy < A.h;
                const int yc = row_in ? yy : 0;
                if (MODE == SRC_UP) {
                    const bf16 *ra = A.a + (((size_t)img * (A.h >> 1) + (yc >> 1)) * (A.w >> 1)) * A.ca;
                    warp_copy_part<CCA, true, kWgHalo>(ra, A.ca, A.w, x0 - 1, dy * CC, row_in, xs, A.a, lane);
                } else {
                    const bf16 *ra = A.a + (((size_t)img * A.h + yc) * A.w) * A.ca;
                    warp_copy_part<CCA, false, kWgHalo>(ra, A.ca, A.w, x0 - 1, dy * CC, row_in, xs, A.a, lane);
                }
                if (CCB > 0) {
                    const bf16 *rb = A.b + (((size_t)img * A.h + yc) * A.w) * A.cb;
                    warp_copy_part<CCB, false, kWgHalo>(rb, A.cb, A.w, x0 - 1, dy * CC + CCA, row_in, xs, A.a, lane);
                }
            }
            // dZ: planes of 8 output channels over 64 pixels, zero past the row end
            for (int i = lane; i < kWgK * zc; i += 32) {
                const int c = i % zc, px = i / zc;
                const bool in = x0 + px < A.w;
                const bf16 *src = in ? A.dz + (((size_t)img * A.h + y) * A.w + x0 + px) * cout + 8 * c : A.dz;
                const uint32_t dst = tc::smem_u32(zs + (size_t)c * kWgPlaneZ + px * 16);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(in ? 16 : 0)
                             : "memory");
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&pp.full[s]);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else if (warp == kWgProdWarps && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t s0 = tc::smem_u32(smem), ones_s = tc::smem_u32(ones);
        const uint32_t idesc = idesc_bf16_mn(128, cout);
        for (int k = 0; k < nsteps; ++k) {
            const uint32_t s = (uint32_t)k % (uint32_t)S;
            if (!pipe_wait(&pp.full[s], ((uint32_t)k / (uint32_t)S) & 1u, abort, A.err)) break;
            tc::fence_after_sync();
            const uint32_t xb = s0 + s * stage_bytes, zb = xb + L.x_bytes;
            for (int kk = 0; kk < kWgK / 16; ++kk) {
                const uint32_t acc = (k == 0 && kk == 0) ? 0u : 1u;
                const uint64_t bd = tc::desc(zb + (uint32_t)(kk * 16 * 16), 128, kWgPlaneZ);
                for (int dx = 0; dx < 3; ++dx)
                    for (int mt = 0; mt < L.mtiles; ++mt) {
                        const uint64_t ad =
                            tc::desc(xb + (uint32_t)(16 * mt * kWgPlaneX + (kk * 16 + dx) * 16), 128, kWgPlaneX);
                        tc::mma_bf16(tmem + (uint32_t)((dx * L.mtiles + mt) * cout), ad, bd, idesc, acc);
                    }
                const uint64_t od = tc::desc(ones_s, 128, 256);
                tc::mma_bf16(tmem + (uint32_t)(3 * L.mtiles * cout), od, bd, idesc, acc);
            }
            tc::commit(&pp.empty[s]);
        }
        // every MMA issued has finished before the accumulators are read
        tc::commit(&pp.drain);
        if (!tc::mbar_wait(&pp.drain, 0u, kConvWaitNs)) {
            *abort = 1;
            atomicExch(A.err, 1);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (!*abort && warp < kWgProdWarps) {
        // rows R = dx * mtiles * 128 + (dy * cin + ci), bias row R = 3 * mtiles * 128;
        // warps w and w + 4 share TMEM lane quarter w % 4 and split the tiles
        const int q = warp & 3;
        const size_t rows_pad = (size_t)3 * L.mtiles * 128 + 1;
        float *dst = A.partial + (size_t)blockIdx.x * rows_pad * cout;
        const int ntile = 3 * L.mtiles + 1;
        for (int tl = 0; tl < ntile; ++tl) {
            if ((tl & 1) != (warp >> 2)) continue;
            for (int j = 0; j < cout; j += 16) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(tl * cout + j), v);
                if (nsteps == 0) {
#pragma unroll
                    for (int e = 0; e < 16; ++e) v[e] = 0.f;
                }
                const int rr = q * 32 + lane;
                if (tl < 3 * L.mtiles) {
                    const size_t r = (size_t)tl * 128 + rr;
                    float4 *o = reinterpret_cast<float4 *>(dst + r * cout + j);
#pragma unroll
                    for (int e = 0; e < 4; ++e) o[e] = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
                } else if (rr == 0) {
                    float4 *o = reinterpret_cast<float4 *>(dst + (rows_pad - 1) * cout + j);
#pragma unroll
                    for (int e = 0; e < 4; ++e) o[e] = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == kWgProdWarps) tc::tmem_dealloc(tmem, ncols);
}

// The weight-gradient kernel for a source mode and the input chunks of
// sources A and B (the convolutions' own variants).
const void *wgrad_kernel_fn(int mode, int cca, int ccb) {
#define TDE_WG_FN(M, A, B) \
    if (mode == M && cca == A && ccb == B) return (const void *)wgrad_tc_kernel<M, A, B>;
    TDE_CONV_VARIANTS(TDE_WG_FN)
#undef TDE_WG_FN
    return nullptr;
}

// Fixed-order sum of `blocks` partial vectors of n floats ([blocks][n]): a
// block takes 32 consecutive elements (coalesced); warp w sums the partials
// w, w + 8, ... with eight loads in flight, then the eight warp sums are added
// in warp order.  Deterministic; the partials' latency is paid about
// blocks / 64 times instead of `blocks` times.
__device__ __forceinline__ bool sum_partials(const float *__restrict__ partial, int blocks, int n, int &e,
                                             float &total) {
    __shared__ float part[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    e = blockIdx.x * 32 + lane;
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 0.f;
    if (e < n) {
        int b = w;
        for (; b + 56 < blocks; b += 64) {
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] += __ldg(partial + (size_t)(b + 8 * k) * n + e);
        }
        for (int k = 0; b < blocks; b += 8, ++k) a[k & 7] += __ldg(partial + (size_t)b * n + e);
    }
    part[w][lane] = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    __syncthreads();
    if (w != 0 || e >= n) return false;
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += part[k][lane];
    total = t;
    return true;
}

// Weight gradients from the per-block partials [blocks][rows_pad][cout]: row
// r = dx * mtiles * 128 + dy * cin + ci (rows past 3 cin of a dx are padding),
// the last row the bias; dw[(co * 9 + 3 dy + dx) * cin + ci].
__global__ void __launch_bounds__(256) wgrad_reduce_kernel(const float *__restrict__ partial, int blocks, int cin,
                                                           int cout, int mtiles, float *__restrict__ dw,
                                                           float *__restrict__ db) {
    const int rows_pad = 3 * mtiles * 128 + 1;
    int e;
    float t;
    if (!sum_partials(partial, blocks, rows_pad * cout, e, t)) return;
    const int r = e / cout, co = e % cout;
    if (r == rows_pad - 1) {
        db[co] = t;
        return;
    }
    const int dx = r / (mtiles * 128), rem = r % (mtiles * 128);
    if (rem >= 3 * cin) return;
    const int dy = rem / cin, ci = rem % cin;
    dw[((size_t)co * 9 + 3 * dy + dx) * cin + ci] = t;
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
    extern __shared__ float rows3[];  // depth rows y-1, y, y+1 with a zero column either side: 3 x (w + 2)
    __shared__ float red[16][16][kInK + 1];
    const int co = threadIdx.x & 15, pl = threadIdx.x >> 4;
    const int W2 = w + 2;
    float s[kInK + 1];
#pragma unroll
    for (int k = 0; k <= kInK; ++k) s[k] = 0.f;
    const int row0 = blockIdx.x * kInRowsPerBlock;
    for (int rr = 0; rr < kInRowsPerBlock; ++rr) {
        const int rowi = row0 + rr;
        if (rowi >= n * h) break;
        const int y = rowi % h, img = rowi / h;
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * W2; i += blockDim.x) {
            const int r = i / W2, x = i % W2 - 1, yy = y + r - 1;
            rows3[i] = (x >= 0 && x < w && yy >= 0 && yy < h) ? depth_m[((size_t)img * h + yy) * w + x] : 0.f;
        }
        __syncthreads();
        for (int x = pl; x < w; x += 16) {
            const size_t p = ((size_t)img * h + y) * w + x;
            const float g = __bfloat162float(dz1[p * 16 + co]);
            if (g == 0.f) continue;
            float d[9];
#pragma unroll
            for (int t = 0; t < 9; ++t) d[t] = rows3[(t / 3) * W2 + x + t % 3];
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

__global__ void __launch_bounds__(256) conv_in_wgrad_reduce_kernel(const float *__restrict__ partial, int blocks,
                                                                   float *__restrict__ dw1, float *__restrict__ db1) {
    int i;  // c * 28 + k
    float t;
    if (!sum_partials(partial, blocks, kInPartial, i, t)) return;
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

// One block per reduced quantity; a fixed-shape tree over the block partials.
__global__ void loss_reduce_kernel(const float *__restrict__ partial, int blocks, float *__restrict__ dhead_w,
                                   float *__restrict__ dhead_b, double *__restrict__ loss2) {
    __shared__ double red[256];
    const int k = blockIdx.x;
    double t = 0.0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) t += (double)partial[(size_t)b * 19 + k];
    red[threadIdx.x] = t;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (k < 2) loss2[k] = red[0];
        else if (k < 18) dhead_w[k - 2] = (float)red[0];
        else dhead_b[0] = (float)red[0];
    }
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

int prepare_kernels() {
    // allow the largest dynamic shared memory a block may have, once, so that
    // launches (also inside stream capture) make no other runtime call
    std::vector<const void *> fns;
#define TDE_CONV_FN(M, A, B) \
    fns.push_back((const void *)conv3x3_tc_kernel<M, A, B>); \
    fns.push_back((const void *)wgrad_tc_kernel<M, A, B>);
    TDE_CONV_VARIANTS(TDE_CONV_FN)
#undef TDE_CONV_FN
    for (const void *fn : fns) {
        cudaFuncAttributes fa;
        TDE_CUDA(cudaFuncGetAttributes(&fa, fn), "refiner: kernel attributes");
        TDE_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(227 * 1024 - fa.sharedSizeBytes)),
                 "refiner: shared memory limit");
    }
    return TDE_OK;
}

int conv_plan(int mode, int ca, int cin, int cout, ConvPlan *out) {
    // Two resident blocks per SM when the tensor memory, the registers and the
    // shared memory allow them at least kConvMinSlots input rows each, else
    // one; the ring takes as many rows (up to kConvMaxSlots) as then fit.  The
    // shared memory is padded so that no further block becomes resident.
    const void *fn = conv_kernel_fn(mode, ca / 8, (cin - ca) / 8);
    if (!fn) return set_error(TDE_ERR_UNSUPPORTED, "refiner conv: no kernel for mode %d with %d + %d input channels", mode,
                              ca, cin - ca);
    cudaFuncAttributes fa;
    TDE_CUDA(cudaFuncGetAttributes(&fa, fn), "refiner: kernel attributes");
    const size_t slot = (size_t)(cin / 8) * kHaloW * 16, wb = (size_t)9 * (cin / 8) * cout * 16;
    const int by_tmem = (int)(512u / (kConvAcc * tmem_cols(cout)));
    const int by_regs = 65536 / (((fa.numRegs + 7) / 8) * 8 * kConvThreads);
    int bps = by_tmem < by_regs ? by_tmem : by_regs;
    bps = bps > 2 ? 2 : bps;
    for (; bps >= 1; --bps) {
        const size_t budget = kSmemPerSM / bps - 1024 - fa.sharedSizeBytes;
        if (budget < wb + kConvMinSlots * slot) continue;
        size_t S = (budget - wb) / slot;
        S = S > (size_t)kConvMaxSlots ? (size_t)kConvMaxSlots : S;
        size_t smem = S * slot + wb;
        const size_t floor = kSmemPerSM / (bps + 1) - 1024 - fa.sharedSizeBytes + 16;
        if (smem < floor) smem = floor;
        out->per_sm = bps;
        out->slots = (int)S;
        out->smem = smem;
        return TDE_OK;
    }
    return set_error(TDE_ERR_UNSUPPORTED, "refiner conv: cin=%d cout=%d does not fit an SM", cin, cout);
}

int launch_conv(const ConvArgs &a, const ConvPlan &plan, int num_sms, cudaStream_t s) {
    const int cin = a.ca + a.cb;
    if (cin % 16 || a.ca % 8 || a.cout % 16 || a.cout < 16 || a.cout > 128 || cin > 128 || a.w <= 0 || a.h <= 0 ||
        a.n <= 0 || (a.head_w && a.cout != 16) || (a.mode_a == SRC_UP && (a.h % 2 || a.w % 2)) ||
        (a.pool_out && (a.h % 2 || a.w % 2 || a.cout > 8 * kPoolMaxChunks)))
        return set_error(TDE_ERR_INVALID_ARG, "refiner conv: unsupported shape cin=%d cout=%d", cin, a.cout);
    if (plan.slots < kConvMinSlots || plan.slots > kConvMaxSlots || plan.per_sm < 1 || plan.smem > 227 * 1024 - 256)
        return set_error(TDE_ERR_INVALID_ARG, "refiner conv: bad launch plan");
    // rows per block: as many as keep every resident block busy
    const int tiles_x = (a.w + kTileM - 1) / kTileM;
    const long row_tiles = (long)a.n * a.h * tiles_x;
    const long slots = (long)num_sms * plan.per_sm;
    // rows per strip: enough that the strips do not outnumber the resident
    // blocks (no second wave), even when the epilogue pools row pairs; with
    // more work than that (training batches), short strips that the resident
    // blocks take in turn, which balances their load better than long ones
    int rows = (int)((row_tiles + slots - 1) / slots);
    rows = rows < 1 ? 1 : rows > kStripRowsOneWave ? kStripRowsBalanced : rows;
    if (a.pool_out) rows += rows & 1;
    const long items = (long)a.n * tiles_x * ((a.h + rows - 1) / rows);
    const int grid = (int)(items < slots ? items : slots);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kConvThreads);
    cfg.dynamicSmemBytes = plan.smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const void *fn = conv_kernel_fn(a.mode_a, a.ca / 8, a.cb / 8);
    if (!fn) return set_error(TDE_ERR_UNSUPPORTED, "refiner conv: no kernel for mode %d with %d + %d input channels",
                              a.mode_a, a.ca, a.cb);
    int S = plan.slots;
    void *args[] = {(void *)&a, (void *)&rows, (void *)&S};
    cudaError_t e = cudaLaunchKernelExC(&cfg, fn, args);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "refiner conv: %s", cudaGetErrorString(e));
    return check_launch("refiner conv");
}

int wgrad_blocks(int num_sms, int cin, int cout) {
    (void)cin;
    (void)cout;
    return num_sms;
}

size_t wgrad_partial_floats(int blocks, int cin, int cout) {
    const WgLayout L = wg_layout(cin, cout);
    return (size_t)blocks * ((size_t)3 * L.mtiles * 128 + 1) * cout;
}

int launch_wgrad(const WgradArgs &a, int blocks, cudaStream_t s) {
    const int cin = a.ca + a.cb;
    const WgLayout L = wg_layout(cin, a.cout);
    if (cin % 8 || a.cout % 16 || a.cout < 16 || L.tcols > 512 || a.mode_a == SRC_POOL)
        return set_error(TDE_ERR_INVALID_ARG, "refiner wgrad: unsupported shape cin=%d cout=%d", cin, a.cout);
    // as many ring stages as one block per SM holds (the ones tile after them)
    const size_t stage = (size_t)L.x_bytes + L.z_bytes, ones = 16u * 256u;
    const size_t budget = 227 * 1024 - 512 - ones;
    int S = (int)(budget / stage);
    S = S > kWgMaxStages ? kWgMaxStages : S;
    if (S < 2) return set_error(TDE_ERR_UNSUPPORTED, "refiner wgrad: cin=%d cout=%d does not fit an SM", cin, a.cout);
    size_t smem = (size_t)S * stage + ones;
    const size_t fl = smem_floor_for_tmem(tmem_cols((int)L.tcols));
    if (smem < fl) smem = fl;
    const void *fn = wgrad_kernel_fn(a.mode_a, a.ca / 8, a.cb / 8);
    if (!fn) return set_error(TDE_ERR_UNSUPPORTED, "refiner wgrad: no kernel for mode %d with %d + %d input channels",
                              a.mode_a, a.ca, a.cb);
    WgradArgs args = a;
    void *kargs[] = {(void *)&args, (void *)&S};
    cudaError_t e = cudaLaunchKernel(fn, dim3(blocks), dim3(kWgThreadsP), kargs, smem, s);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "refiner wgrad: %s", cudaGetErrorString(e));
    return check_launch("refiner wgrad");
}

int launch_wait_selftest(uint64_t limit_ns, unsigned long long *out, cudaStream_t s) {
    wait_selftest_kernel<<<1, 32, 0, s>>>(limit_ns, out);
    return check_launch("wait selftest");
}

int launch_wgrad_reduce(const float *partial, int blocks, int cin, int cout, float *dw, float *db, cudaStream_t s) {
    const WgLayout L = wg_layout(cin, cout);
    const int n = (3 * L.mtiles * 128 + 1) * cout;
    wgrad_reduce_kernel<<<div_up(n, 32), 256, 0, s>>>(partial, blocks, cin, cout, L.mtiles, dw, db);
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
    const size_t rows_bytes = (size_t)3 * (w + 2) * sizeof(float);
    if (rows_bytes + sizeof(float) * 16 * 16 * (kInK + 1) > 48 * 1024)
        return set_error(TDE_ERR_UNSUPPORTED, "refiner: %d columns exceed the input-layer gradient kernel", w);
    conv_in_wgrad_kernel<<<blocks, 256, rows_bytes, s>>>(depth_m, dz1, n, h, w, partial);
    TDE_TRY(check_launch("refiner conv_in wgrad"));
    conv_in_wgrad_reduce_kernel<<<div_up(kInPartial, 32), 256, 0, s>>>(partial, blocks, dw1, db1);
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
    loss_reduce_kernel<<<19, 256, 0, s>>>(partial, blocks, dhead_w, dhead_b, loss2);
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
