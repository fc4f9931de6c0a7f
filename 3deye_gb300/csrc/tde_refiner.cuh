// tde_refiner.cuh -- kernels of the learned depth refiner (a bf16 U-Net that
// predicts a residual for raw depth), shared by k_refiner.cu and the host
// module refiner.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tde {
namespace refiner {

typedef __nv_bfloat16 bf16;

// How a convolution reads its first input.
enum SrcMode { SRC_DIRECT = 0, SRC_POOL = 1, SRC_UP = 2 };

// 3x3 convolution (zero padding) as an implicit GEMM on the tensor cores:
// out[n,y,x,:cout] = epilogue(sum_t sum_ci in[n,y+dy_t,x+dx_t,ci] * w[co,t,ci]).
// The input is the channel concatenation of source A (ca channels, read
// directly, through a 2x2 max pool of a 2H x 2W tensor, or through a 2x
// nearest upsample of an H/2 x W/2 tensor) and source B (cb channels, H x W).
struct ConvArgs {
    const bf16 *a;
    int ca, mode_a;
    const bf16 *b;  // may be null (cb = 0)
    int cb;
    const bf16 *wgt;  // [cout][9][ca + cb]
    const float *bias;  // [cout] or null
    bf16 *out;          // [n][h][w][cout]
    int cout, relu;
    const bf16 *mask;  // null, or [n][h][w][cout]: out = 0 where mask <= 0
    // fused 1x1 head (cout == 16): depth_out = depth_in > 0 ? depth_in + 0.01 (w.out + b) : 0
    const float *head_w, *head_b, *depth_in;
    float *depth_out;     // may be null
    uint16_t *depth_mm;   // may be null: the same depth in mm, rounded, clamped to [0, 32767]
    int n, h, w;
    int *err;  // set to 1 when a wait on the tensor core timed out
    // optional: the 2x2 max pool of `out` ([n][h/2][w/2][cout]), written by
    // the same epilogue (h and w even)
    bf16 *pool_out;
};

// Weight gradient of the same convolution: partial[blk][r][co] with rows
// r = t * cin + ci (r = 9 * cin: bias), summed over the pixels block blk
// visits; reduced by launch_wgrad_reduce.
struct WgradArgs {
    const bf16 *a;
    int ca, mode_a;
    const bf16 *b;
    int cb;
    const bf16 *dz;  // [n][h][w][cout]
    int cout;
    int n, h, w;
    float *partial;
    int *err;
};

// Once per process and device, before any launch: shared-memory limits.
int prepare_kernels();
// Launch geometry of one convolution shape, fixed once: resident blocks per
// SM, input rows in each block's ring, dynamic shared memory per block.
struct ConvPlan {
    int per_sm, slots;
    size_t smem;
};
// ca of the cin input channels come from source A (the rest from B).
int conv_plan(int mode, int ca, int cin, int cout, ConvPlan *out);
// One lane waits, with the kernels' bounded wait, for a barrier phase nothing
// completes; out (device, 2 values): the raised flag and the nanoseconds waited.
int launch_wait_selftest(uint64_t limit_ns, unsigned long long *out, cudaStream_t s);
// Launches only (no other runtime call), so it may be stream-captured.
int launch_conv(const ConvArgs &a, const ConvPlan &plan, int num_sms, cudaStream_t s);
int wgrad_blocks(int num_sms, int cin, int cout);
size_t wgrad_partial_floats(int blocks, int cin, int cout);
int launch_wgrad(const WgradArgs &a, int blocks, cudaStream_t s);
// dw[co][t][ci] and db[co] from the partials of `blocks` blocks
int launch_wgrad_reduce(const float *partial, int blocks, int cin, int cout, float *dw, float *db, cudaStream_t s);

// Input preparation and the first convolution (3 features per tap -> 16
// channels, FP32 on the CUDA cores): depth_m = raw * 0.001 (0 when raw == 0),
// e0a = relu(conv).
int launch_conv_in(const uint16_t *raw, float *depth_m, const float *w1, const float *b1, bf16 *e0a, int n, int h,
                   int w, cudaStream_t s);
// Gradient of the first convolution: partial sums per block, then reduced.
int launch_conv_in_wgrad(const float *depth_m, const bf16 *dz1, int n, int h, int w, float *partial, int blocks,
                         float *dw1, float *db1, cudaStream_t s);
int conv_in_wgrad_blocks(int n, int h);

// Masked L1 loss against target depth (mm) on pixels valid in both, divided
// by n*h*w; with dr its gradient with respect to the head output,
// dz11 = bf16(dr * head_w * (d0 > 0)); head gradients; loss sum
// and valid-pixel count into loss2[0..1] (FP64).
int launch_loss(const float *out_m, const float *depth_m, const uint16_t *target, const bf16 *d0, const float *head_w,
                int n, int h, int w, bf16 *dz11, float *partial, int blocks, float *dhead_w, float *dhead_b,
                double *loss2, cudaStream_t s);
int loss_blocks(int n, int h, int w);

// dz[n,h/2,w/2,c] = bf16(sum_2x2 g[n,y,x,c] * (y_low > 0)), c < ca; g has cu channels.
int launch_up_back(const bf16 *g, int cu, int ca, const bf16 *y_low, bf16 *dz, int n, int h, int w, cudaStream_t s);
// dz[n,y,x,c] = bf16((skip[n,y,x,off+c] + first-argmax(e) ? gp[n,y/2,x/2,c] : 0) * (e > 0)), skip with cu channels.
int launch_pool_back_add(const bf16 *e, const bf16 *gp, const bf16 *skip, int cu, int off, int c, bf16 *dz, int n,
                         int h, int w, cudaStream_t s);

// AdamW on the flat parameter vector (decay applied where decay_mask != 0).
int launch_adamw(float *theta, const float *grad, float *m, float *v, const uint8_t *decay_mask, size_t count,
                 float lr, float beta1, float beta2, float eps, float wd, float bc1, float bc2, cudaStream_t s);

// bf16 copies of one convolution's weights: wq[co][t][ci] = w, and the
// transposed, tap-flipped copy the input gradient uses: wt[ci][8-t][co] = w.
int launch_pack_weights(const float *w, int cout, int cin, bf16 *wq, bf16 *wt, cudaStream_t s);

}  // namespace refiner
}  // namespace tde
