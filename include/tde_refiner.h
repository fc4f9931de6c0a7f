/* tde_refiner.h -- the learned depth refiner: a small bf16 encoder-decoder
 * CNN that predicts a per-pixel residual for raw depth, trained and run by
 * this library's own tensor-core kernels.
 *
 * No counterpart in the reference: it is an optional replacement for the
 * bilateral stage (Apply_Billateral_Filtration, common/src/opencl_wrappers.cpp:216-235)
 * of the per-frame pipeline, enabled with tde_pipeline_set_refiner().
 *
 * Network (NHWC bf16 activations, FP32 accumulation; rows and cols divisible
 * by 8): input per tap of the 3x3 window [100 (d_t - d_centre) m, valid_t,
 * d_t] -> 16 (FP32) -> 16 | pool -> 32 -> 32 | pool -> 48 -> 48 | pool -> 64
 * -> 64 | up, concat -> 48 | up, concat -> 32 | up, concat -> 16 -> 1x1 head
 * r: refined = depth + 0.01 r on valid pixels, 0 elsewhere.  3x3
 * convolutions with ReLU; 194,401 FP32 parameters.
 *
 * Training: masked L1 against a target depth (pixels valid in input and
 * target), divided by batch*rows*cols; AdamW with decoupled weight decay on
 * the convolution weights.
 *
 * All buffers are device pointers unless named "host"; depth is uint16 mm.
 * Entry points return TDE_OK (0) or a negative tde_status.
 */
#ifndef TDE_REFINER_H
#define TDE_REFINER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tde_refiner tde_refiner;

/* Allocates parameters, optimiser state and activations for up to max_batch
 * images of rows x cols; weights He-normal from `seed` (splitmix64 +
 * Box-Muller), biases 0, head weights 0 (the initial refiner is the identity
 * on valid depth). */
int tde_refiner_create(int max_batch, int rows, int cols, uint64_t seed, tde_refiner **out);
int tde_refiner_destroy(tde_refiner *r);

size_t tde_refiner_param_count(void);
/* Flat FP32 parameters in layer order: c1.w[16][9][3], c1.b[16], then for
 * c2..c11 w[cout][9][cin], b[cout], then head.w[16], head.b[1]; c1.w is
 * [16][9][3] in the feature order above. */
int tde_refiner_get_params(tde_refiner *r, float *host, size_t count);
/* Sets the parameters and zeroes the AdamW moments and step count. */
int tde_refiner_set_params(tde_refiner *r, const float *host, size_t count);
int tde_refiner_set_adamw(tde_refiner *r, float beta1, float beta2, float eps, float weight_decay);

/* Inference: raw [batch][rows][cols] -> refined depth in mm (out_mm) and/or
 * metres (out_m); either output may be NULL.  Stream-ordered on `stream`. */
int tde_refiner_forward(tde_refiner *r, const uint16_t *raw, int batch, uint16_t *out_mm, float *out_m, void *stream);

/* Forward, loss and every parameter gradient, without an update. */
int tde_refiner_loss_grad(tde_refiner *r, const uint16_t *raw, const uint16_t *target, int batch, void *stream);
/* Forward, loss, gradients and one AdamW step with learning rate lr. */
int tde_refiner_train_step(tde_refiner *r, const uint16_t *raw, const uint16_t *target, int batch, float lr,
                           void *stream);
/* Synchronises; the gradient of the last loss_grad / train_step. */
int tde_refiner_get_grads(tde_refiner *r, float *host, size_t count);
/* Synchronises; sum over valid pixels of |refined - target| / (batch*rows*cols)
 * and the number of valid pixels, of the last loss_grad / train_step. */
int tde_refiner_last_loss(tde_refiner *r, double *loss, double *valid_pixels);

/* Test access to internal tensors (synchronises).  Ids: 0..10 activations
 * e0a e0 e1a e1 e2a e2 b3a b3 d2 d1 d0 (bf16 NHWC), 11 refined depth (FP32),
 * 12.. gradients dz11 gu0 dz10 gu1 dz9 gu2 dz8 dz7 gp3 dz6 dz5 gp2 dz4 dz3 gp1
 * dz2 dz1 (bf16 NHWC).  `bytes` must equal the tensor's size at the batch of
 * the last call. */
int tde_refiner_get_tensor(tde_refiner *r, int id, void *host, size_t bytes);
size_t tde_refiner_tensor_bytes(tde_refiner *r, int id);

/* TDE_OK when the refiner was created for rows x cols, else TDE_ERR_INVALID_ARG. */
int tde_refiner_check_shape(tde_refiner *r, int rows, int cols);

/* Device-side status: TDE_ERR_DEVICE_TIMEOUT once a tensor-core wait gave up. */
int tde_refiner_status(tde_refiner *r);

/* Self-test of the bounded wait every tensor-core kernel here uses (no
 * counterpart in the reference): one thread waits on a barrier phase that
 * nothing completes, gives up after limit_ns (at most 10 s), raises the flag
 * and returns; out_device (2 device values) receives the flag (1) and the
 * nanoseconds waited.  The context stays usable. */
int tde_wait_selftest(uint64_t limit_ns, unsigned long long *out_device, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TDE_REFINER_H */
