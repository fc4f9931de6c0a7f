// refiner.cu -- host side of the learned depth refiner: parameter and
// activation storage, the forward / backward launch schedule, AdamW, and the
// C-ABI of include/tde_refiner.h.
//
// The network and its gradient routing are fixed here (kConv, kBack); the
// CPU oracle restates the same network in FP64 for the tests.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/tde_refiner.h"
#include "tde_common.cuh"
#include "tde_refiner.cuh"

using namespace tde;
using namespace tde::refiner;

namespace {

enum Act { E0A, E0, E1A, E1, E2A, E2, B3A, B3, D2, D1, D0, ACT_COUNT };
enum Grad {
    G_DZ11, G_U0, G_DZ10, G_U1, G_DZ9, G_U2, G_DZ8, G_DZ7, G_P3, G_DZ6, G_DZ5, G_P2, G_DZ4, G_DZ3, G_P1, G_DZ2, G_DZ1,
    GRAD_COUNT
};
struct TensorSpec { int level, ch; };
const TensorSpec kAct[ACT_COUNT] = {{0, 16}, {0, 16}, {1, 32}, {1, 32}, {2, 48}, {2, 48},
                                    {3, 64}, {3, 64}, {2, 48}, {1, 32}, {0, 16}};
const TensorSpec kGrad[GRAD_COUNT] = {{0, 16}, {0, 48}, {1, 32}, {1, 80}, {2, 48}, {2, 112}, {3, 64}, {3, 64}, {3, 48},
                                      {2, 48}, {2, 48}, {2, 32}, {1, 32}, {1, 32}, {1, 16}, {0, 16}, {0, 16}};

// Convolutions c2..c11 (c1 is the FP32 input convolution).  The encoder's
// 2x2 max pools are written by the epilogues of c2, c4 and c6 (pool_out: the
// pooled copy of `out`) and read directly by c3, c5 and c7 (pool_in: source
// A is that copy; `a` still names the unpooled tensor, whose argmax routes
// the pool's gradient).
struct Conv { int level, a, ca, mode, b, cb, cout, out, pool_in, pool_out; };
constexpr int kConvs = 10;
constexpr int kPools = 3;
const Conv kConv[kConvs] = {
    {0, E0A, 16, SRC_DIRECT, -1, 0, 16, E0, -1, 0},   // c2 (+ pool of e0)
    {1, E0, 16, SRC_POOL, -1, 0, 32, E1A, 0, -1},     // c3
    {1, E1A, 32, SRC_DIRECT, -1, 0, 32, E1, -1, 1},   // c4 (+ pool of e1)
    {2, E1, 32, SRC_POOL, -1, 0, 48, E2A, 1, -1},     // c5
    {2, E2A, 48, SRC_DIRECT, -1, 0, 48, E2, -1, 2},   // c6 (+ pool of e2)
    {3, E2, 48, SRC_POOL, -1, 0, 64, B3A, 2, -1},     // c7
    {3, B3A, 64, SRC_DIRECT, -1, 0, 64, B3, -1, -1},  // c8
    {2, B3, 64, SRC_UP, E2, 48, 48, D2, -1, -1},      // c9
    {1, D2, 48, SRC_UP, E1, 32, 32, D1, -1, -1},      // c10
    {0, D1, 32, SRC_UP, E0, 16, 16, D0, -1, -1},      // c11
};
// The convolution kernel's source mode for conv i: the pooled inputs are read directly.
inline int conv_mode(const Conv &c) { return c.pool_in >= 0 ? (int)SRC_DIRECT : c.mode; }

// Backward routing of conv i: its output gradient dz, the buffer its input
// gradient goes to (masked by `mask` when the input is a ReLU output read
// directly), and how that becomes the next output gradient.
enum Post { POST_NONE, POST_UP, POST_POOL };
struct Back { int dz, gx, mask, post, post_out, skip, skip_cu, skip_off; };
const Back kBack[kConvs] = {
    {G_DZ2, G_DZ1, E0A, POST_NONE, -1, -1, 0, 0},       // c2
    {G_DZ3, G_P1, -1, POST_POOL, G_DZ2, G_U0, 48, 32},  // c3: e0 also feeds c11 (channels 32..47)
    {G_DZ4, G_DZ3, E1A, POST_NONE, -1, -1, 0, 0},       // c4
    {G_DZ5, G_P2, -1, POST_POOL, G_DZ4, G_U1, 80, 48},  // c5: e1 also feeds c10 (48..79)
    {G_DZ6, G_DZ5, E2A, POST_NONE, -1, -1, 0, 0},       // c6
    {G_DZ7, G_P3, -1, POST_POOL, G_DZ6, G_U2, 112, 64}, // c7: e2 also feeds c9 (64..111)
    {G_DZ8, G_DZ7, B3A, POST_NONE, -1, -1, 0, 0},       // c8
    {G_DZ9, G_U2, -1, POST_UP, G_DZ8, -1, 0, 0},        // c9
    {G_DZ10, G_U1, -1, POST_UP, G_DZ9, -1, 0, 0},       // c10
    {G_DZ11, G_U0, -1, POST_UP, G_DZ10, -1, 0, 0},      // c11
};

constexpr int kC1W = 16 * 9 * 3, kC1B = 16;

struct Layout {
    size_t c1w = 0, c1b = 0, w[kConvs] = {}, b[kConvs] = {}, hw = 0, hb = 0, total = 0;
    size_t wq[kConvs] = {}, wq_total = 0;
    Layout() {
        size_t o = 0;
        c1w = o; o += kC1W;
        c1b = o; o += kC1B;
        size_t q = 0;
        for (int i = 0; i < kConvs; ++i) {
            const int cin = kConv[i].ca + kConv[i].cb;
            w[i] = o; o += (size_t)kConv[i].cout * 9 * cin;
            b[i] = o; o += kConv[i].cout;
            wq[i] = q; q += (size_t)kConv[i].cout * 9 * cin;
        }
        hw = o; o += 16;
        hb = o; o += 1;
        total = o;
        wq_total = q;
    }
};
const Layout kL;

// splitmix64 and Box-Muller: a reproducible normal generator
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace

struct tde_refiner {
    int max_batch = 0, rows = 0, cols = 0, num_sms = 0;
    float *theta = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    uint8_t *decay = nullptr;
    bf16 *wq = nullptr, *wt = nullptr;
    float *depth_m = nullptr, *out_m = nullptr;
    bf16 *act[ACT_COUNT] = {};
    bf16 *pooled[kPools] = {};  // 2x2 max pools of e0, e1, e2 (levels 1, 2, 3)
    bf16 *gr[GRAD_COUNT] = {};
    float *wpartial = nullptr;
    int wg_blocks = 0;
    ConvPlan fwd_plan[kConvs] = {}, bwd_plan[kConvs] = {};  // launch geometry per convolution
    float *in_partial = nullptr;
    float *loss_partial = nullptr;
    double *loss2 = nullptr;
    int *err = nullptr;
    int step = 0;
    float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f, wd = 0.01f;
    int last_batch = 0;
    std::vector<void *> allocs;
};

namespace {

template <class T> int dalloc(tde_refiner *r, T **p, size_t count) {
    void *q = nullptr;
    TDE_CUDA(cudaMalloc(&q, count * sizeof(T) + 256), "refiner: cudaMalloc");
    r->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return TDE_OK;
}

size_t pixels(const tde_refiner *r, int batch, int level) {
    return (size_t)batch * (r->rows >> level) * (r->cols >> level);
}

int check_batch(const tde_refiner *r, int batch) {
    if (batch < 1 || batch > r->max_batch)
        return set_error(TDE_ERR_INVALID_ARG, "refiner: batch %d outside [1, %d]", batch, r->max_batch);
    return TDE_OK;
}

int pack_all(tde_refiner *r, cudaStream_t s) {
    for (int i = 0; i < kConvs; ++i)
        TDE_TRY(launch_pack_weights(r->theta + kL.w[i], kConv[i].cout, kConv[i].ca + kConv[i].cb, r->wq + kL.wq[i],
                                    r->wt + kL.wq[i], s));
    return TDE_OK;
}

int forward(tde_refiner *r, const uint16_t *raw, int n, uint16_t *out_mm, cudaStream_t s) {
    TDE_TRY(launch_conv_in(raw, r->depth_m, r->theta + kL.c1w, r->theta + kL.c1b, r->act[E0A], n, r->rows, r->cols, s));
    for (int i = 0; i < kConvs; ++i) {
        const Conv &c = kConv[i];
        ConvArgs a;
        std::memset(&a, 0, sizeof(a));
        a.a = c.pool_in >= 0 ? r->pooled[c.pool_in] : r->act[c.a]; a.ca = c.ca; a.mode_a = conv_mode(c);
        a.b = c.b >= 0 ? r->act[c.b] : nullptr; a.cb = c.cb;
        a.wgt = r->wq + kL.wq[i];
        a.bias = r->theta + kL.b[i];
        a.out = r->act[c.out]; a.cout = c.cout; a.relu = 1;
        a.pool_out = c.pool_out >= 0 ? r->pooled[c.pool_out] : nullptr;
        a.n = n; a.h = r->rows >> c.level; a.w = r->cols >> c.level;
        a.err = r->err;
        if (i == kConvs - 1) {
            a.head_w = r->theta + kL.hw;
            a.head_b = r->theta + kL.hb;
            a.depth_in = r->depth_m;
            a.depth_out = r->out_m;
            a.depth_mm = out_mm;
        }
        TDE_TRY(launch_conv(a, r->fwd_plan[i], r->num_sms, s));
    }
    r->last_batch = n;
    return TDE_OK;
}

int loss_grad(tde_refiner *r, const uint16_t *raw, const uint16_t *target, int n, cudaStream_t s) {
    TDE_TRY(forward(r, raw, n, nullptr, s));
    const int H = r->rows, W = r->cols;
    TDE_TRY(launch_loss(r->out_m, r->depth_m, target, r->act[D0], r->theta + kL.hw, n, H, W, r->gr[G_DZ11],
                        r->loss_partial, loss_blocks(n, H, W), r->grad + kL.hw, r->grad + kL.hb, r->loss2, s));
    for (int i = kConvs - 1; i >= 0; --i) {
        const Conv &c = kConv[i];
        const Back &k = kBack[i];
        const int cin = c.ca + c.cb, h = H >> c.level, w = W >> c.level;
        WgradArgs wa;
        std::memset(&wa, 0, sizeof(wa));
        wa.a = c.pool_in >= 0 ? r->pooled[c.pool_in] : r->act[c.a]; wa.ca = c.ca; wa.mode_a = conv_mode(c);
        wa.b = c.b >= 0 ? r->act[c.b] : nullptr; wa.cb = c.cb;
        wa.dz = r->gr[k.dz]; wa.cout = c.cout;
        wa.n = n; wa.h = h; wa.w = w;
        wa.partial = r->wpartial; wa.err = r->err;
        TDE_TRY(launch_wgrad(wa, r->wg_blocks, s));
        TDE_TRY(launch_wgrad_reduce(r->wpartial, r->wg_blocks, cin, c.cout, r->grad + kL.w[i], r->grad + kL.b[i], s));
        // input gradient: the same convolution on dz with the flipped, transposed weights
        ConvArgs a;
        std::memset(&a, 0, sizeof(a));
        a.a = r->gr[k.dz]; a.ca = c.cout; a.mode_a = SRC_DIRECT;
        a.wgt = r->wt + kL.wq[i];
        a.out = r->gr[k.gx]; a.cout = cin; a.relu = 0;
        a.mask = k.mask >= 0 ? r->act[k.mask] : nullptr;
        a.n = n; a.h = h; a.w = w;
        a.err = r->err;
        TDE_TRY(launch_conv(a, r->bwd_plan[i], r->num_sms, s));
        if (k.post == POST_UP)
            TDE_TRY(launch_up_back(r->gr[k.gx], cin, c.ca, r->act[c.a], r->gr[k.post_out], n, h, w, s));
        else if (k.post == POST_POOL)
            TDE_TRY(launch_pool_back_add(r->act[c.a], r->gr[k.gx], r->gr[k.skip], k.skip_cu, k.skip_off, c.ca,
                                         r->gr[k.post_out], n, h * 2, w * 2, s));
    }
    TDE_TRY(launch_conv_in_wgrad(r->depth_m, r->gr[G_DZ1], n, H, W, r->in_partial, conv_in_wgrad_blocks(n, H),
                                 r->grad + kL.c1w, r->grad + kL.c1b, s));
    return TDE_OK;
}

}  // namespace

extern "C" {

int tde_refiner_create(int max_batch, int rows, int cols, uint64_t seed, tde_refiner **out) {
    if (!out || max_batch < 1 || rows < 8 || cols < 8 || rows % 8 || cols % 8)
        return set_error(TDE_ERR_INVALID_ARG, "refiner_create: rows and cols must be positive multiples of 8");
    *out = nullptr;
    tde_refiner *r = new tde_refiner;
    r->max_batch = max_batch;
    r->rows = rows;
    r->cols = cols;
    int dev = 0;
    int st = TDE_OK;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess) {
        delete r;
        return set_error(TDE_ERR_CUDA, "refiner_create: no CUDA device");
    }
    r->wg_blocks = wgrad_blocks(r->num_sms, 0, 0);
    st = prepare_kernels();
    for (int i = 0; i < kConvs && !st; ++i) {
        const int cin = kConv[i].ca + kConv[i].cb;
        st = conv_plan(conv_mode(kConv[i]), kConv[i].ca, cin, kConv[i].cout, &r->fwd_plan[i]);
        if (!st) st = conv_plan(SRC_DIRECT, kConv[i].cout, kConv[i].cout, cin, &r->bwd_plan[i]);
    }
    if (st) {
        delete r;
        return st;
    }
    size_t wpart = 0;
    for (int i = 0; i < kConvs; ++i) {
        const size_t f = wgrad_partial_floats(r->wg_blocks, kConv[i].ca + kConv[i].cb, kConv[i].cout);
        if (f > wpart) wpart = f;
    }
    const size_t P = kL.total;
    do {
        if ((st = dalloc(r, &r->theta, P)) || (st = dalloc(r, &r->grad, P)) || (st = dalloc(r, &r->m, P)) ||
            (st = dalloc(r, &r->v, P)) || (st = dalloc(r, &r->decay, P)) || (st = dalloc(r, &r->wq, kL.wq_total)) ||
            (st = dalloc(r, &r->wt, kL.wq_total)) || (st = dalloc(r, &r->depth_m, pixels(r, max_batch, 0))) ||
            (st = dalloc(r, &r->out_m, pixels(r, max_batch, 0))) || (st = dalloc(r, &r->wpartial, wpart)) ||
            (st = dalloc(r, &r->in_partial, (size_t)conv_in_wgrad_blocks(max_batch, rows) * 448)) ||
            (st = dalloc(r, &r->loss_partial, (size_t)loss_blocks(max_batch, rows, cols) * 19)) ||
            (st = dalloc(r, &r->loss2, 2)) || (st = dalloc(r, &r->err, 1)))
            break;
        for (int i = 0; i < ACT_COUNT && !st; ++i)
            st = dalloc(r, &r->act[i], pixels(r, max_batch, kAct[i].level) * kAct[i].ch);
        for (int i = 0; i < kConvs && !st; ++i)
            if (kConv[i].pool_out >= 0)
                st = dalloc(r, &r->pooled[kConv[i].pool_out],
                            pixels(r, max_batch, kConv[i].level + 1) * kConv[i].cout);
        for (int i = 0; i < GRAD_COUNT && !st; ++i)
            st = dalloc(r, &r->gr[i], pixels(r, max_batch, kGrad[i].level) * kGrad[i].ch);
    } while (0);
    if (st) {
        tde_refiner_destroy(r);
        return st;
    }
    // initial parameters and the weight-decay mask
    std::vector<float> th(P, 0.f);
    std::vector<uint8_t> dm(P, 0);
    Rng g{seed};
    auto fill = [&](size_t off, size_t count, double sd) {
        for (size_t k = 0; k < count; ++k) {
            th[off + k] = (float)(sd * g.normal());
            dm[off + k] = 1;
        }
    };
    fill(kL.c1w, kC1W, std::sqrt(2.0 / 27.0));
    for (int i = 0; i < kConvs; ++i) {
        const int cin = kConv[i].ca + kConv[i].cb;
        fill(kL.w[i], (size_t)kConv[i].cout * 9 * cin, std::sqrt(2.0 / (9.0 * cin)));
    }
    // head.w stays 0: the refiner starts as the identity on valid depth
    for (int k = 0; k < 16; ++k) dm[kL.hw + k] = 1;
    if ((st = cudaMemcpy(r->decay, dm.data(), P, cudaMemcpyHostToDevice) == cudaSuccess
                  ? TDE_OK
                  : set_error(TDE_ERR_CUDA, "refiner_create: copy")) ||
        (st = cudaMemset(r->err, 0, sizeof(int)) == cudaSuccess ? TDE_OK : set_error(TDE_ERR_CUDA, "memset")) ||
        (st = tde_refiner_set_params(r, th.data(), P))) {
        tde_refiner_destroy(r);
        return st;
    }
    *out = r;
    return TDE_OK;
}

int tde_refiner_destroy(tde_refiner *r) {
    if (!r) return TDE_OK;
    cudaDeviceSynchronize();
    for (void *p : r->allocs) cudaFree(p);
    delete r;
    return TDE_OK;
}

size_t tde_refiner_param_count(void) { return kL.total; }

int tde_refiner_get_params(tde_refiner *r, float *host, size_t count) {
    if (!r || !host || count != kL.total) return set_error(TDE_ERR_INVALID_ARG, "refiner_get_params: bad argument");
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_get_params");
    TDE_CUDA(cudaMemcpy(host, r->theta, count * sizeof(float), cudaMemcpyDeviceToHost), "refiner_get_params");
    return TDE_OK;
}

int tde_refiner_set_params(tde_refiner *r, const float *host, size_t count) {
    if (!r || !host || count != kL.total) return set_error(TDE_ERR_INVALID_ARG, "refiner_set_params: bad argument");
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_set_params");
    TDE_CUDA(cudaMemcpy(r->theta, host, count * sizeof(float), cudaMemcpyHostToDevice), "refiner_set_params");
    TDE_CUDA(cudaMemset(r->m, 0, count * sizeof(float)), "refiner_set_params");
    TDE_CUDA(cudaMemset(r->v, 0, count * sizeof(float)), "refiner_set_params");
    r->step = 0;
    TDE_TRY(pack_all(r, nullptr));
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_set_params");
    return TDE_OK;
}

int tde_refiner_set_adamw(tde_refiner *r, float beta1, float beta2, float eps, float weight_decay) {
    if (!r || !(beta1 >= 0.f && beta1 < 1.f) || !(beta2 >= 0.f && beta2 < 1.f) || !(eps > 0.f) || !(weight_decay >= 0.f))
        return set_error(TDE_ERR_INVALID_ARG, "refiner_set_adamw: bad argument");
    r->b1 = beta1;
    r->b2 = beta2;
    r->eps = eps;
    r->wd = weight_decay;
    return TDE_OK;
}

int tde_refiner_forward(tde_refiner *r, const uint16_t *raw, int batch, uint16_t *out_mm, float *out_m, void *stream) {
    if (!r || !raw) return set_error(TDE_ERR_INVALID_ARG, "refiner_forward: null argument");
    TDE_TRY(check_batch(r, batch));
    cudaStream_t s = as_stream(stream);
    TDE_TRY(forward(r, raw, batch, out_mm, s));
    if (out_m)
        TDE_CUDA(cudaMemcpyAsync(out_m, r->out_m, pixels(r, batch, 0) * sizeof(float), cudaMemcpyDeviceToDevice, s),
                 "refiner_forward: copy");
    return TDE_OK;
}

int tde_refiner_loss_grad(tde_refiner *r, const uint16_t *raw, const uint16_t *target, int batch, void *stream) {
    if (!r || !raw || !target) return set_error(TDE_ERR_INVALID_ARG, "refiner_loss_grad: null argument");
    TDE_TRY(check_batch(r, batch));
    return loss_grad(r, raw, target, batch, as_stream(stream));
}

int tde_refiner_train_step(tde_refiner *r, const uint16_t *raw, const uint16_t *target, int batch, float lr,
                           void *stream) {
    if (!r || !raw || !target || !(lr >= 0.f)) return set_error(TDE_ERR_INVALID_ARG, "refiner_train_step: bad argument");
    TDE_TRY(check_batch(r, batch));
    cudaStream_t s = as_stream(stream);
    TDE_TRY(loss_grad(r, raw, target, batch, s));
    r->step += 1;
    const float bc1 = (float)(1.0 - std::pow((double)r->b1, r->step));
    const float bc2 = (float)(1.0 - std::pow((double)r->b2, r->step));
    TDE_TRY(launch_adamw(r->theta, r->grad, r->m, r->v, r->decay, kL.total, lr, r->b1, r->b2, r->eps, r->wd, bc1, bc2,
                         s));
    return pack_all(r, s);
}

int tde_refiner_get_grads(tde_refiner *r, float *host, size_t count) {
    if (!r || !host || count != kL.total) return set_error(TDE_ERR_INVALID_ARG, "refiner_get_grads: bad argument");
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_get_grads");
    TDE_CUDA(cudaMemcpy(host, r->grad, count * sizeof(float), cudaMemcpyDeviceToHost), "refiner_get_grads");
    return TDE_OK;
}

int tde_refiner_last_loss(tde_refiner *r, double *loss, double *valid_pixels) {
    if (!r) return set_error(TDE_ERR_INVALID_ARG, "refiner_last_loss: null");
    double h[2];
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_last_loss");
    TDE_CUDA(cudaMemcpy(h, r->loss2, sizeof(h), cudaMemcpyDeviceToHost), "refiner_last_loss");
    if (loss) *loss = h[0];
    if (valid_pixels) *valid_pixels = h[1];
    return TDE_OK;
}

size_t tde_refiner_tensor_bytes(tde_refiner *r, int id) {
    if (!r || r->last_batch < 1) return 0;
    if (id >= 0 && id < ACT_COUNT) return pixels(r, r->last_batch, kAct[id].level) * kAct[id].ch * 2;
    if (id == ACT_COUNT) return pixels(r, r->last_batch, 0) * 4;
    const int g = id - ACT_COUNT - 1;
    if (g >= 0 && g < GRAD_COUNT) return pixels(r, r->last_batch, kGrad[g].level) * kGrad[g].ch * 2;
    return 0;
}

int tde_refiner_get_tensor(tde_refiner *r, int id, void *host, size_t bytes) {
    const size_t need = tde_refiner_tensor_bytes(r, id);
    if (!r || !host || need == 0 || bytes != need)
        return set_error(TDE_ERR_INVALID_ARG, "refiner_get_tensor: id %d needs %zu bytes", id, need);
    const void *src = id < ACT_COUNT ? (const void *)r->act[id]
                      : id == ACT_COUNT ? (const void *)r->out_m
                                        : (const void *)r->gr[id - ACT_COUNT - 1];
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_get_tensor");
    TDE_CUDA(cudaMemcpy(host, src, bytes, cudaMemcpyDeviceToHost), "refiner_get_tensor");
    return TDE_OK;
}

int tde_refiner_check_shape(tde_refiner *r, int rows, int cols) {
    if (!r || r->rows != rows || r->cols != cols)
        return set_error(TDE_ERR_INVALID_ARG, "refiner: created for %dx%d, used for %dx%d", r ? r->cols : 0,
                         r ? r->rows : 0, cols, rows);
    return TDE_OK;
}

int tde_wait_selftest(uint64_t limit_ns, unsigned long long *out_device, void *stream) {
    if (!out_device || limit_ns == 0 || limit_ns > 10000000000ull)
        return set_error(TDE_ERR_INVALID_ARG, "wait_selftest: bad arguments");
    return launch_wait_selftest(limit_ns, out_device, static_cast<cudaStream_t>(stream));
}

int tde_refiner_status(tde_refiner *r) {
    if (!r) return set_error(TDE_ERR_INVALID_ARG, "refiner_status: null");
    int e = 0;
    TDE_CUDA(cudaDeviceSynchronize(), "refiner_status");
    TDE_CUDA(cudaMemcpy(&e, r->err, sizeof(int), cudaMemcpyDeviceToHost), "refiner_status");
    return e ? set_error(TDE_ERR_DEVICE_TIMEOUT, "refiner: a tensor-core wait timed out") : TDE_OK;
}

}  // extern "C"
