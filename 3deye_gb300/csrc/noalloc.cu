// noalloc.cu -- TSDF integration for callers that must not allocate.
//
// tde_integrate_tsdf needs a little device scratch per call (the frame's
// per-tile maximum depth and the list of 8^3 bricks that survive culling) and
// obtains it with cudaMallocAsync; tde_integrate_tsdf_ex takes it from the
// caller.  Some callers can do neither: code running where every allocation
// is forbidden once the system is live (real-time loops that have to keep a
// fixed memory footprint, plug-in hosts whose memory manager owns the device,
// embedded deployments with a budget fixed at start-up), or callers that
// have no way to pass a device buffer through their interface at all.
// tde_integrate_tsdf_noalloc serves them: its scratch lives in the fixed
// array below, part of the module's static device memory.
#include <mutex>

#include "tde_common.cuh"
#include "tde_integrate.cuh"

namespace tde {
namespace {

// 1.5 MiB: room for the brick list of a 512^3 volume (262,144 bricks, 1 MiB)
// plus the depth tiles of a 640x480 frame.  Every GPU that loads the library
// holds this array until the process exits.
constexpr size_t kNoAllocScratchBytes = (size_t)3 << 19;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct ScratchSlot {
    unsigned long long ctx_id;  // the context the address belongs to
    void *addr;
};
ScratchSlot g_scratch[kMaxDevices] = {};

// Two driver entry points, fetched through the runtime so the library needs
// no link against the driver library: the current context and its id, which
// stays unique for the life of the process (a context created after
// cudaDeviceReset gets a new one even where its handle value repeats).
typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int current_context_id(unsigned long long *id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return set_error(TDE_ERR_CUDA, "integrate_noalloc: driver entry points cuCtxGetCurrent/cuCtxGetId");
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void *ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0 || !ctx || g_ctx_get_id(ctx, id) != 0)
        return set_error(TDE_ERR_CUDA, "integrate_noalloc: no current CUDA context");
    return TDE_OK;
}

// Device address of the array in the current device's context.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// with cudaGetSymbolAddress, once per device and context, with that device
// current; a later context on the device (after cudaDeviceReset) loads the
// module again and gets its own lookup.
int scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "integrate_noalloc: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(TDE_ERR_UNSUPPORTED, "integrate_noalloc: device %d", dev);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = 0;
    void *p = nullptr;
    if (g_scratch[dev].addr) {
        TDE_TRY(current_context_id(&id));
        if (g_scratch[dev].ctx_id == id) {
            *out = g_scratch[dev].addr;
            return TDE_OK;
        }
    }
    // set-up: also makes the device's primary context current when nothing
    // has used the device yet
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return set_error(TDE_ERR_CUDA, "integrate_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    TDE_TRY(current_context_id(&id));
    g_scratch[dev] = ScratchSlot{id, p};
    *out = p;
    return TDE_OK;
}

}  // namespace
}  // namespace tde

using namespace tde;

extern "C" {

size_t tde_integrate_tsdf_noalloc_max_scratch_bytes(void) { return kNoAllocScratchBytes; }

int tde_integrate_tsdf_noalloc(const float *depth_scaled, void *volume, int format, float trunc,
                               const tde_matrix3f *R_inv, const tde_point3f *t, const tde_intrinsics *intr,
                               const tde_point3f *cell_size, const tde_round_buffer *rb, int max_weight,
                               void *stream) {
    // The same argument checks as tde_integrate_tsdf_ex, which also rejects
    // any configuration whose scratch would not fit the fixed array.
    if (!intr || !rb) return set_error(TDE_ERR_INVALID_ARG, "integrate_noalloc: null intrinsics / round_buffer");
    const size_t need = tde_integrate_tsdf_scratch_bytes(intr->cols, intr->rows, rb);
    if (need == 0) return set_error(TDE_ERR_INVALID_ARG, "integrate_noalloc: bad image size or round_buffer");
    if (need > kNoAllocScratchBytes)
        return set_error(TDE_ERR_CAPACITY,
                         "integrate_noalloc: this frame and volume need %zu bytes of scratch; the fixed array holds "
                         "%zu (use tde_integrate_tsdf or tde_integrate_tsdf_ex)",
                         need, kNoAllocScratchBytes);
    void *scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st != TDE_OK) return st;
    // depth tiles and the brick counter are rewritten (the counter zeroed) by
    // every call before use, so nothing left from an earlier call is read
    return tde_integrate_tsdf_ex(depth_scaled, volume, format, trunc, R_inv, t, intr, cell_size, rb, max_weight,
                                 scratch, kNoAllocScratchBytes, nullptr, stream);
}

}  // extern "C"
