// pipeline.cu -- the per-frame loop (tde_pipeline.h): buffers, the launch
// sequence of one frame, its CUDA-graph capture, live timing.
//
// A frame's preprocessing (filter or refiner, pyramid, vertex and normal
// maps) reads only that frame's depth, so it runs on a second stream into one
// of two input sets while the previous frame is still tracked, integrated and
// raycast on the main stream.  Per frame f, set f & 1:
//   pre stream:  wait set_free[set]; upload depth; preprocessing; record pre_done[set]
//   main stream: wait pre_done[set]; ICP, pose, integration, raycast; record set_free[set]
#include <cmath>
#include <cstddef>
#include <cstring>
#include <new>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/tde_pipeline.h"
#include "../../include/tde_refiner.h"
#include "tde_common.cuh"
#include "tde_icp.cuh"
#include "tde_integrate.cuh"
#include "tde_launch.cuh"

namespace tde {
namespace {

struct FrameOut {
    double pose[12];
    int status;
    int inliers;
};

// Publishes the camera pose of the first frame (no tracking).
__global__ void publish_first_kernel(const IcpState *st, CamPose *cam, FrameOut *out) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            cam->R[3 * r + c] = (float)st->R[3 * r + c];
            cam->R_inv[3 * r + c] = (float)st->R[3 * c + r];
        }
    for (int k = 0; k < 3; ++k) cam->t[k] = (float)st->t[k];
    cam->tracking_ok = 1;
    for (int k = 0; k < 9; ++k) out->pose[k] = st->R[k];
    for (int k = 0; k < 3; ++k) out->pose[9 + k] = st->t[k];
    out->status = 0;
    out->inliers = 0;
}

// Depth of the model surface along the camera axis, from the raycast
// vertex map (volume frame) and the pose it was cast from; 0 where no hit.
__global__ void model_depth_kernel(const float *__restrict__ vmap, const CamPose *__restrict__ cam, int n,
                                   uint16_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float vx = vmap[3 * i], vy = vmap[3 * i + 1], vz = vmap[3 * i + 2];
    float z = 0.f;
    if (!isnan(vx)) z = cam->R[2] * (vx - cam->t[0]) + cam->R[5] * (vy - cam->t[1]) + cam->R[8] * (vz - cam->t[2]);
    out[i] = z > 0.f ? (uint16_t)fminf(rintf(z * 1000.f), (float)TDE_MAX_DEPTH_VALUE) : (uint16_t)0;
}

enum Segment {
    SEG_PRE,         // bilateral filter (or refiner), pyramid, vertex and normal maps, scaled depth, depth tiles
    SEG_ICP,         // ICP iterations; the last one accepts and publishes the pose
    SEG_POST_FIRST,  // pose publication without tracking (first frame)
    SEG_INTEGRATE,
    SEG_RAYCAST,
    SEG_RESIZE,
    SEG_COLOR,       // colour volume update (side stream; reads this frame's snapshot of the model map and pose)
    SEG_COUNT
};
// Stages timed per frame, in order: SEG_PRE, SEG_ICP (SEG_POST_FIRST on the
// first frame), SEG_INTEGRATE, SEG_RAYCAST, SEG_RESIZE.
constexpr int kStages = 5;
constexpr int kEvents = kStages + 1;

}  // namespace
}  // namespace tde

using namespace tde;

struct tde_pipeline {
    tde_pipeline_config cfg;
    tde_round_buffer rb;
    tde_point3f cell;
    cudaStream_t stream = nullptr;      // tracking and fusion
    cudaStream_t pre_stream = nullptr;  // preprocessing of the next frame
    cudaStream_t col_stream = nullptr;  // colour volume update, beside the next frame's tracking
    int prio_low = 0, prio_high = 0;
    cudaEvent_t pre_done[2] = {}, set_free[2] = {};
    cudaEvent_t col_ready[2] = {}, col_done[2] = {};
    int levels = 3;
    int sm_count = 1;  // multiprocessors of the pipeline's device
    tde_intrinsics intr[3];
    // device buffers; raw depth and the current-frame maps come in two sets
    uint16_t *raw[2] = {};
    uint16_t *depth[2][3] = {};
    float *vcur[2][3] = {}, *ncur[2][3] = {};
    float *scaled[2] = {};        // depth along the ray (m), per input set
    void *iscratch[2] = {};       // integration: per-tile maximum depth + brick list, per input set
    float *vmod[3] = {}, *nmod[3] = {};
    IcpState *st = nullptr;
    CamPose *cam = nullptr;
    FrameOut *out = nullptr;
    unsigned long long *stats = nullptr;
    uint8_t *negflags = nullptr;  // per physical brick: may hold a negative value
    uint8_t *satflags = nullptr;  // per logical brick: every voxel at f = 1, maximum weight
    // colour volume (tde_pipeline_enable_color): RGB frames per input set, and
    // per set the level-0 model vertex map and camera pose the update reads
    // (the next frame's raycast and pose publication overwrite the live ones)
    tde_color *colvol = nullptr;
    uint8_t *rgb[2] = {};
    float *vcol[2] = {};
    CamPose *cam_col[2] = {};
    void *cscratch = nullptr;
    int color_max_weight = 0;
    void *volume = nullptr;
    tde_refiner *refiner = nullptr;  // replaces the bilateral filter when set
    // volume shifts: extraction scratch and point buffers, grown on demand
    void *slab_scratch = nullptr;
    size_t slab_scratch_bytes = 0;
    tde_xyzi *slab_points = nullptr;
    float *slab_weights = nullptr;
    tde_color *slab_colors = nullptr;
    uint32_t slab_capacity = 0;
    uint32_t *slab_count = nullptr;
    // graphs per input set: each segment, and the main-stream part of a frame
    cudaGraphExec_t seg_exec[2][SEG_COUNT] = {};
    cudaGraphExec_t main_exec[2][2] = {};  // [set][first frame, tracked frame]
    bool captured = false;
    bool inconsistent = false;  // a restore failed part-way: frames are refused
    int frames = 0;
    // timing
    int timing_cap = 0, timing_n = 0;
    std::vector<cudaEvent_t> ev;  // kEvents per timed frame
};

namespace {

template <class T> int dalloc(T **p, size_t count, const char *what) {
    TDE_CUDA(cudaMalloc((void **)p, count * sizeof(T)), what);
    return TDE_OK;
}

// The model maps (level 0) cast from the published camera pose.
int cast_model(tde_pipeline *p, cudaStream_t s) {
    const tde_pipeline_config &c = p->cfg;
    tde_point3f t0{0, 0, 0};
    tde_matrix3f R0{};
    return launch_raycast(p->volume, c.tsdf_format, p->vmod[0], p->nmod[0], t0, R0, c.trunc, p->intr[0], p->rb, p->cell,
                          p->cam, p->negflags, s);
}

// Records one segment for input set `set` onto stream s.
int record_segment(tde_pipeline *p, Segment seg, int set, cudaStream_t s) {
    const tde_pipeline_config &c = p->cfg;
    const int W = c.intr.cols, H = c.intr.rows;
    uint16_t *raw = p->raw[set], *const *depth = p->depth[set];
    float *const *vcur = p->vcur[set], *const *ncur = p->ncur[set];
    switch (seg) {
    case SEG_PRE: {
        if (p->refiner) {
            // learned refinement replaces the bilateral filter; ICP and
            // integration both use the refined depth
            TDE_TRY(tde_refiner_forward(p->refiner, raw, 1, depth[0], nullptr, s));
            TDE_TRY(launch_vertex_map(depth[0], vcur[0], p->intr[0], s));
        } else {
            TDE_TRY(launch_bilateral(raw, depth[0], W, H, c.sigma_space, c.sigma_color, c.max_depth_mm, vcur[0],
                                     &p->intr[0], s));
        }
        for (int l = 1; l < p->levels; ++l)
            TDE_TRY(launch_pyramid(depth[l - 1], depth[l], p->intr[l - 1].cols, p->intr[l - 1].rows, c.sigma_color,
                                   vcur[l], &p->intr[l], s));
        for (int l = 0; l < p->levels; ++l)
            TDE_TRY(launch_normal_map(vcur[l], ncur[l], p->intr[l].cols, p->intr[l].rows, s));
        // integration inputs: depth along the ray, and its per-tile maxima
        TDE_TRY(launch_scale_depth(p->refiner ? depth[0] : raw, p->scaled[set], p->intr[0], s));
        return launch_depth_max(p->scaled[set], W, H, static_cast<float *>(p->iscratch[set]), s);
    }
    case SEG_ICP: {
        IcpPublish pub;
        pub.cam = p->cam;
        pub.pose12 = p->out->pose;
        pub.status = &p->out->status;
        pub.inliers = &p->out->inliers;
        pub.lost_status = TDE_FRAME_TRACKING_LOST;
        int total = 0, iter = 0;
        for (int l = 0; l < p->levels; ++l) total += c.icp_iters[l];
        for (int l = p->levels - 1; l >= 0; --l) {
            IcpArgs a;
            a.vcur = vcur[l]; a.ncur = ncur[l]; a.vprev = p->vmod[l]; a.nprev = p->nmod[l];
            a.W = p->intr[l].cols; a.H = p->intr[l].rows;
            a.fx = p->intr[l].fx; a.fy = p->intr[l].fy; a.cx = p->intr[l].cx; a.cy = p->intr[l].cy;
            icp_set_thresholds(a, c.dist_thresh, c.angle_thresh);
            a.sm_count = p->sm_count;
            a.narrow = p->refiner != nullptr;  // blocks that fit beside the refiner's convolutions
            for (int it = 0; it < c.icp_iters[l]; ++it, ++iter)
                TDE_TRY(launch_icp_step(a, p->st, iter, iter == total - 1, pub, s));
        }
        return TDE_OK;
    }
    case SEG_POST_FIRST:
        publish_first_kernel<<<1, 1, 0, s>>>(p->st, p->cam, p->out);
        return check_launch("publish_first_pose");
    case SEG_INTEGRATE: {
        IntegrateParams P;
        std::memset(&P, 0, sizeof(P));
        P.trunc = c.trunc; P.max_weight = c.max_weight; P.intr = p->intr[0]; P.rb = p->rb; P.cell = p->cell;
        P.n = voxel_count(p->rb); P.dpose = p->cam;
        return launch_integrate(p->scaled[set], p->volume, c.tsdf_format, P, p->iscratch[set], p->negflags, p->stats, s,
                                p->satflags);
    }
    case SEG_RAYCAST: {
        TDE_TRY(cast_model(p, s));
        if (!p->colvol) return TDE_OK;
        // snapshot of the model map and pose for this frame's colour update
        TDE_CUDA(cudaMemcpyAsync(p->vcol[set], p->vmod[0], (size_t)W * H * 3 * sizeof(float), cudaMemcpyDeviceToDevice,
                                 s), "colour snapshot");
        TDE_CUDA(cudaMemcpyAsync(p->cam_col[set], p->cam, sizeof(CamPose), cudaMemcpyDeviceToDevice, s),
                 "colour snapshot");
        return TDE_OK;
    }
    case SEG_COLOR: {
        if (!p->colvol) return TDE_OK;
        // colour at the model surface cast from this frame's pose
        IntegrateParams P;
        std::memset(&P, 0, sizeof(P));
        P.trunc = c.trunc; P.max_weight = p->color_max_weight; P.intr = p->intr[0]; P.rb = p->rb; P.cell = p->cell;
        P.n = voxel_count(p->rb); P.dpose = p->cam_col[set];
        return launch_integrate_colors(p->colvol, p->rgb[set], p->vcol[set], P, p->cscratch, nullptr, s);
    }
    case SEG_RESIZE:
        if (p->levels < 2) return TDE_OK;
        return launch_resize_model_maps(p->vmod[0], p->nmod[0], p->vmod[1], p->nmod[1],
                                        p->levels > 2 ? p->vmod[2] : nullptr, p->levels > 2 ? p->nmod[2] : nullptr,
                                        p->intr[0].cols, p->intr[0].rows, s);
    default:
        return set_error(TDE_ERR_INVALID_ARG, "bad segment");
    }
}

int capture(tde_pipeline *p, const Segment *segs, int n, int set, cudaGraphExec_t *exec) {
    cudaGraph_t g = nullptr;
    TDE_CUDA(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    int st = TDE_OK;
    for (int i = 0; i < n && st == TDE_OK; ++i) st = record_segment(p, segs[i], set, p->stream);
    cudaError_t e = cudaStreamEndCapture(p->stream, &g);
    if (st != TDE_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    if (*exec) {
        // same topology, new parameters (a volume shift moves the round
        // buffer's origins): update in place, far cheaper than instantiating
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(*exec, g, &info) == cudaSuccess) {
            cudaGraphDestroy(g);
            return TDE_OK;
        }
        (void)cudaGetLastError();  // a topology change: instantiate afresh
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
    }
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
    return TDE_OK;
}

void drop_graphs(tde_pipeline *p) {
    for (auto &row : p->seg_exec)
        for (auto &x : row)
            if (x) { cudaGraphExecDestroy(x); x = nullptr; }
    for (auto &row : p->main_exec)
        for (auto &x : row)
            if (x) { cudaGraphExecDestroy(x); x = nullptr; }
    p->captured = false;
}

// Main-stream segments of a frame, after its preprocessing.
const Segment kMainFirst[] = {SEG_POST_FIRST, SEG_INTEGRATE, SEG_RAYCAST, SEG_RESIZE};
const Segment kMainTracked[] = {SEG_ICP, SEG_INTEGRATE, SEG_RAYCAST, SEG_RESIZE};

// Segments whose kernels take the round buffer by value (a volume shift
// changes it); the others -- preprocessing, ICP, pose publication, model
// pyramid -- read only frame and model maps.
bool reads_round_buffer(Segment sg) { return sg == SEG_INTEGRATE || sg == SEG_RAYCAST || sg == SEG_COLOR; }

// (Re)captures the graphs; existing executables are updated in place.  After
// a volume shift (`shift_only`) the segments that do not read the round
// buffer keep their graphs.
int capture_all(tde_pipeline *p, bool shift_only = false) {
    p->captured = false;
    for (int set = 0; set < 2; ++set) {
        for (int sgi = 0; sgi < SEG_COUNT; ++sgi) {
            Segment sg = (Segment)sgi;
            if (sg == SEG_COLOR && !p->colvol) continue;  // nothing to capture
            if (shift_only && p->seg_exec[set][sgi] && !reads_round_buffer(sg)) continue;
            TDE_TRY(capture(p, &sg, 1, set, &p->seg_exec[set][sgi]));
        }
        TDE_TRY(capture(p, kMainFirst, 4, set, &p->main_exec[set][0]));
        TDE_TRY(capture(p, kMainTracked, 4, set, &p->main_exec[set][1]));
    }
    p->captured = true;
    return TDE_OK;
}

int run_segment(tde_pipeline *p, Segment seg, int set, cudaStream_t s) {
    if (p->cfg.use_graphs) {
        TDE_CUDA(cudaGraphLaunch(p->seg_exec[set][seg], s), "graph launch");
        return TDE_OK;
    }
    return record_segment(p, seg, set, s);
}

// (Re)creates the preprocessing stream.  With the bilateral filter its
// kernels are short and the main stream (the frame-to-frame dependency chain)
// takes the scheduler's priority; the refiner's persistent convolutions need
// their SM share too, so with a refiner both streams have the same priority
// (measured: 2465 vs 2322 frames/s plain, 1810 vs 1646 learned).
int make_pre_stream(tde_pipeline *p) {
    if (p->pre_stream) {
        TDE_CUDA(cudaStreamSynchronize(p->pre_stream), "stream");
        TDE_CUDA(cudaStreamDestroy(p->pre_stream), "stream");
        p->pre_stream = nullptr;
    }
    TDE_CUDA(cudaStreamCreateWithPriority(&p->pre_stream, cudaStreamNonBlocking,
                                          p->refiner ? p->prio_high : p->prio_low),
             "stream");
    return TDE_OK;
}

int sync_streams(tde_pipeline *p) {
    if (p->pre_stream) TDE_CUDA(cudaStreamSynchronize(p->pre_stream), "pipeline sync");
    TDE_CUDA(cudaStreamSynchronize(p->stream), "pipeline sync");
    if (p->col_stream) TDE_CUDA(cudaStreamSynchronize(p->col_stream), "pipeline sync");
    return TDE_OK;
}

int write_pose(tde_pipeline *p, const double *pose12) {
    IcpState h;
    std::memset(&h, 0, sizeof(h));
    for (int k = 0; k < 9; ++k) h.R[k] = pose12[k];
    for (int k = 0; k < 3; ++k) h.t[k] = pose12[9 + k];
    for (int k = 0; k < 9; ++k) h.pose.R_cur[k] = (float)pose12[k];
    for (int k = 0; k < 3; ++k) h.pose.t_cur[k] = (float)pose12[9 + k];
    TDE_CUDA(cudaMemcpyAsync(p->st, &h, sizeof(h), cudaMemcpyHostToDevice, p->stream), "pose upload");
    TDE_CUDA(cudaStreamSynchronize(p->stream), "pose upload");
    return TDE_OK;
}

void release(tde_pipeline *p) {
    if (!p) return;
    if (p->pre_stream) cudaStreamSynchronize(p->pre_stream);
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->col_stream) cudaStreamSynchronize(p->col_stream);
    drop_graphs(p);
    for (auto e : p->ev) cudaEventDestroy(e);
    for (int set = 0; set < 2; ++set) {
        cudaFree(p->raw[set]);
        cudaFree(p->scaled[set]);
        cudaFree(p->iscratch[set]);
        for (int l = 0; l < 3; ++l) {
            cudaFree(p->depth[set][l]); cudaFree(p->vcur[set][l]); cudaFree(p->ncur[set][l]);
        }
        if (p->pre_done[set]) cudaEventDestroy(p->pre_done[set]);
        if (p->set_free[set]) cudaEventDestroy(p->set_free[set]);
        if (p->col_ready[set]) cudaEventDestroy(p->col_ready[set]);
        if (p->col_done[set]) cudaEventDestroy(p->col_done[set]);
        cudaFree(p->vcol[set]);
        cudaFree(p->cam_col[set]);
    }
    for (int l = 0; l < 3; ++l) { cudaFree(p->vmod[l]); cudaFree(p->nmod[l]); }
    cudaFree(p->st); cudaFree(p->cam); cudaFree(p->out);
    cudaFree(p->stats); cudaFree(p->volume); cudaFree(p->negflags); cudaFree(p->satflags);
    cudaFree(p->slab_scratch); cudaFree(p->slab_points); cudaFree(p->slab_weights); cudaFree(p->slab_count);
    cudaFree(p->slab_colors); cudaFree(p->colvol); cudaFree(p->rgb[0]); cudaFree(p->rgb[1]); cudaFree(p->cscratch);
    if (p->pre_stream) cudaStreamDestroy(p->pre_stream);
    if (p->col_stream) cudaStreamDestroy(p->col_stream);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

}  // namespace

// A named NVTX range over the host side of an entry point, for profilers
// that filter on NVTX (ncu --nvtx); a no-op when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// The float camera pose (and its inverse) the raycast and integration read,
// from an FP64 pose.
static int upload_camera(tde_pipeline *p, const double *pose, cudaStream_t s) {
    CamPose cam;
    std::memset(&cam, 0, sizeof(cam));
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            cam.R[3 * r + c] = (float)pose[3 * r + c];
            cam.R_inv[3 * r + c] = (float)pose[3 * c + r];
        }
    for (int a = 0; a < 3; ++a) cam.t[a] = (float)pose[9 + a];
    cam.tracking_ok = 1;
    TDE_CUDA(cudaMemcpyAsync(p->cam, &cam, sizeof(cam), cudaMemcpyHostToDevice, s), "camera upload");
    return TDE_OK;
}

// Checkpoint layout: this header, then the TSDF volume, the brick flags
// (negative ever written, per brick and super-brick), the saturation flags
// and, with a colour volume, the colour volume.
// The geometry fields (intrinsics, truncation, weight cap, colour weight cap)
// are the ones the stored volume was fused with: a pipeline whose values differ
// would read the volume at other positions or scales, so restore refuses it.
struct CheckpointHeader {
    char magic[8];  // "TDECKPT2"
    int32_t tsdf_format, has_color;
    int32_t cols, rows, levels, max_weight;
    int64_t frames;
    tde_round_buffer rb;
    double pose12[12];
    uint64_t volume_bytes, negflags_bytes, satflags_bytes, color_bytes;
    tde_intrinsics intr;
    float trunc;
    int32_t color_max_weight;
};
static_assert(sizeof(CheckpointHeader) == 272, "checkpoint header layout");
static const char kCheckpointMagic[8] = {'T', 'D', 'E', 'C', 'K', 'P', 'T', '2'};

static CheckpointHeader checkpoint_layout(const tde_pipeline *p) {
    CheckpointHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kCheckpointMagic, 8);
    h.tsdf_format = p->cfg.tsdf_format;
    h.has_color = p->colvol != nullptr;
    h.cols = p->cfg.intr.cols;
    h.rows = p->cfg.intr.rows;
    h.levels = p->levels;
    h.max_weight = p->cfg.max_weight;
    h.intr = p->cfg.intr;
    h.trunc = p->cfg.trunc;
    h.color_max_weight = p->colvol ? p->color_max_weight : 0;
    h.frames = p->frames;
    h.rb = p->rb;
    h.volume_bytes = tde_tsdf_volume_bytes(p->cfg.tsdf_format, &p->rb);
    h.negflags_bytes = brick_flags_bytes(p->rb);
    h.satflags_bytes = brick_count(p->rb);
    h.color_bytes = p->colvol ? voxel_count(p->rb) * sizeof(tde_color) : 0;
    return h;
}

// Count pass and scatter into the pipeline's point buffers (grown once when
// short); the total goes to *count.  `launch(capacity)` enqueues one
// extraction on the pipeline stream.
template <class Launch>
static int extract_points(tde_pipeline *p, const char *what, uint32_t *count, Launch launch) {
    cudaStream_t s = p->stream;
    const size_t need = tde_extract_slice_scratch_bytes(&p->rb);
    if (need > p->slab_scratch_bytes) {
        cudaFree(p->slab_scratch);
        p->slab_scratch = nullptr;
        p->slab_scratch_bytes = 0;
        TDE_CUDA(cudaMalloc(&p->slab_scratch, need), what);
        p->slab_scratch_bytes = need;
    }
    if (!p->slab_count) TDE_CUDA(cudaMalloc((void **)&p->slab_count, sizeof(uint32_t)), what);
    for (int pass = 0; pass < 2; ++pass) {
        TDE_TRY(launch(p->slab_capacity));
        uint32_t n = 0;
        TDE_CUDA(cudaMemcpyAsync(&n, p->slab_count, sizeof(n), cudaMemcpyDeviceToHost, s), what);
        TDE_CUDA(cudaStreamSynchronize(s), what);
        if (n <= p->slab_capacity) {
            *count = n;
            return TDE_OK;
        }
        cudaFree(p->slab_points);
        cudaFree(p->slab_weights);
        cudaFree(p->slab_colors);
        p->slab_points = nullptr;
        p->slab_weights = nullptr;
        p->slab_colors = nullptr;
        p->slab_capacity = 0;
        const uint32_t cap = n + n / 4 + 1024;
        TDE_CUDA(cudaMalloc((void **)&p->slab_points, (size_t)cap * sizeof(tde_xyzi)), what);
        TDE_CUDA(cudaMalloc((void **)&p->slab_weights, (size_t)cap * sizeof(float)), what);
        TDE_CUDA(cudaMalloc((void **)&p->slab_colors, (size_t)cap * sizeof(tde_color)), what);
        p->slab_capacity = cap;
    }
    return set_error(TDE_ERR_CAPACITY, "%s: point count changed between passes", what);
}

// Up to `capacity` of the n extracted points (and weights / colours when
// asked) to host memory.
static int points_to_host(tde_pipeline *p, const char *what, uint32_t n, tde_xyzi *points, float *weights,
                          tde_color *colors, uint32_t capacity) {
    const uint32_t ncopy = n < capacity ? n : capacity;
    if (!ncopy) return TDE_OK;
    TDE_CUDA(cudaMemcpy(points, p->slab_points, (size_t)ncopy * sizeof(tde_xyzi), cudaMemcpyDeviceToHost), what);
    if (weights)
        TDE_CUDA(cudaMemcpy(weights, p->slab_weights, (size_t)ncopy * sizeof(float), cudaMemcpyDeviceToHost), what);
    if (colors)
        TDE_CUDA(cudaMemcpy(colors, p->slab_colors, (size_t)ncopy * sizeof(tde_color), cudaMemcpyDeviceToHost),
                 what);
    return TDE_OK;
}

extern "C" {

int tde_pipeline_create(const tde_pipeline_config *cfg, const double *pose12, tde_pipeline **out) {
    if (!cfg || !pose12 || !out) return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: null argument");
    const tde_pipeline_config &c = *cfg;
    if (c.intr.cols <= 0 || c.intr.rows <= 0 || !(c.intr.fx > 0.f) || !(c.intr.fy > 0.f))
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: bad intrinsics");
    if (c.icp_levels < 1 || c.icp_levels > 3) return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: icp_levels");
    if (!valid_format(c.tsdf_format)) return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: tsdf_format");
    if (!(c.trunc > 0.f) || c.max_weight < 1 || c.max_weight > 32767 || !(c.sigma_space > 0.f) ||
        !(c.sigma_color > 0.f))
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: bad filter / truncation parameters");
    if ((c.intr.cols >> (c.icp_levels - 1)) < 8 || (c.intr.rows >> (c.icp_levels - 1)) < 8)
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: image too small for the pyramid");
    for (int l = 0; l < c.icp_levels; ++l)
        if (c.icp_iters[l] < 0 || c.icp_iters[l] > 100) return set_error(TDE_ERR_INVALID_ARG, "pipeline_create: icp_iters");
    tde_pipeline *p = new (std::nothrow) tde_pipeline();
    if (!p) return set_error(TDE_ERR_OOM, "pipeline_create: host allocation");
    p->cfg = c;
    p->levels = c.icp_levels;
    int st = tde_round_buffer_init(&p->rb, c.voxels, c.volume_size);
    if (st == TDE_OK && !valid_round_buffer(&p->rb)) st = set_error(TDE_ERR_INVALID_ARG, "pipeline_create: volume size");
    if (st != TDE_OK) { delete p; return st; }
    p->cell = tde_point3f{c.volume_size.x / c.voxels.x, c.volume_size.y / c.voxels.y, c.volume_size.z / c.voxels.z};
    for (int l = 0; l < 3; ++l) {
        int div = 1 << l;
        p->intr[l] = tde_intrinsics{c.intr.fx / div, c.intr.fy / div, c.intr.cx / div, c.intr.cy / div,
                                    c.intr.cols >> l, c.intr.rows >> l};
    }
    auto fail = [&](int code) { release(p); return code; };
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&p->prio_low, &p->prio_high);
    if (e != cudaSuccess) return fail(cuda_fail(e, "stream priorities"));
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || p->sm_count < 1) return fail(cuda_fail(e, "multiprocessor count"));
    e = cudaStreamCreateWithPriority(&p->stream, cudaStreamNonBlocking, p->prio_high);
    if (e != cudaSuccess) return fail(cuda_fail(e, "stream"));
    if ((st = make_pre_stream(p))) return fail(st);
    for (int set = 0; set < 2; ++set) {
        if ((e = cudaEventCreateWithFlags(&p->pre_done[set], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&p->set_free[set], cudaEventDisableTiming)) != cudaSuccess)
            return fail(cuda_fail(e, "event"));
    }
    const size_t npx = (size_t)c.intr.cols * c.intr.rows;
    for (int set = 0; set < 2; ++set) {
        if ((st = dalloc(&p->raw[set], npx, "raw depth")) || (st = dalloc(&p->scaled[set], npx, "scaled depth")) ||
            (st = dalloc(reinterpret_cast<char **>(&p->iscratch[set]),
                         integrate_scratch_bytes(c.intr.cols, c.intr.rows, p->rb), "integration scratch")))
            return fail(st);
        for (int l = 0; l < p->levels; ++l) {
            size_t n = (size_t)p->intr[l].cols * p->intr[l].rows;
            if ((st = dalloc(&p->depth[set][l], n, "depth pyramid")) ||
                (st = dalloc(&p->vcur[set][l], 3 * n, "vertex map")) ||
                (st = dalloc(&p->ncur[set][l], 3 * n, "normal map")))
                return fail(st);
        }
    }
    for (int l = 0; l < p->levels; ++l) {
        size_t n = (size_t)p->intr[l].cols * p->intr[l].rows;
        if ((st = dalloc(&p->vmod[l], 3 * n, "model vertices")) || (st = dalloc(&p->nmod[l], 3 * n, "model normals")))
            return fail(st);
    }
    if ((st = dalloc(&p->st, 1, "icp state")) || (st = dalloc(&p->cam, 1, "camera pose")) ||
        (st = dalloc(&p->out, 1, "frame out")) || (st = dalloc(&p->stats, 3, "stats")) ||
        (st = dalloc(&p->negflags, brick_flags_bytes(p->rb), "brick flags")) ||
        (st = dalloc(&p->satflags, brick_count(p->rb), "saturation flags")))
        return fail(st);
    e = cudaMemsetAsync(p->satflags, 0, brick_count(p->rb), p->stream);
    if (e != cudaSuccess) return fail(cuda_fail(e, "saturation flags"));
    e = cudaMemsetAsync(p->negflags, 0, brick_flags_bytes(p->rb), p->stream);
    if (e != cudaSuccess) return fail(cuda_fail(e, "brick flags"));
    e = cudaMemsetAsync(p->stats, 0, 3 * sizeof(unsigned long long), p->stream);
    if (e != cudaSuccess) return fail(cuda_fail(e, "stats"));
    if (!c.integrate_stats) { cudaFree(p->stats); p->stats = nullptr; }
    // model maps start empty (NaN) so the first ICP finds nothing before a raycast
    const size_t vb = tde_tsdf_volume_bytes(c.tsdf_format, &p->rb);
    e = cudaMalloc(&p->volume, vb);
    if (e != cudaSuccess) return fail(cuda_fail(e, "TSDF volume"));
    if ((st = launch_tsdf_init(p->volume, c.tsdf_format, voxel_count(p->rb), p->stream))) return fail(st);
    if ((st = write_pose(p, pose12))) return fail(st);
    if (c.use_graphs && (st = capture_all(p))) return fail(st);
    *out = p;
    return TDE_OK;
}

int tde_pipeline_destroy(tde_pipeline *p) {
    release(p);
    return TDE_OK;
}

void *tde_pipeline_stream(tde_pipeline *p) { return p ? (void *)p->stream : nullptr; }

int tde_pipeline_enqueue_rgbd(tde_pipeline *p, const uint16_t *depth, const uint8_t *rgb, int on_device,
                              double *pose_out12, int *status_out) {
    NvtxRange range("tde_pipeline_enqueue");
    if (!p || !depth) return set_error(TDE_ERR_INVALID_ARG, "pipeline_enqueue: null argument");
    if (p->inconsistent)
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_enqueue: a restore failed part-way; restore a checkpoint first");
    if ((p->colvol != nullptr) != (rgb != nullptr))
        return set_error(TDE_ERR_INVALID_ARG, p->colvol ? "pipeline_enqueue: the colour volume needs an RGB frame"
                                                        : "pipeline_enqueue: an RGB frame needs tde_pipeline_enable_color");
    const int depth_on_device = on_device;
    const size_t rgb_bytes = (size_t)p->cfg.intr.cols * p->cfg.intr.rows * 3;
    const size_t bytes = (size_t)p->cfg.intr.cols * p->cfg.intr.rows * sizeof(uint16_t);
    const cudaMemcpyKind kind = depth_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const int set = p->frames & 1;
    const bool first = p->frames == 0;
    const bool timed = p->timing_n < p->timing_cap;
    if (timed) {
        // timed frames run serially on the main stream, so that each pair of
        // events brackets one stage alone
        cudaEvent_t *ev = &p->ev[kEvents * p->timing_n];
        TDE_CUDA(cudaMemcpyAsync(p->raw[set], depth, bytes, kind, p->stream), "depth upload");
        if (rgb) TDE_CUDA(cudaMemcpyAsync(p->rgb[set], rgb, rgb_bytes, kind, p->stream), "rgb upload");
        const Segment order[kStages] = {SEG_PRE, first ? SEG_POST_FIRST : SEG_ICP, SEG_INTEGRATE, SEG_RAYCAST,
                                        SEG_RESIZE};
        TDE_CUDA(cudaEventRecord(ev[0], p->stream), "event");
        for (int k = 0; k < kStages; ++k) {
            TDE_TRY(run_segment(p, order[k], set, p->stream));
            // timed frames count the colour update with the raycast
            if (order[k] == SEG_RAYCAST && p->colvol) TDE_TRY(run_segment(p, SEG_COLOR, set, p->stream));
            TDE_CUDA(cudaEventRecord(ev[k + 1], p->stream), "event");
        }
        p->timing_n++;
    } else {
        // preprocessing on the second stream, once the frame two back no
        // longer reads this input set
        TDE_CUDA(cudaStreamWaitEvent(p->pre_stream, p->set_free[set], 0), "wait");
        // the colour update of the frame two back reads this set's RGB frame
        if (rgb) TDE_CUDA(cudaStreamWaitEvent(p->pre_stream, p->col_done[set], 0), "wait");
        TDE_CUDA(cudaMemcpyAsync(p->raw[set], depth, bytes, kind, p->pre_stream), "depth upload");
        if (rgb) TDE_CUDA(cudaMemcpyAsync(p->rgb[set], rgb, rgb_bytes, kind, p->pre_stream), "rgb upload");
        TDE_TRY(run_segment(p, SEG_PRE, set, p->pre_stream));
        TDE_CUDA(cudaEventRecord(p->pre_done[set], p->pre_stream), "event");
        TDE_CUDA(cudaStreamWaitEvent(p->stream, p->pre_done[set], 0), "wait");
        // ... and this set's model-map and pose snapshots, which the raycast rewrites
        if (p->colvol) TDE_CUDA(cudaStreamWaitEvent(p->stream, p->col_done[set], 0), "wait");
        if (p->cfg.use_graphs) {
            TDE_CUDA(cudaGraphLaunch(p->main_exec[set][first ? 0 : 1], p->stream), "graph launch");
        } else {
            const Segment *segs = first ? kMainFirst : kMainTracked;
            const int n = 4;
            for (int k = 0; k < n; ++k) TDE_TRY(record_segment(p, segs[k], set, p->stream));
        }
        if (p->colvol) {
            // the colour update runs beside the next frame's tracking; only the
            // frame after next waits for it
            TDE_CUDA(cudaEventRecord(p->col_ready[set], p->stream), "event");
            TDE_CUDA(cudaStreamWaitEvent(p->col_stream, p->col_ready[set], 0), "wait");
            TDE_TRY(run_segment(p, SEG_COLOR, set, p->col_stream));
            TDE_CUDA(cudaEventRecord(p->col_done[set], p->col_stream), "event");
        }
    }
    TDE_CUDA(cudaEventRecord(p->set_free[set], p->stream), "event");
    if (pose_out12)
        TDE_CUDA(cudaMemcpyAsync(pose_out12, p->out->pose, sizeof(p->out->pose), cudaMemcpyDeviceToHost, p->stream),
                 "pose download");
    if (status_out)
        TDE_CUDA(cudaMemcpyAsync(status_out, &p->out->status, sizeof(int), cudaMemcpyDeviceToHost, p->stream),
                 "status download");
    p->frames++;
    return TDE_OK;
}

int tde_pipeline_enqueue(tde_pipeline *p, const uint16_t *depth, int depth_on_device, double *pose_out12,
                         int *status_out) {
    return tde_pipeline_enqueue_rgbd(p, depth, nullptr, depth_on_device, pose_out12, status_out);
}

int tde_pipeline_enable_color(tde_pipeline *p, int max_weight) {
    if (!p || max_weight < 1) return set_error(TDE_ERR_INVALID_ARG, "pipeline_enable_color: bad argument");
    TDE_TRY(tde_pipeline_sync(p));
    if (!p->colvol) {
        const size_t n = voxel_count(p->rb), px = (size_t)p->cfg.intr.cols * p->cfg.intr.rows;
        int st;
        if ((st = dalloc(&p->colvol, n, "colour volume")) || (st = dalloc(&p->rgb[0], 3 * px, "rgb frame")) ||
            (st = dalloc(&p->rgb[1], 3 * px, "rgb frame")) || (st = dalloc(&p->vcol[0], 3 * px, "colour snapshot")) ||
            (st = dalloc(&p->vcol[1], 3 * px, "colour snapshot")) ||
            (st = dalloc(&p->cam_col[0], 1, "colour snapshot")) || (st = dalloc(&p->cam_col[1], 1, "colour snapshot")) ||
            (st = dalloc(reinterpret_cast<char **>(&p->cscratch),
                         integrate_colors_scratch_bytes(p->cfg.intr.cols, p->cfg.intr.rows, p->rb), "colour scratch")))
            return st;
        TDE_CUDA(cudaStreamCreateWithPriority(&p->col_stream, cudaStreamNonBlocking, p->prio_low), "colour stream");
        for (int set = 0; set < 2; ++set) {
            TDE_CUDA(cudaEventCreateWithFlags(&p->col_ready[set], cudaEventDisableTiming), "event");
            TDE_CUDA(cudaEventCreateWithFlags(&p->col_done[set], cudaEventDisableTiming), "event");
        }
        TDE_CUDA(cudaMemsetAsync(p->colvol, 0, n * sizeof(tde_color), p->stream), "colour volume");
    }
    p->color_max_weight = max_weight;
    TDE_TRY(tde_pipeline_sync(p));
    if (p->cfg.use_graphs) return capture_all(p);
    return TDE_OK;
}

int tde_pipeline_color_volume(tde_pipeline *p, tde_color **color_volume) {
    if (!p || !color_volume) return set_error(TDE_ERR_INVALID_ARG, "pipeline_color_volume: null");
    *color_volume = p->colvol;
    return TDE_OK;
}

int tde_pipeline_sync(tde_pipeline *p) {
    if (!p) return set_error(TDE_ERR_INVALID_ARG, "pipeline_sync: null");
    return sync_streams(p);
}

int tde_pipeline_process(tde_pipeline *p, const uint16_t *depth, int depth_on_device, double *pose12, int *status) {
    TDE_TRY(tde_pipeline_enqueue(p, depth, depth_on_device, nullptr, nullptr));
    TDE_TRY(tde_pipeline_sync(p));
    FrameOut o;
    TDE_CUDA(cudaMemcpy(&o, p->out, sizeof(o), cudaMemcpyDeviceToHost), "frame out");
    if (pose12) std::memcpy(pose12, o.pose, sizeof(o.pose));
    if (status) *status = o.status;
    return TDE_OK;
}

int tde_pipeline_pose(tde_pipeline *p, double *pose12) {
    if (!p || !pose12) return set_error(TDE_ERR_INVALID_ARG, "pipeline_pose: null");
    TDE_TRY(tde_pipeline_sync(p));
    IcpState h;
    TDE_CUDA(cudaMemcpy(&h, p->st, sizeof(h), cudaMemcpyDeviceToHost), "pose");
    std::memcpy(pose12, h.R, 9 * sizeof(double));
    std::memcpy(pose12 + 9, h.t, 3 * sizeof(double));
    return TDE_OK;
}

int tde_pipeline_volume(tde_pipeline *p, void **volume, tde_round_buffer *rb) {
    if (!p) return set_error(TDE_ERR_INVALID_ARG, "pipeline_volume: null");
    if (volume) *volume = p->volume;
    if (rb) *rb = p->rb;
    return TDE_OK;
}

int tde_pipeline_model_maps(tde_pipeline *p, int level, const float **vmap, const float **nmap) {
    if (!p || level < 0 || level >= p->levels) return set_error(TDE_ERR_INVALID_ARG, "pipeline_model_maps: level");
    if (vmap) *vmap = p->vmod[level];
    if (nmap) *nmap = p->nmod[level];
    return TDE_OK;
}

int tde_pipeline_render(tde_pipeline *p, const tde_light_source *light, uint8_t *image) {
    if (!p || !image) return set_error(TDE_ERR_INVALID_ARG, "pipeline_render: null argument");
    if (light && light->number != 0 && light->number != 1)
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_render: light.number %d (0 or 1)", light->number);
    // no light given: one light at the camera centre, read on the device
    // after the last enqueued frame published its pose
    const float *at_camera =
        light ? nullptr
              : reinterpret_cast<const float *>(reinterpret_cast<const char *>(p->cam) + offsetof(CamPose, t));
    return launch_generate_image(p->vmod[0], p->nmod[0], p->intr[0].cols, p->intr[0].rows,
                                 light ? light->pos : tde_point3f{0.f, 0.f, 0.f}, light ? light->number : 1,
                                 at_camera, image, p->stream);
}

int tde_pipeline_frame_maps(tde_pipeline *p, int level, const uint16_t **depth, const float **vmap,
                            const float **nmap) {
    if (!p || level < 0 || level >= p->levels) return set_error(TDE_ERR_INVALID_ARG, "pipeline_frame_maps: level");
    const int set = p->frames > 0 ? (p->frames - 1) & 1 : 0;  // the last enqueued frame's set
    if (depth) *depth = p->depth[set][level];
    if (vmap) *vmap = p->vcur[set][level];
    if (nmap) *nmap = p->ncur[set][level];
    return TDE_OK;
}

int tde_pipeline_frame_count(tde_pipeline *p) { return p ? p->frames : 0; }

int tde_pipeline_enable_timing(tde_pipeline *p, int capacity) {
    if (!p || capacity < 0) return set_error(TDE_ERR_INVALID_ARG, "pipeline_enable_timing: bad argument");
    TDE_TRY(tde_pipeline_sync(p));
    for (auto e : p->ev) cudaEventDestroy(e);
    p->ev.assign((size_t)kEvents * capacity, nullptr);
    for (auto &e : p->ev) TDE_CUDA(cudaEventCreate(&e), "event create");
    p->timing_cap = capacity;
    p->timing_n = 0;
    return TDE_OK;
}

int tde_pipeline_timings(tde_pipeline *p, float *integrate_ms, float *raycast_ms, int capacity) {
    if (!p || capacity < 0) return set_error(TDE_ERR_INVALID_ARG, "pipeline_timings: bad argument");
    TDE_TRY(tde_pipeline_sync(p));
    int n = p->timing_n < capacity ? p->timing_n : capacity;
    for (int i = 0; i < n; ++i) {
        cudaEvent_t *ev = &p->ev[kEvents * i];
        if (integrate_ms) TDE_CUDA(cudaEventElapsedTime(&integrate_ms[i], ev[2], ev[3]), "elapsed");
        if (raycast_ms) TDE_CUDA(cudaEventElapsedTime(&raycast_ms[i], ev[3], ev[4]), "elapsed");
    }
    return n;
}

int tde_pipeline_stage_timings(tde_pipeline *p, float *ms, int capacity) {
    if (!p || !ms || capacity < 0) return set_error(TDE_ERR_INVALID_ARG, "pipeline_stage_timings: bad argument");
    TDE_TRY(tde_pipeline_sync(p));
    int n = p->timing_n < capacity ? p->timing_n : capacity;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < kStages; ++k)
            TDE_CUDA(cudaEventElapsedTime(&ms[(size_t)i * kStages + k], p->ev[kEvents * i + k],
                                          p->ev[kEvents * i + k + 1]),
                     "elapsed");
    return n;
}

int tde_pipeline_integrate_stats(tde_pipeline *p, uint64_t *rw, int reset) {
    if (!p || !rw) return set_error(TDE_ERR_INVALID_ARG, "pipeline_integrate_stats: null");
    if (!p->stats) return set_error(TDE_ERR_UNSUPPORTED, "pipeline_integrate_stats: created without integrate_stats");
    TDE_TRY(tde_pipeline_sync(p));
    unsigned long long h[3];
    TDE_CUDA(cudaMemcpy(h, p->stats, sizeof(h), cudaMemcpyDeviceToHost), "stats");
    rw[0] = h[0];
    rw[1] = h[1];
    rw[2] = h[2];
    if (reset) TDE_CUDA(cudaMemset(p->stats, 0, sizeof(h)), "stats reset");
    return TDE_OK;
}

int tde_pipeline_launches_per_frame(tde_pipeline *p) {
    if (!p) return 0;
    int icp = 0;
    for (int l = 0; l < p->levels; ++l) icp += p->cfg.icp_iters[l];
    // bilateral (or the refiner's 11 convolutions + the level-0 vertex map),
    // pyramid levels, normal maps, scaled depth, depth tiles; ICP, brick
    // cull, integrate, raycast, the model-map pyramid; with colour, model
    // distances, their tiles, the colour brick cull and the colour update
    const int pre = p->refiner ? 12 : 1;
    return pre + (p->levels - 1) + p->levels + 2 + icp + 1 + 1 + 1 + (p->levels > 1 ? 1 : 0) + (p->colvol ? 4 : 0);
}

int tde_pipeline_set_round_buffer(tde_pipeline *p, const tde_round_buffer *rb) {
    if (!p || !valid_round_buffer(rb)) return set_error(TDE_ERR_INVALID_ARG, "pipeline_set_round_buffer: bad argument");
    if (rb->voxels_size.x != p->rb.voxels_size.x || rb->voxels_size.y != p->rb.voxels_size.y ||
        rb->voxels_size.z != p->rb.voxels_size.z)
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_set_round_buffer: the volume resolution cannot change");
    TDE_TRY(tde_pipeline_sync(p));
    p->rb = *rb;
    // logical bricks now name other voxels
    TDE_CUDA(cudaMemsetAsync(p->satflags, 0, brick_count(p->rb), p->stream), "saturation flags");
    if (p->cfg.use_graphs) return capture_all(p);
    return TDE_OK;
}

__global__ void popcount_kernel(const unsigned *__restrict__ bits, size_t words, unsigned long long *count) {
    unsigned long long c = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        c += __popc(bits[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(count, c);
}

int tde_pipeline_raycast_records(tde_pipeline *p, int skip_empty, uint64_t *records) {
    if (!p || !records) return set_error(TDE_ERR_INVALID_ARG, "pipeline_raycast_records: null argument");
    TDE_TRY(tde_pipeline_sync(p));
    const size_t n = voxel_count(p->rb), words = (n + 31) / 32;
    const int W = p->cfg.intr.cols, H = p->cfg.intr.rows;
    unsigned *bits = nullptr;
    unsigned long long *cnt = nullptr;
    float *vm = nullptr, *nm = nullptr;
    int st = TDE_OK;
    if (cudaMalloc((void **)&bits, words * 4) != cudaSuccess || cudaMalloc((void **)&cnt, 8) != cudaSuccess ||
        cudaMalloc((void **)&vm, (size_t)W * H * 12) != cudaSuccess ||
        cudaMalloc((void **)&nm, (size_t)W * H * 12) != cudaSuccess)
        st = set_error(TDE_ERR_OOM, "pipeline_raycast_records: allocation");
    if (st == TDE_OK) {
        cudaMemsetAsync(bits, 0, words * 4, p->stream);
        cudaMemsetAsync(cnt, 0, 8, p->stream);
        tde_point3f t0{0, 0, 0};
        tde_matrix3f R0{};
        st = launch_raycast(p->volume, p->cfg.tsdf_format, vm, nm, t0, R0, p->cfg.trunc, p->intr[0], p->rb, p->cell,
                            p->cam, skip_empty ? p->negflags : nullptr, p->stream, bits);
        if (st == TDE_OK) {
            popcount_kernel<<<1024, 256, 0, p->stream>>>(bits, words, cnt);
            unsigned long long h = 0;
            if (cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
                cudaStreamSynchronize(p->stream) != cudaSuccess)
                st = set_error(TDE_ERR_CUDA, "pipeline_raycast_records: %s", cudaGetErrorString(cudaGetLastError()));
            *records = h;
        }
    }
    cudaFree(bits); cudaFree(cnt); cudaFree(vm); cudaFree(nm);
    return st;
}

int tde_pipeline_model_depth(tde_pipeline *p, uint16_t *out) {
    if (!p || !out) return set_error(TDE_ERR_INVALID_ARG, "pipeline_model_depth: null argument");
    const int n = p->cfg.intr.cols * p->cfg.intr.rows;
    model_depth_kernel<<<div_up(n, 256), 256, 0, p->stream>>>(p->vmod[0], p->cam, n, out);
    return check_launch("pipeline_model_depth");
}

int tde_pipeline_set_refiner(tde_pipeline *p, tde_refiner *r) {
    if (!p) return set_error(TDE_ERR_INVALID_ARG, "pipeline_set_refiner: null pipeline");
    if (r) {
        int st = tde_refiner_check_shape(r, p->cfg.intr.rows, p->cfg.intr.cols);
        if (st != TDE_OK) return st;
    }
    TDE_TRY(tde_pipeline_sync(p));
    p->refiner = r;
    TDE_TRY(make_pre_stream(p));
    if (p->cfg.use_graphs) return capture_all(p);
    return TDE_OK;
}

int tde_pipeline_shift_needed(tde_pipeline *p, float ahead_m, float radius_m, int *delta3) {
    if (!p || !delta3 || !(radius_m >= 0.f) || !(ahead_m >= 0.f))
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_shift_needed: bad argument");
    double pose[12];
    TDE_TRY(tde_pipeline_pose(p, pose));
    return tde_pipeline_shift_needed_pose(p, pose, ahead_m, radius_m, delta3);
}

int tde_pipeline_shift_needed_pose(tde_pipeline *p, const double *pose, float ahead_m, float radius_m, int *delta3) {
    if (!p || !pose || !delta3 || !(radius_m >= 0.f) || !(ahead_m >= 0.f))
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_shift_needed: bad argument");
    const float *vs = &p->rb.volume_size.x;
    const float *cs = &p->cell.x;
    bool out = false;
    double off[3];
    for (int a = 0; a < 3; ++a) {
        // the point ahead_m along the optical axis (third column of R)
        off[a] = pose[9 + a] + ahead_m * pose[3 * a + 2] - 0.5 * vs[a];
        out |= std::fabs(off[a]) > radius_m;
    }
    for (int a = 0; a < 3; ++a) delta3[a] = out ? (int)std::lround(off[a] / cs[a]) : 0;
    return TDE_OK;
}

int tde_pipeline_shift(tde_pipeline *p, const int *delta3, tde_xyzi *points, float *weights, uint32_t capacity,
                       uint32_t *count) {
    return tde_pipeline_shift_ex(p, delta3, points, weights, nullptr, capacity, count);
}

int tde_pipeline_shift_ex(tde_pipeline *p, const int *delta3, tde_xyzi *points, float *weights, tde_color *colors,
                          uint32_t capacity, uint32_t *count) {
    NvtxRange range("tde_pipeline_shift");
    if (!p || !delta3 || !count || (capacity && !points))
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_shift: bad argument");
    const int *N = &p->rb.voxels_size.x;
    for (int a = 0; a < 3; ++a)
        if (delta3[a] <= -N[a] || delta3[a] >= N[a])
            return set_error(TDE_ERR_INVALID_ARG, "pipeline_shift: |delta| must be below the volume size");
    TDE_TRY(tde_pipeline_sync(p));
    cudaStream_t s = p->stream;
    // the slab leaving the volume, in the black-zone coordinates of
    // scan_slice_of_both_volumes.cl:63-74 (logical voxel + origin_GRID); an
    // axis without a shift gets an empty range
    tde_point3i mn, mx;
    int *pmn = &mn.x, *pmx = &mx.x;
    const int *org = &p->rb.origin_GRID.x;
    for (int a = 0; a < 3; ++a) {
        if (delta3[a] > 0) { pmn[a] = org[a]; pmx[a] = org[a] + delta3[a] - 1; }
        else if (delta3[a] < 0) { pmn[a] = org[a] + N[a] + delta3[a]; pmx[a] = org[a] + N[a] - 1; }
        else { pmn[a] = 1 << 30; pmx[a] = -(1 << 30); }
    }
    TDE_TRY(extract_points(p, "pipeline_shift", count, [&](uint32_t cap) {
        return tde_extract_slice(p->volume, p->cfg.tsdf_format, p->colvol, mn, mx, &p->rb, p->slab_scratch,
                                 p->slab_scratch_bytes, p->slab_points, p->colvol ? p->slab_colors : nullptr,
                                 p->slab_weights, cap, p->slab_count, s);
    }));
    TDE_TRY(points_to_host(p, "pipeline_shift", *count, points, weights, p->colvol ? colors : nullptr, capacity));
    TDE_TRY(tde_clean_tsdf_slice(p->volume, p->cfg.tsdf_format, mn, mx, &p->rb, s));
    if (p->colvol) TDE_TRY(tde_clean_color_slice(p->colvol, mn, mx, &p->rb, s));
    // logical bricks name other voxels after the shift (and the slab was cleaned)
    TDE_CUDA(cudaMemsetAsync(p->satflags, 0, brick_count(p->rb), s), "pipeline_shift: saturation flags");
    // brick flags only ever over-approximate; after cleaning, the cleared
    // voxels hold 0 >= 0 so stale flags stay conservative
    // advance the round buffer (round_buffer.h:25-63 fields)
    int *ogrid = &p->rb.origin_GRID.x;
    float *oglob = &p->rb.origin_GRID_global.x, *ometric = &p->rb.origin_metric.x;
    const float *cs = &p->cell.x;
    for (int a = 0; a < 3; ++a) {
        ogrid[a] = ((ogrid[a] + delta3[a]) % N[a] + N[a]) % N[a];
        oglob[a] += (float)delta3[a];
        ometric[a] += (float)delta3[a] * cs[a];
    }
    // the pose moves into the new volume frame; the model maps are cast again
    double pose[12];
    TDE_TRY(tde_pipeline_pose(p, pose));
    for (int a = 0; a < 3; ++a) pose[9 + a] -= (double)delta3[a] * cs[a];
    TDE_TRY(write_pose(p, pose));
    TDE_TRY(upload_camera(p, pose, s));
    TDE_TRY(cast_model(p, s));
    TDE_TRY(record_segment(p, SEG_RESIZE, 0, s));
    TDE_CUDA(cudaStreamSynchronize(s), "pipeline_shift");
    if (p->cfg.use_graphs) return capture_all(p, true);
    return TDE_OK;
}

int tde_pipeline_extract_volume(tde_pipeline *p, tde_xyzi *points, float *weights, tde_color *colors,
                                uint32_t capacity, uint32_t *count) {
    NvtxRange range("tde_pipeline_extract_volume");
    if (!p || !count || (capacity && !points))
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_extract_volume: bad argument");
    TDE_TRY(tde_pipeline_sync(p));
    cudaStream_t s = p->stream;
    TDE_TRY(extract_points(p, "pipeline_extract_volume", count, [&](uint32_t cap) {
        return tde_extract_tsdf_volume(p->volume, p->cfg.tsdf_format, &p->rb, p->cell, p->slab_scratch,
                                       p->slab_scratch_bytes, p->slab_points, p->slab_weights, cap, p->slab_count,
                                       s);
    }));
    if (p->colvol && colors)
        TDE_TRY(tde_extract_color_volume(p->colvol, &p->rb, p->slab_points, *count, p->cell, p->slab_colors, s));
    TDE_CUDA(cudaStreamSynchronize(s), "pipeline_extract_volume");
    return points_to_host(p, "pipeline_extract_volume", *count, points, weights, p->colvol ? colors : nullptr,
                          capacity);
}

size_t tde_pipeline_checkpoint_bytes(tde_pipeline *p) {
    if (!p) return 0;
    const CheckpointHeader h = checkpoint_layout(p);
    return sizeof(h) + h.volume_bytes + h.negflags_bytes + h.satflags_bytes + h.color_bytes;
}

int tde_pipeline_checkpoint(tde_pipeline *p, void *buffer, size_t bytes) {
    NvtxRange range("tde_pipeline_checkpoint");
    if (!p || !buffer) return set_error(TDE_ERR_INVALID_ARG, "pipeline_checkpoint: null argument");
    if (bytes < tde_pipeline_checkpoint_bytes(p))
        return set_error(TDE_ERR_CAPACITY, "pipeline_checkpoint: %zu < %zu bytes", bytes,
                         tde_pipeline_checkpoint_bytes(p));
    TDE_TRY(tde_pipeline_sync(p));
    CheckpointHeader h = checkpoint_layout(p);
    TDE_TRY(tde_pipeline_pose(p, h.pose12));
    char *o = static_cast<char *>(buffer);
    std::memcpy(o, &h, sizeof(h));
    o += sizeof(h);
    TDE_CUDA(cudaMemcpy(o, p->volume, h.volume_bytes, cudaMemcpyDeviceToHost), "pipeline_checkpoint: volume");
    o += h.volume_bytes;
    TDE_CUDA(cudaMemcpy(o, p->negflags, h.negflags_bytes, cudaMemcpyDeviceToHost), "pipeline_checkpoint: flags");
    o += h.negflags_bytes;
    TDE_CUDA(cudaMemcpy(o, p->satflags, h.satflags_bytes, cudaMemcpyDeviceToHost), "pipeline_checkpoint: flags");
    o += h.satflags_bytes;
    if (h.color_bytes)
        TDE_CUDA(cudaMemcpy(o, p->colvol, h.color_bytes, cudaMemcpyDeviceToHost), "pipeline_checkpoint: colour");
    return TDE_OK;
}

int tde_pipeline_restore(tde_pipeline *p, const void *buffer, size_t bytes) {
    NvtxRange range("tde_pipeline_restore");
    if (!p || !buffer) return set_error(TDE_ERR_INVALID_ARG, "pipeline_restore: null argument");
    CheckpointHeader h;
    if (bytes < sizeof(h)) return set_error(TDE_ERR_INVALID_ARG, "pipeline_restore: %zu bytes, no header", bytes);
    std::memcpy(&h, buffer, sizeof(h));
    if (std::memcmp(h.magic, kCheckpointMagic, 8) != 0)
        return set_error(TDE_ERR_INVALID_ARG, "pipeline_restore: not a pipeline checkpoint");
    if (!valid_round_buffer(&h.rb)) return set_error(TDE_ERR_INVALID_ARG, "pipeline_restore: bad round buffer");
    // the checkpoint must describe this pipeline's shapes and storage
    const CheckpointHeader mine = checkpoint_layout(p);
    if (h.tsdf_format != mine.tsdf_format || h.cols != mine.cols || h.rows != mine.rows || h.levels != mine.levels ||
        h.rb.voxels_size.x != mine.rb.voxels_size.x || h.rb.voxels_size.y != mine.rb.voxels_size.y ||
        h.rb.voxels_size.z != mine.rb.voxels_size.z || h.has_color != mine.has_color ||
        h.volume_bytes != mine.volume_bytes || h.negflags_bytes != mine.negflags_bytes ||
        h.satflags_bytes != mine.satflags_bytes || h.color_bytes != mine.color_bytes || h.frames < 0 ||
        h.frames > 0x7fffffff)
        return set_error(TDE_ERR_INVALID_ARG,
                         "pipeline_restore: the checkpoint's format, frame size, volume size or colour volume "
                         "differs from this pipeline's");
    // the metric geometry the volume was fused with: the volume edge (metres),
    // camera, truncation and weight caps, compared bit for bit
    if (std::memcmp(&h.rb.volume_size, &mine.rb.volume_size, sizeof(h.rb.volume_size)) != 0 ||
        std::memcmp(&h.intr, &mine.intr, sizeof(h.intr)) != 0 ||
        std::memcmp(&h.trunc, &mine.trunc, sizeof(h.trunc)) != 0 || h.max_weight != mine.max_weight ||
        h.color_max_weight != mine.color_max_weight)
        return set_error(TDE_ERR_INVALID_ARG,
                         "pipeline_restore: the checkpoint's volume edge, intrinsics, truncation or weight cap "
                         "differs from this pipeline's");
    const size_t need = sizeof(h) + h.volume_bytes + h.negflags_bytes + h.satflags_bytes + h.color_bytes;
    if (bytes < need) return set_error(TDE_ERR_INVALID_ARG, "pipeline_restore: %zu < %zu bytes", bytes, need);
    TDE_TRY(tde_pipeline_sync(p));
    // from here on a failure leaves the device state half replaced: the
    // pipeline refuses frames until a restore succeeds
    p->inconsistent = true;
    const char *i = static_cast<const char *>(buffer) + sizeof(h);
    TDE_CUDA(cudaMemcpy(p->volume, i, h.volume_bytes, cudaMemcpyHostToDevice), "pipeline_restore: volume");
    i += h.volume_bytes;
    TDE_CUDA(cudaMemcpy(p->negflags, i, h.negflags_bytes, cudaMemcpyHostToDevice), "pipeline_restore: flags");
    i += h.negflags_bytes;
    TDE_CUDA(cudaMemcpy(p->satflags, i, h.satflags_bytes, cudaMemcpyHostToDevice), "pipeline_restore: flags");
    i += h.satflags_bytes;
    if (h.color_bytes)
        TDE_CUDA(cudaMemcpy(p->colvol, i, h.color_bytes, cudaMemcpyHostToDevice), "pipeline_restore: colour");
    p->rb = h.rb;
    p->frames = (int)h.frames;
    TDE_TRY(write_pose(p, h.pose12));
    // the model maps the next frame tracks against: cast from the restored
    // volume and pose, as the checkpointed frame cast them
    cudaStream_t s = p->stream;
    TDE_TRY(upload_camera(p, h.pose12, s));
    TDE_TRY(cast_model(p, s));
    TDE_TRY(record_segment(p, SEG_RESIZE, 0, s));
    TDE_CUDA(cudaStreamSynchronize(s), "pipeline_restore");
    if (p->cfg.use_graphs) TDE_TRY(capture_all(p, true));
    p->inconsistent = false;
    return TDE_OK;
}

int tde_pipeline_set_pose(tde_pipeline *p, const double *pose12) {
    if (!p || !pose12) return set_error(TDE_ERR_INVALID_ARG, "pipeline_set_pose: null");
    TDE_TRY(tde_pipeline_sync(p));
    return write_pose(p, pose12);
}

}  // extern "C"
