// capi.cu -- extern "C" entry points of tde_capi.h: argument validation,
// error reporting and dispatch to the kernel launchers.
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>

#include "tde_common.cuh"
#include "tde_icp.cuh"
#include "tde_integrate.cuh"
#include "tde_launch.cuh"
#include "tde_slab.cuh"

namespace tde {

static thread_local char g_err[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return TDE_OK;
}

bool valid_round_buffer(const tde_round_buffer *rb) {
    if (!rb) return false;
    const tde_point3i &n = rb->voxels_size;
    if (n.x <= 0 || n.y <= 0 || n.z <= 0) return false;
    if ((long long)n.x * n.y * n.z > 2147483647LL) return false;  // int address arithmetic
    // calculate_address (raycast.cl:44) wraps with `addr > buffer_length`, which
    // leaves addr == buffer_length in range when start_index != 0.  The reference
    // always uses start_index 0 and a wrapped origin (round_buffer.cpp:34-40), so
    // those are required here; every address then stays below the voxel count.
    if (rb->buffer_length != n.x * n.y * n.z || rb->start_index != 0) return false;
    const tde_point3i &o = rb->origin_GRID;
    if (o.x < 0 || o.y < 0 || o.z < 0 || o.x >= n.x || o.y >= n.y || o.z >= n.z) return false;
    return true;
}

namespace {

bool valid_intr(const tde_intrinsics *in) {
    return in && in->cols > 0 && in->rows > 0 && in->fx != 0.f && in->fy != 0.f && std::isfinite(in->fx) &&
           std::isfinite(in->fy) && std::isfinite(in->cx) && std::isfinite(in->cy);
}

}  // namespace

int launch_tsdf_init(void *vol, int fmt, size_t n, cudaStream_t stream) {
    // every format's empty record is all-zero bits (f = +0, w = 0)
    size_t bytes = fmt == TDE_TSDF_F32 ? n * 6 : n * 4;
    cudaError_t e = cudaMemsetAsync(vol, 0, bytes, stream);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "tsdf_init: %s", cudaGetErrorString(e));
    return TDE_OK;
}

}  // namespace tde

using namespace tde;

#define TDE_REQUIRE(cond, ...)                                                                     \
    do {                                                                                           \
        if (!(cond)) return set_error(TDE_ERR_INVALID_ARG, __VA_ARGS__);                           \
    } while (0)

extern "C" {

const char *tde_last_error(void) { return g_err; }
const char *tde_version(void) { return "3deye-gb300 0.1 (sm_103a)"; }

size_t tde_tsdf_volume_bytes(int format, const tde_round_buffer *rb) {
    if (!valid_format(format) || !valid_round_buffer(rb)) return 0;
    size_t n = voxel_count(*rb);
    return format == TDE_TSDF_F32 ? n * 6 : n * 4;
}

int tde_tsdf_init(void *volume, int format, const tde_round_buffer *rb, void *stream) {
    TDE_REQUIRE(volume, "tsdf_init: null volume");
    TDE_REQUIRE(valid_format(format), "tsdf_init: bad format %d", format);
    TDE_REQUIRE(valid_round_buffer(rb), "tsdf_init: bad round_buffer");
    return launch_tsdf_init(volume, format, voxel_count(*rb), as_stream(stream));
}

int tde_round_buffer_init(tde_round_buffer *rb, tde_point3i voxels, tde_point3f metric) {
    TDE_REQUIRE(rb, "round_buffer_init: null");
    TDE_REQUIRE(voxels.x > 0 && voxels.y > 0 && voxels.z > 0, "round_buffer_init: bad voxel counts");
    std::memset(rb, 0, sizeof(*rb));
    rb->voxels_size = voxels;
    rb->volume_size = metric;
    rb->start_index = 0;
    rb->buffer_length = voxels.x * voxels.y * voxels.z;
    return TDE_OK;
}

int tde_determine_extract_step(unsigned depth, int divisor, unsigned *step, unsigned *num_of_steps) {
    TDE_REQUIRE(step && num_of_steps, "determine_extract_step: null output");
    TDE_REQUIRE(divisor != 0, "determine_extract_step: divisor is zero");
    unsigned s;
    switch (depth) {
    case 512: s = 256; break;
    case 256: s = 128; break;
    case 128: s = 64; break;
    default: return set_error(TDE_ERR_UNSUPPORTED, "determine_extract_step: depth %u not in {128,256,512}", depth);
    }
    s /= (unsigned)divisor;
    TDE_REQUIRE(s != 0 && depth % s == 0, "determine_extract_step: depth %u not a multiple of step %u", depth, s);
    unsigned n = depth / s;
    if (n == 0) { n = 1; s = depth; }
    *step = s;
    *num_of_steps = n;
    return TDE_OK;
}

// ---------------------------------------------------------------------------
int tde_bilateral_filter(const uint16_t *depth, uint16_t *filtered, int cols, int rows, float sigma_space,
                         float sigma_color, uint32_t max_distance_mm, void *stream) {
    TDE_REQUIRE(depth && filtered, "bilateral: null buffer");
    TDE_REQUIRE(depth != filtered, "bilateral: in-place filtering is not supported");
    TDE_REQUIRE(cols > 0 && rows > 0, "bilateral: bad size %dx%d", cols, rows);
    TDE_REQUIRE(sigma_space > 0.f && sigma_color > 0.f, "bilateral: sigmas must be positive");
    return launch_bilateral(depth, filtered, cols, rows, sigma_space, sigma_color, max_distance_mm, nullptr,
                            nullptr, as_stream(stream));
}

int tde_depth_pyramid_level(const uint16_t *src, uint16_t *dst, int src_cols, int src_rows, float sigma_color,
                            void *stream) {
    TDE_REQUIRE(src && dst && src != dst, "depth_pyramid: bad buffers");
    TDE_REQUIRE(src_cols >= 2 && src_rows >= 2, "depth_pyramid: bad size %dx%d", src_cols, src_rows);
    TDE_REQUIRE(sigma_color > 0.f, "depth_pyramid: bad sigma");
    return launch_pyramid(src, dst, src_cols, src_rows, sigma_color, nullptr, nullptr, as_stream(stream));
}

int tde_bilateral_pyramid(const uint16_t *depth, uint16_t *const *levels, int num_levels, int cols, int rows,
                          float sigma_space, float sigma_color, uint32_t max_distance_mm, void *stream) {
    TDE_REQUIRE(levels && num_levels >= 1 && num_levels <= 8, "bilateral_pyramid: bad levels");
    for (int l = 0; l < num_levels; ++l) TDE_REQUIRE(levels[l], "bilateral_pyramid: null level %d", l);
    TDE_REQUIRE((cols >> (num_levels - 1)) >= 1 && (rows >> (num_levels - 1)) >= 1, "bilateral_pyramid: too many levels");
    int st = tde_bilateral_filter(depth, levels[0], cols, rows, sigma_space, sigma_color, max_distance_mm, stream);
    for (int l = 1; l < num_levels && st == TDE_OK; ++l)
        st = tde_depth_pyramid_level(levels[l - 1], levels[l], cols >> (l - 1), rows >> (l - 1), sigma_color, stream);
    return st;
}

int tde_vertex_map(const uint16_t *depth, float *vmap, const tde_intrinsics *intr, void *stream) {
    TDE_REQUIRE(depth && vmap, "vertex_map: null buffer");
    TDE_REQUIRE(valid_intr(intr), "vertex_map: bad intrinsics");
    return launch_vertex_map(depth, vmap, *intr, as_stream(stream));
}

int tde_normal_map(const float *vmap, float *nmap, int cols, int rows, void *stream) {
    TDE_REQUIRE(vmap && nmap && vmap != nmap, "normal_map: bad buffers");
    TDE_REQUIRE(cols > 0 && rows > 0, "normal_map: bad size");
    return launch_normal_map(vmap, nmap, cols, rows, as_stream(stream));
}

// ---------------------------------------------------------------------------
size_t tde_estimate_combined_gbuf_floats(int cols, int rows) {
    if (cols <= 0 || rows <= 0) return 0;
    // partials + the ICP state block (counter, pose) placed after them
    return icp_gbuf_floats(cols, rows) + (sizeof(IcpState) + 255) / sizeof(float) + 64;
}

int tde_estimate_combined(const float *vmap_cur, const float *nmap_cur, const float *vmap_prev_g,
                          const float *nmap_prev_g, const tde_matrix3f *R_cur, const tde_point3f *t_cur,
                          const tde_matrix3f *R_prev_inv, const tde_point3f *t_prev, const tde_intrinsics *intr,
                          float dist_thresh, float angle_thresh, float *gbuf, float *mbuf, void *stream) {
    TDE_REQUIRE(vmap_cur && nmap_cur && vmap_prev_g && nmap_prev_g, "estimate_combined: null map");
    TDE_REQUIRE(R_cur && t_cur && R_prev_inv && t_prev, "estimate_combined: null pose");
    TDE_REQUIRE(valid_intr(intr), "estimate_combined: bad intrinsics");
    TDE_REQUIRE(gbuf && mbuf, "estimate_combined: null gbuf/mbuf");
    cudaStream_t s = as_stream(stream);
    // state block: 256-byte aligned, after the partials
    size_t part = icp_gbuf_floats(intr->cols, intr->rows);
    uintptr_t sp = reinterpret_cast<uintptr_t>(gbuf + part);
    sp = (sp + 255) & ~uintptr_t(255);
    IcpState *st = reinterpret_cast<IcpState *>(sp);
    IcpState h;
    std::memset(&h, 0, sizeof(h));
    const float *Rc = &R_cur->row[0].x, *Rp = &R_prev_inv->row[0].x;
    for (int k = 0; k < 9; ++k) { h.pose.R_cur[k] = Rc[k]; h.pose.R_prev_inv[k] = Rp[k]; h.R[k] = Rc[k]; }
    h.pose.t_cur[0] = t_cur->x; h.pose.t_cur[1] = t_cur->y; h.pose.t_cur[2] = t_cur->z;
    h.pose.t_prev[0] = t_prev->x; h.pose.t_prev[1] = t_prev->y; h.pose.t_prev[2] = t_prev->z;
    cudaError_t e = cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "estimate_combined: %s", cudaGetErrorString(e));
    IcpArgs a;
    a.vcur = vmap_cur; a.ncur = nmap_cur; a.vprev = vmap_prev_g; a.nprev = nmap_prev_g;
    a.W = intr->cols; a.H = intr->rows;
    a.fx = intr->fx; a.fy = intr->fy; a.cx = intr->cx; a.cy = intr->cy;
    icp_set_thresholds(a, dist_thresh, angle_thresh);
    int st_code = launch_icp(a, st, mbuf, s);
    if (st_code) return st_code;
    // the host copy of h must outlive the async copy above
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "estimate_combined: %s", cudaGetErrorString(e));
    return TDE_OK;
}

int tde_transform_estimation(const float *gbuf, float *out, int buf_length, int group_stride, void *stream) {
    TDE_REQUIRE(gbuf && out, "transform_estimation: null buffer");
    TDE_REQUIRE(buf_length >= 0 && group_stride >= buf_length, "transform_estimation: bad lengths");
    return launch_transform_estimation(gbuf, out, buf_length, group_stride, as_stream(stream));
}

int tde_clean_buff(float *gbuf, int width, void *stream) {
    TDE_REQUIRE(gbuf && width > 0, "clean_buff: bad arguments");
    return launch_clean_buff(gbuf, width, as_stream(stream));
}

int tde_icp_solve_device(const double *sums28, int n, double *pose12, double *x6, int *ok, void *stream) {
    TDE_REQUIRE(n >= 0, "icp_solve_device: n < 0");
    TDE_REQUIRE(n == 0 || (sums28 && pose12 && x6 && ok), "icp_solve_device: null argument");
    return launch_icp_solve(sums28, n, pose12, x6, ok, as_stream(stream));
}

int tde_icp_solve_update_host(const float *mbuf27, double *R9, double *t3, double *x6) {
    TDE_REQUIRE(mbuf27 && R9 && t3, "icp_solve_update_host: null argument");
    double A[6][6], b[6];
    int s = 0;
    for (int k = 0; k < 6; ++k)
        for (int j = k; j < 7; ++j) {
            double v = mbuf27[s++];
            if (j == 6) b[k] = v; else { A[k][j] = v; A[j][k] = v; }
        }
    double L[6][6] = {{0}};
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j <= i; ++j) {
            double acc = A[i][j];
            for (int k = 0; k < j; ++k) acc -= L[i][k] * L[j][k];
            if (i == j) {
                if (!(acc > 1e-30)) return set_error(TDE_ERR_INVALID_ARG, "icp_solve: system not positive definite");
                L[i][i] = std::sqrt(acc);
            } else {
                L[i][j] = acc / L[j][j];
            }
        }
    double y[6], x[6];
    for (int i = 0; i < 6; ++i) {
        double acc = b[i];
        for (int k = 0; k < i; ++k) acc -= L[i][k] * y[k];
        y[i] = acc / L[i][i];
    }
    for (int i = 5; i >= 0; --i) {
        double acc = y[i];
        for (int k = i + 1; k < 6; ++k) acc -= L[k][i] * x[k];
        x[i] = acc / L[i][i];
    }
    double Ri[9];
    so3_exp(x, Ri);
    double Rn[9], tn[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) Rn[3 * r + c] = Ri[3 * r] * R9[c] + Ri[3 * r + 1] * R9[3 + c] + Ri[3 * r + 2] * R9[6 + c];
        tn[r] = Ri[3 * r] * t3[0] + Ri[3 * r + 1] * t3[1] + Ri[3 * r + 2] * t3[2] + x[3 + r];
    }
    std::memcpy(R9, Rn, sizeof(Rn));
    std::memcpy(t3, tn, sizeof(tn));
    if (x6) std::memcpy(x6, x, sizeof(x));
    return TDE_OK;
}

// ---------------------------------------------------------------------------
int tde_scale_depth(const uint16_t *depth, float *scaled, const tde_intrinsics *intr, void *stream) {
    TDE_REQUIRE(depth && scaled, "scale_depth: null buffer");
    TDE_REQUIRE(valid_intr(intr), "scale_depth: bad intrinsics");
    return launch_scale_depth(depth, scaled, *intr, as_stream(stream));
}

static int integrate_checks(const float *depth_scaled, void *volume, int format, float trunc, const tde_matrix3f *R_inv,
                            const tde_point3f *t, const tde_intrinsics *intr, const tde_point3f *cell,
                            const tde_round_buffer *rb, int max_weight) {
    TDE_REQUIRE(depth_scaled && volume, "integrate: null buffer");
    TDE_REQUIRE(valid_format(format), "integrate: bad format %d", format);
    TDE_REQUIRE(R_inv && t && cell, "integrate: null pose/cell");
    TDE_REQUIRE(valid_intr(intr), "integrate: bad intrinsics");
    TDE_REQUIRE(valid_round_buffer(rb), "integrate: bad round_buffer");
    TDE_REQUIRE(trunc > 0.f && std::isfinite(trunc), "integrate: bad truncation distance");
    TDE_REQUIRE(max_weight >= 1 && max_weight <= 32767, "integrate: bad max weight %d", max_weight);
    TDE_REQUIRE(cell->x > 0.f && cell->y > 0.f && cell->z > 0.f, "integrate: bad cell size");
    return TDE_OK;
}

static IntegrateParams integrate_params(float trunc, const tde_matrix3f *R_inv, const tde_point3f *t,
                                        const tde_intrinsics *intr, const tde_point3f *cell, const tde_round_buffer *rb,
                                        int max_weight) {
    IntegrateParams P;
    std::memcpy(P.R_inv, &R_inv->row[0].x, sizeof(P.R_inv));
    P.t[0] = t->x; P.t[1] = t->y; P.t[2] = t->z;
    P.trunc = trunc; P.max_weight = max_weight; P.intr = *intr; P.rb = *rb; P.cell = *cell;
    P.n = voxel_count(*rb); P.dpose = nullptr;
    return P;
}

size_t tde_integrate_tsdf_scratch_bytes(int cols, int rows, const tde_round_buffer *rb) {
    if (cols <= 0 || rows <= 0 || !valid_round_buffer(rb)) return 0;
    return integrate_scratch_bytes(cols, rows, *rb);
}

size_t tde_brick_flags_bytes(const tde_round_buffer *rb) {
    if (!valid_round_buffer(rb)) return 0;
    return brick_flags_bytes(*rb);
}

int tde_integrate_tsdf_ex(const float *depth_scaled, void *volume, int format, float trunc, const tde_matrix3f *R_inv,
                          const tde_point3f *t, const tde_intrinsics *intr, const tde_point3f *cell,
                          const tde_round_buffer *rb, int max_weight, void *scratch, size_t scratch_bytes,
                          uint8_t *brick_flags, void *stream) {
    int st = integrate_checks(depth_scaled, volume, format, trunc, R_inv, t, intr, cell, rb, max_weight);
    if (st) return st;
    TDE_REQUIRE(scratch && scratch_bytes >= tde_integrate_tsdf_scratch_bytes(intr->cols, intr->rows, rb),
                "integrate: scratch smaller than tde_integrate_tsdf_scratch_bytes()");
    TDE_REQUIRE((reinterpret_cast<uintptr_t>(scratch) & 255) == 0, "integrate: scratch must be 256-byte aligned");
    cudaStream_t s = as_stream(stream);
    if ((st = launch_depth_max(depth_scaled, intr->cols, intr->rows, static_cast<float *>(scratch), s))) return st;
    IntegrateParams P = integrate_params(trunc, R_inv, t, intr, cell, rb, max_weight);
    return launch_integrate(depth_scaled, volume, format, P, scratch, brick_flags, nullptr, s);
}

size_t tde_integrate_colors_scratch_bytes(int cols, int rows, const tde_round_buffer *rb) {
    if (cols <= 0 || rows <= 0 || !valid_round_buffer(rb)) return 0;
    return integrate_colors_scratch_bytes(cols, rows, *rb);
}

int tde_integrate_colors_ex(tde_color *color_volume, const uint8_t *rgb, const float *vertex_map,
                            const tde_intrinsics *intr, const tde_matrix3f *R_inv, const tde_point3f *t, float trunc,
                            int max_weight, const tde_point3f *cell, const tde_round_buffer *rb, void *scratch,
                            size_t scratch_bytes, uint64_t *updated, void *stream) {
    TDE_REQUIRE(color_volume && rgb && vertex_map && R_inv && t && cell, "integrate_colors: null argument");
    TDE_REQUIRE(valid_intr(intr), "integrate_colors: bad intrinsics");
    TDE_REQUIRE(valid_round_buffer(rb), "integrate_colors: bad round_buffer");
    TDE_REQUIRE(trunc > 0.f && std::isfinite(trunc), "integrate_colors: truncation must be positive");
    TDE_REQUIRE(max_weight >= 1, "integrate_colors: max_weight must be >= 1");
    TDE_REQUIRE(cell->x > 0.f && cell->y > 0.f && cell->z > 0.f, "integrate_colors: bad cell size");
    TDE_REQUIRE(scratch && scratch_bytes >= tde_integrate_colors_scratch_bytes(intr->cols, intr->rows, rb),
                "integrate_colors: scratch smaller than tde_integrate_colors_scratch_bytes()");
    TDE_REQUIRE((reinterpret_cast<uintptr_t>(scratch) & 255) == 0, "integrate_colors: scratch must be 256-byte aligned");
    IntegrateParams P = integrate_params(trunc, R_inv, t, intr, cell, rb, max_weight);
    return launch_integrate_colors(color_volume, rgb, vertex_map, P, scratch,
                                   reinterpret_cast<unsigned long long *>(updated), as_stream(stream));
}

int tde_integrate_colors(tde_color *color_volume, const uint8_t *rgb, const float *vertex_map,
                         const tde_intrinsics *intr, const tde_matrix3f *R_inv, const tde_point3f *t, float trunc,
                         int max_weight, const tde_point3f *cell, const tde_round_buffer *rb, void *stream) {
    TDE_REQUIRE(valid_intr(intr) && valid_round_buffer(rb), "integrate_colors: bad intrinsics or round_buffer");
    cudaStream_t s = as_stream(stream);
    const size_t sb = tde_integrate_colors_scratch_bytes(intr->cols, intr->rows, rb);
    void *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sb, s);
    if (e != cudaSuccess) return set_error(TDE_ERR_OOM, "integrate_colors: scratch: %s", cudaGetErrorString(e));
    int st = tde_integrate_colors_ex(color_volume, rgb, vertex_map, intr, R_inv, t, trunc, max_weight, cell, rb, scratch,
                                     sb, nullptr, stream);
    e = cudaFreeAsync(scratch, s);
    if (st == TDE_OK && e != cudaSuccess) return set_error(TDE_ERR_CUDA, "integrate_colors: %s", cudaGetErrorString(e));
    return st;
}

int tde_integrate_tsdf(const float *depth_scaled, void *volume, int format, float trunc, const tde_matrix3f *R_inv,
                       const tde_point3f *t, const tde_intrinsics *intr, const tde_point3f *cell,
                       const tde_round_buffer *rb, int max_weight, void *stream) {
    int st = integrate_checks(depth_scaled, volume, format, trunc, R_inv, t, intr, cell, rb, max_weight);
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    const size_t sb = tde_integrate_tsdf_scratch_bytes(intr->cols, intr->rows, rb);
    void *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sb, s);
    if (e != cudaSuccess) return set_error(TDE_ERR_OOM, "integrate: scratch: %s", cudaGetErrorString(e));
    st = tde_integrate_tsdf_ex(depth_scaled, volume, format, trunc, R_inv, t, intr, cell, rb, max_weight, scratch, sb,
                               nullptr, stream);
    e = cudaFreeAsync(scratch, s);
    if (st == TDE_OK && e != cudaSuccess) return set_error(TDE_ERR_CUDA, "integrate: %s", cudaGetErrorString(e));
    return st;
}

int tde_raycast_ex(const void *volume, int format, float *vmap, float *nmap, const tde_point3f *t,
                   const tde_matrix3f *R, float trunc, const tde_intrinsics *intr, const tde_round_buffer *rb,
                   const tde_point3f *cell, const uint8_t *brick_flags, void *stream) {
    TDE_REQUIRE(volume && vmap && nmap, "raycast: null buffer");
    TDE_REQUIRE(valid_format(format), "raycast: bad format %d", format);
    TDE_REQUIRE(t && R && cell, "raycast: null pose/cell");
    TDE_REQUIRE(valid_intr(intr), "raycast: bad intrinsics");
    TDE_REQUIRE(valid_round_buffer(rb), "raycast: bad round_buffer");
    TDE_REQUIRE(trunc > 0.f && std::isfinite(trunc), "raycast: bad truncation distance");
    TDE_REQUIRE(cell->x > 0.f && cell->y > 0.f && cell->z > 0.f, "raycast: bad cell size");
    return launch_raycast(volume, format, vmap, nmap, *t, *R, trunc, *intr, *rb, *cell, nullptr, brick_flags,
                          as_stream(stream));
}

int tde_raycast(const void *volume, int format, float *vmap, float *nmap, const tde_point3f *t, const tde_matrix3f *R,
                float trunc, const tde_intrinsics *intr, const tde_round_buffer *rb, const tde_point3f *cell,
                void *stream) {
    return tde_raycast_ex(volume, format, vmap, nmap, t, R, trunc, intr, rb, cell, nullptr, stream);
}

int tde_resize_vertex_map(const float *src, float *dst, int src_cols, int src_rows, void *stream) {
    TDE_REQUIRE(src && dst && src != dst, "resize_vertex_map: bad buffers");
    TDE_REQUIRE(src_cols >= 2 && src_rows >= 2, "resize_vertex_map: bad size");
    return launch_resize_map(src, dst, src_cols, src_rows, false, as_stream(stream));
}

int tde_resize_normal_map(const float *src, float *dst, int src_cols, int src_rows, void *stream) {
    TDE_REQUIRE(src && dst && src != dst, "resize_normal_map: bad buffers");
    TDE_REQUIRE(src_cols >= 2 && src_rows >= 2, "resize_normal_map: bad size");
    return launch_resize_map(src, dst, src_cols, src_rows, true, as_stream(stream));
}

int tde_transform_maps(const float *vmap_src, const float *nmap_src, float *vmap_dst, float *nmap_dst,
                       const tde_matrix3f *R, const tde_point3f *t, int cols, int rows, void *stream) {
    TDE_REQUIRE(vmap_src && nmap_src && vmap_dst && nmap_dst, "transform_maps: null buffer");
    TDE_REQUIRE(R && t && cols > 0 && rows > 0, "transform_maps: bad arguments");
    return launch_transform_maps(vmap_src, nmap_src, vmap_dst, nmap_dst, *R, *t, cols, rows, as_stream(stream));
}

// ---------------------------------------------------------------------------
size_t tde_extract_slice_scratch_bytes(const tde_round_buffer *rb) {
    if (!valid_round_buffer(rb)) return 0;
    return slab_scratch_bytes(*rb);
}

int tde_extract_slice(const void *volume, int format, const tde_color *color_volume, tde_point3i min_bounds,
                      tde_point3i max_bounds, const tde_round_buffer *rb, void *scratch, size_t scratch_bytes,
                      tde_xyzi *points, tde_color *colors, float *weights, uint32_t capacity,
                      uint32_t *count_device, void *stream) {
    TDE_REQUIRE(volume && scratch && count_device, "extract_slice: null buffer");
    TDE_REQUIRE(points || capacity == 0, "extract_slice: null points with capacity %u", capacity);
    TDE_REQUIRE(valid_format(format), "extract_slice: bad format %d", format);
    TDE_REQUIRE(valid_round_buffer(rb), "extract_slice: bad round_buffer");
    return launch_extract_slice(volume, format, color_volume, min_bounds, max_bounds, *rb, scratch, scratch_bytes,
                                points, colors, weights, capacity, count_device, 0, nullptr, as_stream(stream));
}

int tde_extract_color_slice(const tde_color *color_volume, tde_point3i min_bounds, tde_point3i max_bounds,
                            const tde_round_buffer *rb, void *scratch, size_t scratch_bytes, tde_color *colors,
                            uint32_t capacity, uint32_t *count_device, void *stream) {
    TDE_REQUIRE(color_volume && scratch && count_device, "extract_color_slice: null buffer");
    TDE_REQUIRE(colors || capacity == 0, "extract_color_slice: null colours with capacity %u", capacity);
    TDE_REQUIRE(valid_round_buffer(rb), "extract_color_slice: bad round_buffer");
    return launch_extract_color_slice(color_volume, min_bounds, max_bounds, *rb, scratch, scratch_bytes, colors,
                                      capacity, count_device, as_stream(stream));
}

size_t tde_extract_tsdf_volume_scratch_bytes(const tde_round_buffer *rb) {
    if (!valid_round_buffer(rb)) return 0;
    return slab_scratch_bytes(*rb);
}

static bool valid_cell(tde_point3f c) {
    return std::isfinite(c.x) && std::isfinite(c.y) && std::isfinite(c.z) && c.x > 0.f && c.y > 0.f && c.z > 0.f;
}

int tde_extract_tsdf_volume(const void *volume, int format, const tde_round_buffer *rb, tde_point3f cell_size,
                            void *scratch, size_t scratch_bytes, tde_xyzi *points, float *weights, uint32_t capacity,
                            uint32_t *count_device, void *stream) {
    TDE_REQUIRE(volume && scratch && count_device, "extract_tsdf_volume: null buffer");
    TDE_REQUIRE(points || capacity == 0, "extract_tsdf_volume: null points with capacity %u", capacity);
    TDE_REQUIRE(valid_format(format), "extract_tsdf_volume: bad format %d", format);
    TDE_REQUIRE(valid_round_buffer(rb), "extract_tsdf_volume: bad round_buffer");
    TDE_REQUIRE(valid_cell(cell_size), "extract_tsdf_volume: cell size must be finite and positive");
    // every voxel is in the zone: the slab scan over the whole volume, in
    // chunks of determine_extract_step(depth, divisor 2)
    const tde_point3i lo = {INT_MIN, INT_MIN, INT_MIN}, hi = {INT_MAX, INT_MAX, INT_MAX};
    return launch_extract_slice(volume, format, nullptr, lo, hi, *rb, scratch, scratch_bytes, points, nullptr,
                                weights, capacity, count_device, slab_chunk_depth(rb->voxels_size.z, 2), &cell_size,
                                as_stream(stream));
}

int tde_extract_color_volume(const tde_color *color_volume, const tde_round_buffer *rb, const tde_xyzi *points,
                             uint32_t num_points, tde_point3f cell_size, tde_color *colors, void *stream) {
    TDE_REQUIRE(color_volume && (num_points == 0 || (points && colors)), "extract_color_volume: null buffer");
    TDE_REQUIRE(valid_round_buffer(rb), "extract_color_volume: bad round_buffer");
    TDE_REQUIRE(valid_cell(cell_size), "extract_color_volume: cell size must be finite and positive");
    return launch_gather_colors(color_volume, *rb, points, num_points, cell_size, colors, as_stream(stream));
}

int tde_generate_image(const float *vmap, const float *nmap, int cols, int rows, const tde_light_source *light,
                       uint8_t *image, void *stream) {
    TDE_REQUIRE(vmap && nmap && image && light, "generate_image: null buffer");
    TDE_REQUIRE(cols > 0 && rows > 0, "generate_image: bad size %dx%d", cols, rows);
    TDE_REQUIRE(light->number == 0 || light->number == 1, "generate_image: light.number %d (0 or 1)",
                light->number);
    return launch_generate_image(vmap, nmap, cols, rows, light->pos, light->number, nullptr, image,
                                 as_stream(stream));
}

int tde_clean_tsdf_slice(void *volume, int format, tde_point3i min_bounds, tde_point3i max_bounds,
                         const tde_round_buffer *rb, void *stream) {
    TDE_REQUIRE(volume, "clean_tsdf_slice: null volume");
    TDE_REQUIRE(valid_format(format), "clean_tsdf_slice: bad format %d", format);
    TDE_REQUIRE(valid_round_buffer(rb), "clean_tsdf_slice: bad round_buffer");
    return launch_clean_tsdf_slice(volume, format, min_bounds, max_bounds, *rb, as_stream(stream));
}

int tde_clean_color_slice(tde_color *color_volume, tde_point3i min_bounds, tde_point3i max_bounds,
                          const tde_round_buffer *rb, void *stream) {
    TDE_REQUIRE(color_volume, "clean_color_slice: null volume");
    TDE_REQUIRE(valid_round_buffer(rb), "clean_color_slice: bad round_buffer");
    return launch_clean_color_slice(color_volume, min_bounds, max_bounds, *rb, as_stream(stream));
}

// ---------------------------------------------------------------------------
int tde_device_malloc(void **ptr, size_t bytes) {
    TDE_REQUIRE(ptr, "device_malloc: null");
    cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 1);
    if (e != cudaSuccess)
        return set_error(e == cudaErrorMemoryAllocation ? TDE_ERR_OOM : TDE_ERR_CUDA, "device_malloc(%zu): %s", bytes,
                         cudaGetErrorString(e));
    return TDE_OK;
}

int tde_device_free(void *ptr) {
    cudaError_t e = cudaFree(ptr);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "device_free: %s", cudaGetErrorString(e));
    return TDE_OK;
}

int tde_memcpy(void *dst, const void *src, size_t bytes, int kind) {
    TDE_REQUIRE((dst && src) || bytes == 0, "memcpy: null pointer");
    TDE_REQUIRE(kind >= 0 && kind <= 2, "memcpy: bad kind %d", kind);
    const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost
                                                                              : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpy(dst, src, bytes, k);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "memcpy: %s", cudaGetErrorString(e));
    return TDE_OK;
}

int tde_memset(void *ptr, int value, size_t bytes) {
    TDE_REQUIRE(ptr || bytes == 0, "memset: null pointer");
    cudaError_t e = cudaMemset(ptr, value, bytes);
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    return TDE_OK;
}

int tde_device_synchronize(void) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return set_error(TDE_ERR_CUDA, "synchronize: %s", cudaGetErrorString(e));
    return TDE_OK;
}

}  // extern "C"
