/*
 * tde_capi.h -- C-ABI of the GB300 KinectFusion per-frame pipeline.
 *
 * This is the drop-in boundary for 3deye's OpenCL path.  Every entry point
 * takes plain device pointers, sizes and POD structs whose layouts are byte-
 * identical to the reference's shared host/device types; no torch or CUDA
 * types appear in the signatures (a stream is an opaque `void *`, NULL meaning
 * the legacy default stream).  Each call validates its arguments, enqueues its
 * kernels on the given stream and returns a status code; nothing blocks unless
 * the comment says so.  The C++ layer in include/3deye/ restores the
 * reference's free-function API (opencl_wrappers.h) on top of these calls.
 *
 * Reference citations are paths inside the 3deye project.
 */
#ifndef TDE_CAPI_H
#define TDE_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes.  The reference aborts (common/inc/opencl_utils.h:22-50) or   */
/* throws on misuse; here every call reports instead.                         */
/* ------------------------------------------------------------------------ */
#define TDE_OK 0
#define TDE_ERR_INVALID_ARG (-1)  /* null pointer, bad size, bad format      */
#define TDE_ERR_OOM (-2)          /* device allocation failed                */
#define TDE_ERR_CUDA (-3)         /* a CUDA runtime call failed              */
#define TDE_ERR_DEVICE_TIMEOUT (-4) /* a bounded device-side wait gave up    */
#define TDE_ERR_CAPACITY (-5)     /* output buffer smaller than the result   */
#define TDE_ERR_NOT_FOUND (-6)    /* unknown kernel name                     */
#define TDE_ERR_UNSUPPORTED (-7)  /* configuration outside the supported set */

/* Last error message of the calling thread ("" when none). */
const char *tde_last_error(void);
/* Library version string. */
const char *tde_version(void);

/* ------------------------------------------------------------------------ */
/* Shared POD types (layout pinned by static_assert in the implementation).  */
/* ------------------------------------------------------------------------ */
/* point_3f / vector_3f: common/inc/elementary_points.h:35-41 */
typedef struct tde_point3f { float x, y, z; } tde_point3f;
/* point_3i: common/inc/elementary_points.h:43-48 */
typedef struct tde_point3i { int x, y, z; } tde_point3i;
/* matrix_3f, three rows: common/inc/types/elementary_matrix_template.h:1-3 */
typedef struct tde_matrix3f { tde_point3f row[3]; } tde_matrix3f;
/* intrinsics: common/inc/types/intrinsics.h:8-26 */
typedef struct tde_intrinsics { float fx, fy, cx, cy; int cols, rows; } tde_intrinsics;
/* round_buffer (72 bytes): common/inc/types/round_buffer.h:25-63 */
typedef struct tde_round_buffer {
    int start_index, end_index, buffer_length;
    tde_point3i origin_GRID;
    tde_point3f origin_GRID_global;
    tde_point3f origin_metric;
    tde_point3f volume_size;
    tde_point3i voxels_size;
} tde_round_buffer;
/* Tsdf {short value; short weight;}: common/inc/types/base_points.h:75-78 */
typedef struct tde_tsdf_i16 { int16_t value; int16_t weight; } tde_tsdf_i16;
/* Color {uchar r,g,b,w}: common/inc/types/base_points.h:87-99 */
typedef struct tde_color { uint8_t r, g, b, w; } tde_color;
/* XYZI {float x,y,z,w}: common/inc/types/base_points.h:135-157 */
typedef struct tde_xyzi { float x, y, z, w; } tde_xyzi;

/* Vertex and normal maps are Point_XYZ / Point_NXYZ arrays: three floats per
 * pixel, row-major, NaN marking an invalid pixel (base_points.h:172-186). */

/* ------------------------------------------------------------------------ */
/* TSDF storage formats.                                                     */
/*   TDE_TSDF_I16: the reference record {int16 v, int16 w}; f = v / 32767,   */
/*                 v = clamp(rtz(f * 32767), +-32767) (GPU/opencl/raycast.cl:9-27). */
/*   TDE_TSDF_F16: {binary16 f, uint16 w}, 4 bytes per voxel.                 */
/*   TDE_TSDF_F32: two planes in one buffer: float f[N], then uint16 w[N].    */
/* Voxel (x,y,z) lives at calculate_address (raycast.cl:29-47): cyclic over  */
/* origin_GRID, x fastest.                                                    */
/* ------------------------------------------------------------------------ */
#define TDE_TSDF_I16 0
#define TDE_TSDF_F16 1
#define TDE_TSDF_F32 2

/* Bytes a volume of this format and size occupies (0 on bad arguments). */
size_t tde_tsdf_volume_bytes(int format, const tde_round_buffer *rb);

/* init_tsdf (named at common/inc/constants.h:168): every voxel f = 0, w = 0. */
int tde_tsdf_init(void *volume, int format, const tde_round_buffer *rb, void *stream);

/* round_buffer(point_3i voxels, point_3f metric) constructor semantics:
 * common/src/round_buffer.cpp:5-40,84-89 (origins zero, start_index 0,
 * buffer_length = voxel count). Host-only. */
int tde_round_buffer_init(tde_round_buffer *rb, tde_point3i voxels, tde_point3f metric_size);

/* determine_extract_step(depth, step, num_of_steps, divisor):
 * common/src/mem_utils.cpp:43-85.  Depth must be 128, 256 or 512
 * (TDE_ERR_UNSUPPORTED otherwise, where the reference throws).  Host-only. */
int tde_determine_extract_step(unsigned depth, int divisor, unsigned *step, unsigned *num_of_steps);

/* ======================================================================== */
/* a1/a2: depth preprocessing                                                */
/* ======================================================================== */
/* Apply_Billateral_Filtration: common/src/opencl_wrappers.cpp:216-235,
 * kernel GPU/opencl/compute_bilateral_filtering.cl:8-57.  13x13 window
 * [c-6, min(c+7, W-1)) as the reference, weight exp(-(d2*0.5/ss^2 +
 * dz2*0.5/sc^2)), result rte(sum1/sum2) clamped to [0, 32767] and set to 0
 * above max_distance_mm (the reference's intended output; it writes sum1).
 * Pass sigma_space = 4.5, sigma_color = 30 for the reference constants
 * (common/inc/common_defines.h:20-23).  `max_distance_mm` is an integer in
 * millimetres where the reference host passes float bits (opencl_wrappers.cpp:231). */
int tde_bilateral_filter(const uint16_t *depth, uint16_t *filtered, int cols, int rows,
                         float sigma_space, float sigma_color, uint32_t max_distance_mm, void *stream);

/* Create_Pyramid: opencl_wrappers.cpp:245-271 (kernel compute_depth_pyramid,
 * absent from the reference).  dst is (src_cols>>1) x (src_rows>>1): the mean
 * of the valid pixels of the 5x5 window around (2x,2y) whose depth differs
 * from the centre by less than 3*sigma_color mm; 0 when the centre is 0. */
int tde_depth_pyramid_level(const uint16_t *src, uint16_t *dst, int src_cols, int src_rows,
                            float sigma_color, void *stream);

/* Bilateral filter then pyramid: writes levels[0..num_levels-1] (level l has
 * cols>>l x rows>>l pixels), enqueuing the two calls above in sequence. */
int tde_bilateral_pyramid(const uint16_t *depth, uint16_t *const *levels, int num_levels, int cols,
                          int rows, float sigma_space, float sigma_color, uint32_t max_distance_mm,
                          void *stream);

/* ======================================================================== */
/* a3/a4: vertex and normal maps                                             */
/* ======================================================================== */
/* Create_Vertex_Maps (one level): opencl_wrappers.cpp:281-305, intrinsics of
 * the level from intrinsics::operator() (common/src/intrinsics.cpp:7-18).
 * v = (z (u-cx)/fx, z (v-cy)/fy, z), z = depth_mm / 1000; NaN where depth 0. */
int tde_vertex_map(const uint16_t *depth, float *vmap, const tde_intrinsics *intr_level, void *stream);

/* Create_Normal_Maps (one level): opencl_wrappers.cpp:315-343 (kernel
 * compute_normal_map_eigen, absent).  Normal = eigenvector of the smallest
 * eigenvalue of the covariance of the valid vertices in the 7x7 window
 * (at least 24 valid), oriented towards the camera (n.v < 0); NaN otherwise. */
int tde_normal_map(const float *vmap, float *nmap, int cols, int rows, void *stream);

/* ======================================================================== */
/* a5/a6: ICP                                                                */
/* ======================================================================== */
/* Floats of scratch that tde_estimate_combined needs for its per-block
 * partial sums at a cols x rows level. */
size_t tde_estimate_combined_gbuf_floats(int cols, int rows);

/* Estimate_Combined: opencl_wrappers.cpp:364-438 (kernel estimate_combined,
 * absent; stage two transform_estimation.cl:4-53).  Projective point-to-plane
 * association of the current maps (camera frame) against the previous model
 * maps (global frame) with the current pose (R_cur, t_cur) and the previous
 * pose inverse (R_prev_inv, t_prev); rejects pairs farther than dist_thresh
 * metres or with sin(angle) >= angle_thresh.  Writes the 27 sums
 * [A00..A05 b0 A11..A15 b1 ... A55 b5] (the unpack order of
 * opencl_wrappers.cpp:426-437) to mbuf (device, 27 floats) in one launch,
 * using gbuf (device, tde_estimate_combined_gbuf_floats floats) as scratch.
 * Sums are compensated FP32. */
int tde_estimate_combined(const float *vmap_cur, const float *nmap_cur, const float *vmap_prev_g,
                          const float *nmap_prev_g, const tde_matrix3f *R_cur, const tde_point3f *t_cur,
                          const tde_matrix3f *R_prev_inv, const tde_point3f *t_prev,
                          const tde_intrinsics *intr, float dist_thresh, float angle_thresh,
                          float *gbuf, float *mbuf, void *stream);

/* transform_estimation (GPU/opencl/transform_estimation.cl:4-53): out[g] =
 * sum of gbuf[g*group_stride .. g*group_stride + buf_length), g = 0..26.
 * The reference hard-codes group_stride = 1200. */
int tde_transform_estimation(const float *gbuf, float *out, int buf_length, int group_stride, void *stream);

/* Clean_Buff (opencl_wrappers.cpp:994-1006, clean_buff.cl:4-11): zero 27 rows
 * of `width` floats. */
int tde_clean_buff(float *gbuf, int width, void *stream);

/* Host FP64 solve of the 27-sum system and pose update (the missing L4 step;
 * the reference's only solve is the RGBD one at opencl_wrappers.cpp:1282-1326).
 * x = A^-1 b by Cholesky; R <- exp([w]x) R, t <- exp([w]x) t + v with
 * x = (w, v).  Returns TDE_ERR_INVALID_ARG if A is not positive definite. */
int tde_icp_solve_update_host(const float *mbuf27, double *R9, double *t3, double *x6);

/* The pipeline's on-device solve-and-update step on n independent systems
 * (one warp each; device pointers; FP64 in and out: the system is solved in
 * FP32 with one float-float refinement step and the pose moved in
 * float-float): sums28[28 n] = the 27 terms in
 * the order above and an inlier count (not read), pose12[12 n] = row-major R
 * then t, updated in place, x6[6 n] = the step (w, v), ok[n] = 1 when A is
 * positive definite (else the pose is left unchanged).  Enqueued on
 * `stream`; nothing blocks. */
int tde_icp_solve_device(const double *sums28, int n, double *pose12, double *x6, int *ok, void *stream);

/* ======================================================================== */
/* a7: TSDF integration                                                      */
/* ======================================================================== */
/* scale_depth (kernel absent; called at opencl_wrappers.cpp:37-43):
 * scaled = depth_mm / 1000 * sqrt(((x-cx)/fx)^2 + ((y-cy)/fy)^2 + 1). */
int tde_scale_depth(const uint16_t *depth, float *scaled, const tde_intrinsics *intr, void *stream);

/* Integrate_Tsdf_Data: opencl_wrappers.cpp:21-64 (kernel
 * integrate_tsdf_volume, absent).  Voxel (x,y,z) centre is
 * ((x+.5)cs.x, (y+.5)cs.y, (z+.5)cs.z) in volume coordinates; the camera
 * centre t and R_inv (world->camera rotation) are in the same frame.  Voxels
 * that project outside the image, onto an invalid pixel, or lie more than
 * trunc behind the surface are not touched (whole 8^3 bricks that provably
 * qualify are skipped without being read).  Others get
 * f = (f w + min(1, sdf/trunc)) / (w + 1), w = min(w + 1, max_weight).
 * MAX_TSDF_WEIGHT is 128 (common/inc/common_defines.h:10). */
int tde_integrate_tsdf(const float *depth_scaled, void *volume, int format, float trunc,
                       const tde_matrix3f *R_inv, const tde_point3f *t, const tde_intrinsics *intr,
                       const tde_point3f *cell_size, const tde_round_buffer *rb, int max_weight,
                       void *stream);

/* Integrate_Tsdf_Data with caller-provided memory: `scratch` (device,
 * 256-byte aligned, tde_integrate_tsdf_scratch_bytes) holds the frame's
 * per-tile maximum depth, used to skip 8^3 bricks that lie entirely more than
 * trunc behind the observed surface, and the list of surviving bricks;
 * tde_integrate_tsdf allocates it on the stream itself.
 * `brick_flags` (device, tde_brick_flags_bytes, zero-initialised with the
 * volume; may be NULL) gets a 1 for every physical 8^3 brick, and every
 * physical 32^3 super-brick (stored after the brick flags), that receives a
 * negative value -- a 0 proves the brick has none, which tde_raycast_ex uses
 * to skip loads and, across whole super-bricks, samples.  Same results as
 * tde_integrate_tsdf. */
size_t tde_integrate_tsdf_scratch_bytes(int cols, int rows, const tde_round_buffer *rb);
size_t tde_brick_flags_bytes(const tde_round_buffer *rb);
int tde_integrate_tsdf_ex(const float *depth_scaled, void *volume, int format, float trunc,
                          const tde_matrix3f *R_inv, const tde_point3f *t, const tde_intrinsics *intr,
                          const tde_point3f *cell_size, const tde_round_buffer *rb, int max_weight,
                          void *scratch, size_t scratch_bytes, uint8_t *brick_flags, void *stream);

/* Integration that allocates nothing (no counterpart in the reference, whose
 * host code allocates per call).  For callers that cannot call cudaMalloc --
 * real-time loops with a memory footprint fixed at start-up, plug-in hosts
 * whose allocator owns the device, interfaces with no way to pass a scratch
 * buffer -- this takes its scratch from a fixed array in the library's static
 * device memory (tde_integrate_tsdf_noalloc_max_scratch_bytes(): 1.5 MiB,
 * enough for a 512^3 volume with a 640x480 frame; every GPU that loads the
 * library holds it until exit).  Same results as tde_integrate_tsdf; a
 * configuration needing more scratch is rejected with TDE_ERR_CAPACITY.
 * The first call on a device looks up the array's device address there
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is kept per device and CUDA context: after cudaDeviceReset the
 * next call looks it up again in the new context (again outside capture).
 * All calls share the one array: calls whose GPU work overlaps (other
 * streams, other threads) race on it and must be serialised by the caller. */
size_t tde_integrate_tsdf_noalloc_max_scratch_bytes(void);
int tde_integrate_tsdf_noalloc(const float *depth_scaled, void *volume, int format, float trunc,
                               const tde_matrix3f *R_inv, const tde_point3f *t, const tde_intrinsics *intr,
                               const tde_point3f *cell_size, const tde_round_buffer *rb, int max_weight,
                               void *stream);

/* Colour integration: Integrate_Colors (opencl_wrappers.cpp:181-214, declared at
 * opencl_wrappers.h:59-70; its kernel integrate_color_volume is absent from the
 * reference and is restated from KinectFusion's colour averaging).  color_volume holds
 * one tde_color {r, g, b, w} per voxel at the TSDF's cyclic addresses; rgb is the
 * frame, cols x rows pixels of 3 bytes (r, g, b); vertex_map is the model surface
 * raycast from the same pose (volume frame, 3 floats per pixel, NaN where empty).
 * Each voxel whose centre projects into the frame, where the model point lies
 * closer than `trunc` to that centre, takes the weighted running mean of its
 * colour and the pixel's (each channel rounded to nearest, ties to even) and its
 * weight grows by one up to min(max_weight, 255).  Bricks no update can reach are
 * skipped (the model's distances from the camera bound the voxels that can
 * change); results equal a sweep of every voxel.  R_inv, t: volume -> camera
 * rotation and the camera centre, as for tde_integrate_tsdf.  The _ex form takes
 * 256-byte aligned device scratch of tde_integrate_colors_scratch_bytes() and, in
 * `updated` (device, may be NULL), adds the count of voxels updated. */
size_t tde_integrate_colors_scratch_bytes(int cols, int rows, const tde_round_buffer *rb);
int tde_integrate_colors(tde_color *color_volume, const uint8_t *rgb, const float *vertex_map,
                         const tde_intrinsics *intr, const tde_matrix3f *R_inv, const tde_point3f *t, float trunc,
                         int max_weight, const tde_point3f *cell_size, const tde_round_buffer *rb, void *stream);
int tde_integrate_colors_ex(tde_color *color_volume, const uint8_t *rgb, const float *vertex_map,
                            const tde_intrinsics *intr, const tde_matrix3f *R_inv, const tde_point3f *t, float trunc,
                            int max_weight, const tde_point3f *cell_size, const tde_round_buffer *rb, void *scratch,
                            size_t scratch_bytes, uint64_t *updated, void *stream);

/* ======================================================================== */
/* a8/a9: raycast and model maps                                             */
/* ======================================================================== */
/* Raycast: opencl_wrappers.cpp:66-95, kernel GPU/opencl/raycast.cl:182-405.
 * Same march (step 0.8 trunc), zero-crossing test, secant refinement and
 * central-difference normals as the reference, evaluated with the same IEEE
 * float operations.  Writes global-frame vertex and normal maps. */
int tde_raycast(const void *volume, int format, float *vmap, float *nmap, const tde_point3f *t,
                const tde_matrix3f *R, float trunc, const tde_intrinsics *intr,
                const tde_round_buffer *rb, const tde_point3f *cell_size, void *stream);

/* Raycast with the brick flags kept by tde_integrate_tsdf_ex: samples in a
 * brick flagged 0 are known to be >= 0, and the march only needs such a
 * value when the previous sample was negative or the next one is; otherwise
 * their loads are skipped.  Same output as tde_raycast. */
int tde_raycast_ex(const void *volume, int format, float *vmap, float *nmap, const tde_point3f *t,
                   const tde_matrix3f *R, float trunc, const tde_intrinsics *intr,
                   const tde_round_buffer *rb, const tde_point3f *cell_size, const uint8_t *brick_flags,
                   void *stream);

/* Resize_Vertex_Map / Resize_Normal_Map: opencl_wrappers.cpp:97-146 (kernels
 * absent).  `src_cols` x `src_rows` is the source level; dst is half size.
 * Vertex: mean of the 2x2 block if all four are valid, else NaN.  Normal: the
 * normalised mean under the same rule. */
int tde_resize_vertex_map(const float *src, float *dst, int src_cols, int src_rows, void *stream);
int tde_resize_normal_map(const float *src, float *dst, int src_cols, int src_rows, void *stream);

/* Transform_Maps: opencl_wrappers.cpp:148-179, kernel transform_map.cl:6-65.
 * v' = R v + t, n' = R n, NaN passes through. */
int tde_transform_maps(const float *vmap_src, const float *nmap_src, float *vmap_dst, float *nmap_dst,
                       const tde_matrix3f *R, const tde_point3f *t, int cols, int rows, void *stream);

/* ======================================================================== */
/* a10-a12: cyclic volume, slab extraction, slab cleaning                    */
/* ======================================================================== */
/* Scratch bytes tde_extract_slice needs for a volume with this round buffer. */
size_t tde_extract_slice_scratch_bytes(const tde_round_buffer *rb);

/* Extract_Slice: opencl_wrappers.cpp:856-964 with kernels
 * scan_slice_of_both_volumes.cl:76-208 and extract_slice_as_cloud.cl:72-201.
 * Voxels in the "black zone" (scan_slice_of_both_volumes.cl:63-74) emit a
 * point for each sign change towards +x, +y, +z (both voxels with w != 0 and
 * f != 1; the +z test stops at the chunk end z+1 < chunk_end) and one for a
 * set colour.  Output order is the reference's: z chunks of
 * determine_extract_step(depth, divisor 4) in order; in each chunk the +x,
 * +y, +z and colour points, each group in (z, y, x) raster order.  Points are
 * {x+dx, y+dy, z+dz, 1.0f} in voxel units; colors[i] is the colour of the
 * voxel a point names.  `color_volume` may be NULL (no colour points, zero
 * colours); `colors` and `weights` (the named voxel's weight) may be NULL.
 * The total point count goes to *count_device (device uint32).  Points past
 * `capacity` are not written; the host wrapper reads the count and retries.
 * Bit-exact with the reference on the scan's predicate set. */
int tde_extract_slice(const void *volume, int format, const tde_color *color_volume,
                      tde_point3i min_bounds, tde_point3i max_bounds, const tde_round_buffer *rb,
                      void *scratch, size_t scratch_bytes, tde_xyzi *points, tde_color *colors,
                      float *weights, uint32_t capacity, uint32_t *count_device, void *stream);

/* Extract_Color_Slice: opencl_wrappers.cpp:687-782 (declared at
 * opencl_wrappers.h:149-156 and :193-199); its kernels
 * scan_slice_of_color_volume and extract_color_slice_as_cloud are not in the
 * reference's sources.  The colour plane of Extract_Slice on its own: every
 * voxel of the black zone whose colour is set (any of r, g, b, w non-zero,
 * Color_Point_Is_Set, scan_slice_of_both_volumes.cl:53-58) gives its colour,
 * in (z, y, x) raster order of logical voxels -- the order the reference's z
 * chunks of determine_extract_step(depth, divisor 2) give for a single plane.
 * Scratch: tde_extract_slice_scratch_bytes().  The count goes to
 * *count_device; colours past `capacity` are not written. */
int tde_extract_color_slice(const tde_color *color_volume, tde_point3i min_bounds, tde_point3i max_bounds,
                            const tde_round_buffer *rb, void *scratch, size_t scratch_bytes, tde_color *colors,
                            uint32_t capacity, uint32_t *count_device, void *stream);

/* Scratch bytes tde_extract_tsdf_volume needs (the same as the slab's). */
size_t tde_extract_tsdf_volume_scratch_bytes(const tde_round_buffer *rb);

/* Extract_Tsdf_Volume: opencl_wrappers.cpp:440-543.  Its kernels
 * (scan_the_whole_array, extract_tsdf_cloud) are not in the reference's
 * sources; the wrapper shows the shape: z chunks of
 * determine_extract_step(depth, divisor 2), three predicate planes per chunk
 * (3 * width * height * step), an in-place prefix scan, and a scatter that
 * is given Cell_Size.  Restated as the slab extraction above with every voxel
 * in the zone and no colour plane: the same +x/+y/+z predicates (the +z test
 * stops at the chunk end) in the same per-chunk plane/raster order.  A point
 * is the metric centre of the voxel it names, {(x+dx+0.5f)*cell.x,
 * (y+dy+0.5f)*cell.y, (z+dz+0.5f)*cell.z, 1.0f} in logical (origin-relative)
 * coordinates -- the V of extract_slice_as_cloud.cl:99-112 -- each step
 * rounded to float.  `weights` (the named voxel's weight) may be NULL.
 * Reads the volume twice (count, then scatter): HBM-bound. */
int tde_extract_tsdf_volume(const void *volume, int format, const tde_round_buffer *rb, tde_point3f cell_size,
                            void *scratch, size_t scratch_bytes, tde_xyzi *points, float *weights, uint32_t capacity,
                            uint32_t *count_device, void *stream);

/* Extract_Color_Volume: opencl_wrappers.cpp:545-581 (kernel extract_colors,
 * absent).  colors[i] = colour of the voxel floor(points[i] / cell) (per
 * axis, correctly rounded float division) of the logical volume; zero for a
 * point outside it.  Inverts tde_extract_tsdf_volume's voxel centres. */
int tde_extract_color_volume(const tde_color *color_volume, const tde_round_buffer *rb, const tde_xyzi *points,
                             uint32_t num_points, tde_point3f cell_size, tde_color *colors, void *stream);

/* Clean_Tsdf_Slice: opencl_wrappers.cpp:835-854 (kernel clean_tsdf_slice,
 * absent): black-zone voxels get f = 0, w = 0. */
int tde_clean_tsdf_slice(void *volume, int format, tde_point3i min_bounds, tde_point3i max_bounds,
                         const tde_round_buffer *rb, void *stream);

/* Clean_Color_Slice: opencl_wrappers.cpp:814-833, clean_color_slice.cl:41-67. */
int tde_clean_color_slice(tde_color *color_volume, tde_point3i min_bounds, tde_point3i max_bounds,
                          const tde_round_buffer *rb, void *stream);

/* ======================================================================== */
/* Shaded model image                                                        */
/* ======================================================================== */
/* light_source: common/inc/types/light_source.h:4-8 */
typedef struct tde_light_source { tde_point3f pos; int number; } tde_light_source;

/* Generate_Image: opencl_wrappers.cpp:967-992 (kernel generate_image, absent;
 * restated from the published KinectFusion image generator).  For a pixel
 * whose vertex and normal are valid: w = |dot(normalize(light.pos - v), n)|
 * (w = 1 when light.number is 0; 0 when the light sits on v), grey level
 * clamp(trunc(205 w) + 50, 0, 255) in all three channels; invalid pixels
 * are 0.  `image` is cols*rows*3 bytes (RGB8, row-major) on the device.
 * light.number must be 0 or 1 (light_source holds one position).  Every
 * float operation is correctly rounded: the image is exact. */
int tde_generate_image(const float *vmap, const float *nmap, int cols, int rows, const tde_light_source *light,
                       uint8_t *image, void *stream);

/* ======================================================================== */
/* f4: dense RGB-D (photometric) odometry                                   */
/* ======================================================================== */
/* The reference's second tracker: Prepare_Data_For_RGBD,
 * Generate_Intensity_And_Depth_Pyramid, Create_Intensity_Derivatives,
 * Accumulate_Points_Of_Interest_For_RGBD, Fill_List_Of_Valid_Correspondence_RGBD,
 * Compute_Least_Squares_Equation and Estimate_Isometry_By_RGBD
 * (opencl_wrappers.cpp:345-362, 1008-1466; declared at opencl_wrappers.h:99-103,
 * 227-292), after the RGB-D odometry of OpenCV's contrib rgbd module
 * (Steinbruecker, Sturm, Cremers 2011).  The reference copy does not run as
 * written; these entry points implement the method it follows, with its
 * conventions: 8-bit grey intensity (BT.601 luma, 14-bit fixed point), depth
 * in metres (raw mm x 0.001, valid in (0, max_depth)), 3x3 Sobel derivatives
 * (int16, zero on the image border), SOBEL_SCALE 1/8,
 * DEFAULT_DEPTH_THRESHOLD_RGBD 0.07 m.  Poses map previous-frame camera
 * points to current-frame ones (P_curr = R P_prev + t), row-major R then t,
 * FP64. */
#define TDE_RGBD_MAX_LEVELS 4
/* point_2i: common/inc/elementary_points.h */
typedef struct tde_point2i { int x, y; } tde_point2i;

/* Prepare_Data_For_RGBD: intensity (cols x rows bytes) and metric depth
 * (floats) from a depth frame (uint16 mm) and an RGB frame (3 bytes a pixel). */
int tde_rgbd_prepare(const uint16_t *depth_mm, const uint8_t *rgb, int cols, int rows, uint8_t *intensity,
                     float *depth_m, void *stream);
/* One pyramid step (Generate_Intensity_And_Depth_Pyramid's kernel
 * generate_intensity_and_depth_pyramid, absent): intensity = rounded mean of
 * each 2x2 block, depth = the block's top-left sample; outputs cols/2 x rows/2. */
int tde_rgbd_pyramid(const uint8_t *intensity, const float *depth_m, int cols, int rows, uint8_t *intensity_half,
                     float *depth_half, void *stream);
/* Create_Intensity_Derivatives (kernel create_intensity_derivatives, absent):
 * 3x3 Sobel dI/dx and dI/dy as int16. */
int tde_rgbd_derivatives(const uint8_t *intensity, int cols, int rows, int16_t *dx, int16_t *dy, void *stream);
/* Accumulate_Points_Of_Interest_For_RGBD (scan_for_interest_point.cl with its
 * x/y indexing corrected, extract_interest_points absent): the pixels with
 * dx^2 + dy^2 >= scale, raster order, into points (up to capacity); the count
 * to *count_device.  Scratch: tde_rgbd_points_scratch_bytes(). */
size_t tde_rgbd_points_scratch_bytes(int cols, int rows);
int tde_rgbd_points_of_interest(const int16_t *dx, const int16_t *dy, int cols, int rows, float scale, void *scratch,
                                size_t scratch_bytes, tde_point2i *points, uint32_t capacity, uint32_t *count_device,
                                void *stream);
/* R' = K R K^-1 and t' = K t of a pose (the projective form the
 * correspondence search takes; Calculate_Supplementary_Isometry_Using_Camera_Matrix,
 * opencl_wrappers.cpp:1176-1196), FP64 then float: proj12 = R' row-major, t'.
 * Host only. */
int tde_rgbd_projective(const double *pose12, const tde_intrinsics *intr, float *proj12);
/* Fill_List_Of_Valid_Correspondence_RGBD (scan_list_of_valid_correspondence.cl):
 * each point p of the previous frame (all pixels when points is NULL) with
 * depth z maps to q = z R' [p 1] + t' and pixel round(q.xy / q.z) of the
 * current frame; the pair is kept when that pixel lies in the image, has
 * depth within max_depth_diff of q.z and a Sobel gradient of at least
 * min_gradient / SOBEL_SCALE (the current frame's dx, dy; both NULL for no
 * gradient test, as for points already filtered by
 * tde_rgbd_points_of_interest).  corr_prev[i], corr_curr[i] = the pixels and
 * diff[i] = I_curr - I_prev for kept pairs, (0, 0), (0, 0), 100 otherwise (the
 * reference's marker); *count_device and *sum_r2_device (double) receive the
 * kept count and the sum of squared differences.  proj12 is host memory. */
int tde_rgbd_correspondences(const uint8_t *i_prev, const float *d_prev, const uint8_t *i_curr, const float *d_curr,
                             const int16_t *dx, const int16_t *dy, int cols, int rows, const tde_point2i *points,
                             uint32_t npoints, const float *proj12, float max_depth_diff, float max_depth,
                             float min_gradient, tde_point2i *corr_prev, tde_point2i *corr_curr, float *diff,
                             uint32_t *count_device, double *sum_r2_device, void *stream);
/* Compute_Least_Squares_Equation (compute_least_squares_equation.cl with its
 * row indexing corrected): over every kept pair of the previous frame's
 * pixels for pose12 (host) at this level's intrinsics, sigma = sqrt(mean
 * diff^2), w = 1 / (sigma + |diff|), C = w J (J the photometric Jacobian of the
 * current-frame point for a left perturbation exp(xi)); sums_device[0..26] =
 * the upper triangle of [A | b] with A = sum C C^T, b = -sum w diff C (the
 * 27-term layout of Estimate_Combined), sums_device[27] = the pair count;
 * *sigma_device = sigma.  Scratch: tde_rgbd_odometry_scratch_bytes(). */
int tde_rgbd_lsm(const uint8_t *i_prev, const float *d_prev, const uint8_t *i_curr, const float *d_curr,
                 const int16_t *dx, const int16_t *dy, const tde_intrinsics *intr, const double *pose12,
                 float max_depth_diff, float max_depth, float min_gradient, void *scratch, size_t scratch_bytes,
                 double *sums_device, float *sigma_device, void *stream);

/* A frame's pyramid (level 0 finest; dx, dy needed for the current frame only). */
typedef struct tde_rgbd_frame {
    const uint8_t *intensity[TDE_RGBD_MAX_LEVELS];
    const float *depth[TDE_RGBD_MAX_LEVELS];
    const int16_t *dx[TDE_RGBD_MAX_LEVELS];
    const int16_t *dy[TDE_RGBD_MAX_LEVELS];
} tde_rgbd_frame;
typedef struct tde_rgbd_params {
    int levels;                                /* 1..4 (OpenCV's default 4) */
    int iters[TDE_RGBD_MAX_LEVELS];            /* per level, 0 finest: 7, 7, 7, 10 */
    float min_gradient[TDE_RGBD_MAX_LEVELS];   /* Sobel / 8 units: 10 each */
    float max_depth_diff;                      /* DEFAULT_DEPTH_THRESHOLD_RGBD 0.07 m */
    float max_depth;                           /* 35 m */
} tde_rgbd_params;
/* The defaults above. */
void tde_rgbd_default_params(tde_rgbd_params *params);
size_t tde_rgbd_odometry_scratch_bytes(int cols, int rows);
/* Estimate_Isometry_By_RGBD: Gauss-Newton on the weighted photometric error,
 * coarse to fine, params->iters[l] steps at level l, each T <- exp(xi) T with
 * the 6x6 solve of the ICP path; intr0 is level 0's camera.  Starts from
 * init_pose12 (host; identity when NULL); the result goes to pose12_device
 * and *status_device: bit 0 (1) set when a step's solve failed (too few
 * pairs or A not positive definite) and kept its pose, bit 1 (2) when at
 * least one step solved.
 * Launches only, nothing synchronises; 256-byte aligned scratch of
 * tde_rgbd_odometry_scratch_bytes(). */
int tde_rgbd_odometry(const tde_rgbd_frame *prev, const tde_rgbd_frame *curr, const tde_intrinsics *intr0,
                      const tde_rgbd_params *params, const double *init_pose12, double *pose12_device,
                      int *status_device, void *scratch, size_t scratch_bytes, void *stream);

/* ======================================================================== */
/* Device memory helpers for hosts that do not include the CUDA headers      */
/* (the C++ layer of include/3deye/ replaces gpu_array_base's cl_mem          */
/* allocation, common/src/opencl_helper.cpp:344-420, with these).            */
/* ======================================================================== */
int tde_device_malloc(void **ptr, size_t bytes);
int tde_device_free(void *ptr);
/* kind: 0 host->device, 1 device->host, 2 device->device; synchronous. */
int tde_memcpy(void *dst, const void *src, size_t bytes, int kind);
int tde_memset(void *ptr, int value, size_t bytes);
int tde_device_synchronize(void);

#ifdef __cplusplus
}
#endif
#endif /* TDE_CAPI_H */
