/*
 * oracle.h -- CPU oracle of the KinectFusion per-frame pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/, by __graft_entry__.smoke() as
 * the checker, and by bench.py's CPU-baseline leg; never by the product path.
 *
 * Each function restates one stage of the reference (file:line cited at the
 * definition) in plain C.  Where the reference kernel exists, the
 * restatement is pinned against that kernel compiled as C (oracle/_ref, see
 * tests/golden/make_golden.py); where it is absent from the reference tree
 * (integration, pyramid, vertex/normal maps, ICP association, resize, prefix
 * scan, clean_tsdf_slice) parity is unpinned and the stage follows the
 * KinectFusion method.  Built with -ffp-contract=off so float expressions are
 * the same IEEE operations as the CUDA kernels built with -fmad=false.
 */
#ifndef TDE_ORACLE_H
#define TDE_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#include "tde_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

size_t or_voxel_address(int x, int y, int z, const tde_round_buffer *rb);
uint16_t or_float_to_half(float f);
float or_half_to_float(uint16_t h);

int or_raycast(const void *vol, int fmt, float *vmap, float *nmap, const float *t, const float *R, float trunc,
               const tde_intrinsics *intr, const tde_round_buffer *rb, const float *cell);
int64_t or_raycast_records(const void *vol, int fmt, float *vmap, float *nmap, const float *t, const float *R,
                           float trunc, const tde_intrinsics *intr, const tde_round_buffer *rb, const float *cell,
                           uint32_t *touched);
int or_bilateral(const uint16_t *src, uint16_t *dst, int W, int H, float ss, float sc, uint32_t max_mm,
                 float *ratio_out);
int or_pyramid(const uint16_t *src, uint16_t *dst, int sW, int sH, float sigma_color);
int or_scale_depth(const uint16_t *depth, float *scaled, const tde_intrinsics *intr);
int or_vertex_map(const uint16_t *depth, float *vmap, const tde_intrinsics *intr);
int or_normal_map(const float *vmap, float *nmap, int W, int H);
int or_icp_terms(const float *vcur, const float *ncur, const float *vprev, const float *nprev, const float *pose24,
                 const tde_intrinsics *intr, float dist_thresh, float angle_thresh, double *sums28,
                 uint8_t *inlier_mask);
int or_icp_solve(const double *sums27, double *R9, double *t3, double *x6);
int or_integrate(const float *depth_scaled, void *vol, int fmt, float trunc, const float *R_inv, const float *t,
                 const tde_intrinsics *intr, const float *cell, const tde_round_buffer *rb, int max_weight,
                 uint64_t *stats2);
int or_resize_map(const float *src, float *dst, int sc, int sr, int normal);
int or_transform_maps(const float *vs, const float *ns, float *vd, float *nd, const float *R, const float *t, int W,
                      int H);
int or_transform_estimation(const float *gbuf, float *out, int len, int stride);
int64_t or_extract_slice(const void *vol, int fmt, const tde_color *color, const int *mn, const int *mx,
                         const tde_round_buffer *rb, int chunk_depth, tde_xyzi *pts, tde_color *cols, float *wts,
                         int64_t capacity);
int64_t or_extract_tsdf_volume(const void *vol, int fmt, const tde_round_buffer *rb, int step, const float *cell,
                               tde_xyzi *pts, float *wts, int64_t capacity);
void or_extract_color_volume(const tde_color *color, const tde_round_buffer *rb, const tde_xyzi *pts, int64_t n,
                             const float *cell, tde_color *out);
void or_generate_image(const float *vmap, const float *nmap, int64_t npix, const float *light, int nlights,
                       uint8_t *image);
int or_clean_tsdf_slice(void *vol, int fmt, const int *mn, const int *mx, const tde_round_buffer *rb);
int or_clean_color_slice(tde_color *col, const int *mn, const int *mx, const tde_round_buffer *rb);
int or_integrate_colors(tde_color *col, const uint8_t *rgb, const float *vmap, float trunc, const float *Ri,
                        const float *t, const tde_intrinsics *in, const float *cell, const tde_round_buffer *rb,
                        int max_weight, uint64_t *updated);
int or_set_threads(int n);

/* synthetic scenes (oracle_scene.c) */
int or_render_depth(const double *scene, int nprim, const double *pose12, const tde_intrinsics *intr,
                    float *depth_m);
int or_apply_noise(const float *depth_m, uint16_t *depth_mm, int W, int H, uint32_t seed, uint32_t frame,
                   float max_range_m, float dropout);
int or_render_rgb(const double *scene, int nprim, const double *pose, const tde_intrinsics *in, uint8_t *rgb);

/* dense RGB-D odometry (oracle_rgbd.c) */
int or_rgbd_prepare(const uint16_t *depth_mm, const uint8_t *rgb, int W, int H, uint8_t *I, float *D);
int or_rgbd_pyramid(const uint8_t *I, const float *D, int W, int H, uint8_t *I2, float *D2);
int or_rgbd_sobel(const uint8_t *I, int W, int H, int16_t *dx, int16_t *dy);
int or_rgbd_points(const int16_t *dx, const int16_t *dy, int W, int H, float scale, int *points, int capacity);
void or_rgbd_projective(const double *R, const double *t, const tde_intrinsics *in, float *proj);
int or_rgbd_pairs(const uint8_t *Ip, const float *Dp, const uint8_t *Ic, const float *Dc, const int16_t *dx,
                  const int16_t *dy, const tde_intrinsics *in, const double *R, const double *t, float max_depth_diff,
                  float max_depth, float min_gradient, int *kept, float *resid, double *sum_r2);
int or_rgbd_lsm(const uint8_t *Ip, const float *Dp, const uint8_t *Ic, const float *Dc, const int16_t *dx,
                const int16_t *dy, const tde_intrinsics *in, const double *R, const double *t, float max_depth_diff,
                float max_depth, float min_gradient, double *sums, float *sigma_out);
int or_rgbd_row_single(int u, int v, float z, const float *Rt12, const tde_intrinsics *in, float dIdx, float dIdy,
                       float r, float sigma, float *row7);
int or_rgbd_odometry(const uint8_t *const *Ip, const float *const *Dp, const uint8_t *const *Ic,
                     const float *const *Dc, const int16_t *const *dx, const int16_t *const *dy,
                     const tde_intrinsics *in0, int levels, const int *iters, float max_depth_diff, float max_depth,
                     const float *min_gradient, double *pose12);

#ifdef __cplusplus
}
#endif

/* Full-FP64 model stages for the storage precision study (oracle_f64.c):
 * FP64 TSDF values with int32 weights, FP64 raycast maps, FP64 ICP terms. */
int or_scale_depth_f64(const uint16_t *depth, double *scaled, const tde_intrinsics *in);
int or_integrate_f64(const double *depth, double *tsdf, int32_t *weight, double trunc, const double *Ri,
                     const double *t, const tde_intrinsics *in, const double *cell, const tde_round_buffer *rb,
                     int max_weight);
int or_raycast_f64(const double *tsdf, double *vmap, double *nmap, const double *t, const double *R, double trunc,
                   const tde_intrinsics *intr, const tde_round_buffer *rb, const double *cell);
int or_icp_terms_f64(const float *vcur, const float *ncur, const double *vprev, const double *nprev,
                     const double *Rc, const double *tc, const double *Rpi, const double *tp,
                     const tde_intrinsics *in, double dist_thresh, double angle_thresh, double *sums);

#endif
