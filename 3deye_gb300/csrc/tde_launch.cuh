// tde_launch.cuh -- internal launchers of the depth and raycast kernels.
#pragma once
#include "tde_common.cuh"
#include "tde_integrate.cuh"

namespace tde {

int launch_bilateral(const uint16_t *src, uint16_t *dst, int W, int H, float ss, float sc, uint32_t max_mm,
                     float *vmap, const tde_intrinsics *intr, cudaStream_t stream);
int launch_pyramid(const uint16_t *src, uint16_t *dst, int sW, int sH, float sigma_color, float *vmap,
                   const tde_intrinsics *intr_dst, cudaStream_t stream);
int launch_scale_depth(const uint16_t *depth, float *scaled, const tde_intrinsics &intr, cudaStream_t stream);
int launch_vertex_map(const uint16_t *depth, float *vmap, const tde_intrinsics &intr, cudaStream_t stream);
int launch_normal_map(const float *vmap, float *nmap, int W, int H, cudaStream_t stream);

int launch_raycast(const void *volume, int format, float *vmap, float *nmap, const tde_point3f &t,
                   const tde_matrix3f &R, float trunc, const tde_intrinsics &intr, const tde_round_buffer &rb,
                   const tde_point3f &cell, const CamPose *dpose, const uint8_t *neg_flags, cudaStream_t stream,
                   unsigned *touched = nullptr);  // touched: measurement bitmap of records read, or null
int launch_resize_map(const float *src, float *dst, int sc, int sr, bool normal, cudaStream_t stream);
// Vertex and normal maps of level 0 (c0 x r0) -> levels 1 and (v2, n2 not
// null) 2, bit-identical to two rounds of launch_resize_map.
int launch_resize_model_maps(const float *v0, const float *n0, float *v1, float *n1, float *v2, float *n2, int c0,
                             int r0, cudaStream_t stream);
int launch_transform_maps(const float *vs, const float *ns, float *vd, float *nd, const tde_matrix3f &R,
                          const tde_point3f &t, int W, int H, cudaStream_t stream);
int launch_transform_estimation(const float *gbuf, float *out, int len, int stride, cudaStream_t stream);
int launch_clean_buff(float *g, int width, cudaStream_t stream);
int launch_tsdf_init(void *vol, int fmt, size_t n, cudaStream_t stream);
// Generate_Image shading; light_dev (3 floats on the device) replaces
// `light` when not null.
int launch_generate_image(const float *vmap, const float *nmap, int W, int H, const tde_point3f &light, int nlights,
                          const float *light_dev, uint8_t *image, cudaStream_t stream);

}  // namespace tde
