// tde_slab.cuh -- slab extraction / cleaning launchers.
#pragma once
#include "tde_common.cuh"

namespace tde {

// determine_extract_step(depth, divisor) (common/src/mem_utils.cpp:43-85);
// depths outside its table: 64-voxel chunks when they divide the depth.
int slab_chunk_depth(int depth, int divisor);
size_t slab_scratch_bytes(const tde_round_buffer &rb);
int launch_extract_slice(const void *vol, int fmt, const tde_color *color, tde_point3i mn, tde_point3i mx,
                         const tde_round_buffer &rb, void *scratch, size_t scratch_bytes, tde_xyzi *pts,
                         tde_color *cols, float *wts, uint32_t capacity, uint32_t *count, int step,
                         const tde_point3f *cell, cudaStream_t stream);
// Extract_Color_Slice: colours of the set voxels of the black zone, raster order.
int launch_extract_color_slice(const tde_color *color, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                               void *scratch, size_t scratch_bytes, tde_color *cols, uint32_t capacity,
                               uint32_t *count, cudaStream_t stream);
// Extract_Color_Volume: colour of the voxel containing each metric point.
int launch_gather_colors(const tde_color *color, const tde_round_buffer &rb, const tde_xyzi *pts, uint32_t n,
                         tde_point3f cell, tde_color *out, cudaStream_t stream);
int launch_clean_tsdf_slice(void *vol, int fmt, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                            cudaStream_t stream);
int launch_clean_color_slice(tde_color *col, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                             cudaStream_t stream);

}  // namespace tde
