// tde_slab.cuh -- slab extraction / cleaning launchers.
#pragma once
#include "tde_common.cuh"

namespace tde {

int slab_chunk_depth(int depth);
size_t slab_scratch_bytes(const tde_round_buffer &rb);
int launch_extract_slice(const void *vol, int fmt, const tde_color *color, tde_point3i mn, tde_point3i mx,
                         const tde_round_buffer &rb, void *scratch, size_t scratch_bytes, tde_xyzi *pts,
                         tde_color *cols, float *wts, uint32_t capacity, uint32_t *count, cudaStream_t stream);
int launch_clean_tsdf_slice(void *vol, int fmt, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                            cudaStream_t stream);
int launch_clean_color_slice(tde_color *col, tde_point3i mn, tde_point3i mx, const tde_round_buffer &rb,
                             cudaStream_t stream);

}  // namespace tde
