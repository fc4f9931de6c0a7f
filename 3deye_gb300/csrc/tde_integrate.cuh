// tde_integrate.cuh -- integration launch parameters.
#pragma once
#include "tde_common.cuh"

namespace tde {

// Camera pose as the pipeline keeps it on the device: R (camera -> volume,
// row-major), t (camera centre in the volume frame) and R^T.
struct CamPose {
    float R[9];
    float t[3];
    float R_inv[9];
    int tracking_ok;
};

struct IntegrateParams {
    float R_inv[9];   // volume -> camera rotation
    float t[3];       // camera centre, volume frame
    float trunc;
    int max_weight;
    tde_intrinsics intr;
    tde_round_buffer rb;
    tde_point3f cell;
    size_t n;         // voxel count
    const CamPose *dpose;  // when set, R_inv and t are read from here
};

// Max observed depth per screen tile: level l has (16 << l)-pixel tiles.
constexpr int kDepthMaxLevels = 5;
// Per screen tile: the largest scaled depth (level) and the smallest
// non-zero one (level_min, kNoDepth where the tile has none).
struct DepthMaxPyramid {
    float *level[kDepthMaxLevels];
    float *level_min[kDepthMaxLevels];
    int tiles_x[kDepthMaxLevels];
};

// Physical 8^3 brick holding logical voxel (x, y, z) (cyclic volume).
__host__ __device__ __forceinline__ size_t physical_brick(int x, int y, int z, const tde_round_buffer &rb) {
    const int px = wrap_mod(x + rb.origin_GRID.x, rb.voxels_size.x);
    const int py = wrap_mod(y + rb.origin_GRID.y, rb.voxels_size.y);
    const int pz = wrap_mod(z + rb.origin_GRID.z, rb.voxels_size.z);
    const size_t nbx = (size_t)(rb.voxels_size.x + 7) / 8, nby = (size_t)(rb.voxels_size.y + 7) / 8;
    return (size_t)(px >> 3) + nbx * ((size_t)(py >> 3) + nby * (size_t)(pz >> 3));
}

// 32^3-voxel super-bricks (flag set together with the brick flag), stored
// after the brick flags; only used when every volume dimension is a multiple
// of 32.
__host__ __device__ __forceinline__ size_t physical_superbrick(int x, int y, int z, const tde_round_buffer &rb) {
    const int px = wrap_mod(x + rb.origin_GRID.x, rb.voxels_size.x);
    const int py = wrap_mod(y + rb.origin_GRID.y, rb.voxels_size.y);
    const int pz = wrap_mod(z + rb.origin_GRID.z, rb.voxels_size.z);
    const size_t nsx = (size_t)(rb.voxels_size.x + 31) / 32, nsy = (size_t)(rb.voxels_size.y + 31) / 32;
    return (size_t)(px >> 5) + nsx * ((size_t)(py >> 5) + nsy * (size_t)(pz >> 5));
}

size_t depth_max_floats(int W, int H);
size_t brick_count(const tde_round_buffer &rb);
size_t superbrick_count(const tde_round_buffer &rb);
// bytes of the flag buffer: brick flags, then super-brick flags
inline size_t brick_flags_bytes(const tde_round_buffer &rb) { return brick_count(rb) + superbrick_count(rb); }
int launch_depth_max(const float *depth_scaled, int W, int H, float *scratch, cudaStream_t stream);
// neg_flags (may be null): per physical brick, set to 1 when a write leaves a
// negative value there; a 0 therefore guarantees the brick holds no negative
// TSDF value.
// Scratch of one integration: the depth max / min pyramids (filled by
// launch_depth_max at its start) followed by the surviving-brick list.
size_t integrate_scratch_bytes(int W, int H, const tde_round_buffer &rb);
// sat_flags (may be null): per logical brick (brick_count bytes, zero when a
// pipeline starts or the round buffer moves), 1 when the last integration
// that swept the brick left every voxel at f = 1 with the maximum weight.
// Such a brick lying entirely more than the truncation distance in front of
// every observed depth it projects to would be left unchanged voxel by voxel,
// so it is not swept.
int launch_integrate(const float *depth_scaled, void *volume, int format, const IntegrateParams &P, void *scratch,
                     uint8_t *neg_flags, unsigned long long *stats, cudaStream_t stream, uint8_t *sat_flags = nullptr);
// Colour integration (Integrate_Colors): scratch of integrate_colors_scratch_bytes (256-byte aligned);
// `updated` (may be null) accumulates the count of voxels updated.
size_t integrate_colors_scratch_bytes(int W, int H, const tde_round_buffer &rb);
int launch_integrate_colors(tde_color *col, const uint8_t *rgb, const float *vmap, const IntegrateParams &P,
                            void *scratch, unsigned long long *updated, cudaStream_t stream);

}  // namespace tde
