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

int launch_integrate(const float *depth_scaled, void *volume, int format, const IntegrateParams &P,
                     unsigned long long *stats, cudaStream_t stream);

}  // namespace tde
