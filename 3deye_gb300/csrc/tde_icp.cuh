// tde_icp.cuh -- ICP launch arguments and the device-resident pose state.
#pragma once
#include "tde_common.cuh"

namespace tde {

constexpr int kIcpTerms = 28;        // 27 system terms + inlier count
constexpr int kIcpMinInliers = 6;    // fewer pairs cannot constrain 6 DoF
constexpr int kIcpStatusSolveFailed = 1;
// Copies of the cross-block accumulators: more spread the blocks' atomics,
// fewer shorten the totals read every block makes after the hand-off
// (measured at 640x480, ICP per frame: 1 copy 0.158, 2 0.152, 4 0.146,
// 8 0.148 ms).
constexpr int kIcpAccCopies = 4;
constexpr int kIcpAccBuffers = 3;  // pipeline launches rotate through these

// Float pose consumed by the association: current estimate (camera ->
// global) and the previous frame's inverse (global -> previous camera).
struct IcpPose {
    float R_cur[9], t_cur[3];
    float R_prev_inv[9], t_prev[3];
};

// Device-resident ICP state.  R/t carry the estimate in FP64; `pose` is its
// float mirror read by the kernels.
struct IcpState {
    double R[9], t[3];
    double sums[kIcpTerms];
    double x[6];
    IcpPose pose;
    int status, inliers, iterations, pad0;
    unsigned counter;  // blocks done in the running launch (reset by the last block)
    unsigned pad1[3];
    // Pipeline form: the pose launch i associated with, in slot i & 1, as
    // float-float pairs (x = hi, y = lo; R row-major, then t), and the FP64
    // pose the frame started from (kept when a solve fails).
    float2 pose_it[2][12];
    double R_start[9], t_start[3];
    // Cross-block sums as 126-bit fixed point (2^-64 units) in three 42-bit
    // limbs; integer atomics make the total independent of block order.
    // Block b adds into copy b % kIcpAccCopies to spread atomic traffic.
    // Pipeline launch i of a frame adds into buffer i % kIcpAccBuffers; the
    // one-shot form uses buffer 0.
    unsigned long long acc[kIcpAccBuffers][kIcpAccCopies][kIcpTerms][3];
};

struct CamPose;

// Where the frame's last ICP launch publishes the pose it accepts.
struct IcpPublish {
    CamPose *cam;      // float pose and inverse for integration and raycast
    double *pose12;    // row-major R, then t
    int *status;       // 0, or lost_status when a solve failed (the start pose is kept)
    int *inliers;
    int lost_status;
};

struct IcpArgs {
    const float *vcur, *ncur, *vprev, *nprev;
    int W, H;
    float fx, fy, cx, cy;
    // squared thresholds (float products, as the oracle forms them): a pair is
    // kept when |dv|^2 <= dist2 and |n x n_model|^2 < angle2
    float dist2, angle2;
    int sm_count;  // multiprocessors of the device (spreads the per-block solves)
    int narrow;    // 1: small blocks on every level (kernels of another stream share the SMs)
};
inline void icp_set_thresholds(IcpArgs &a, float dist_thresh, float angle_thresh) {
    a.dist2 = dist_thresh * dist_thresh;
    a.angle2 = angle_thresh * angle_thresh;
    a.sm_count = 1;
    a.narrow = 0;
}

// exp of the rotation part x[0..2] (Rodrigues), row-major 3x3.
__host__ __device__ inline void so3_exp(const double *x, double *R) {
    double wx = x[0], wy = x[1], wz = x[2];
    double th2 = wx * wx + wy * wy + wz * wz;
    double A, B;
    if (th2 < 1e-20) {
        A = 1.0 - th2 / 6.0;
        B = 0.5 - th2 / 24.0;
    } else {
        double th = sqrt(th2), sn, cs;
        sincos(th, &sn, &cs);
        A = sn / th;
        B = (1.0 - cs) / th2;
    }
    // R = I + A [w]x + B ([w]x)^2,  ([w]x)^2 = w w^T - th2 I
    R[0] = 1.0 + B * (wx * wx - th2); R[1] = -A * wz + B * wx * wy;       R[2] = A * wy + B * wx * wz;
    R[3] = A * wz + B * wx * wy;       R[4] = 1.0 + B * (wy * wy - th2); R[5] = -A * wx + B * wy * wz;
    R[6] = -A * wy + B * wx * wz;      R[7] = A * wx + B * wy * wz;       R[8] = 1.0 + B * (wz * wz - th2);
}

size_t icp_gbuf_floats(int W, int H);

// One-shot form: the 27 sums (and the inlier count) for the pose in
// st->pose, exact totals to mbuf[0..26]; no solve.
int launch_icp(const IcpArgs &a, IcpState *st, float *mbuf, cudaStream_t stream);
// Pipeline form: launch `iter` of a frame's ICP (iterations of all levels
// counted together), with a programmatic dependency on the previous kernel in
// the stream.  Launch 0 starts from st->R / st->t (and records it as the
// frame's start and association reference); launch i > 0 first solves the
// totals of launch i - 1 and updates the pose (every block, identically); the
// frame's last launch (`last`) also solves its own totals, accepts the pose
// (or returns to the start pose when a solve failed), commits it to st->R /
// st->t and publishes it through `pub`.
int launch_icp_step(const IcpArgs &a, IcpState *st, int iter, bool last, const IcpPublish &pub, cudaStream_t stream);
// The pipeline's float-float solve-and-update step alone (FP64 in and out), on n systems (device
// arrays: sums[28 n], pose[12 n] in place, x[6 n], ok[n]).
int launch_icp_solve(const double *sums, int n, double *pose, double *x, int *ok, cudaStream_t stream);

}  // namespace tde
