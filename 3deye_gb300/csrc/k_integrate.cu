// k_integrate.cu -- projective TSDF integration (Integrate_Tsdf_Data,
// common/src/opencl_wrappers.cpp:21-64; the reference kernel
// integrate_tsdf_volume is absent, this follows the KinectFusion update).
//
// One thread per (x, y) voxel column, sweeping z.  The z range whose voxels
// can land inside the image in front of the camera is bounded analytically per
// column (each image edge is a linear inequality in z); the bound is widened
// by a tolerance and only limits which voxels are evaluated -- the per-voxel
// test below, identical to the CPU oracle's, decides.  Voxels more than
// `trunc` behind the observed surface are neither read nor written; a voxel
// whose record does not change is not written.
//
// Built with -fmad=false so every voxel decision and value equals the oracle's.
#include "tde_common.cuh"
#include "tde_integrate.cuh"

namespace tde {
namespace {

constexpr int kZBatch = 4;

__device__ __forceinline__ void bound_linear(float p, float q, float tol, float &lo, float &hi) {
    // keep z with p + q z >= -tol
    if (fabsf(q) < 1e-20f) {
        if (p < -tol) { lo = 1.f; hi = 0.f; }
        return;
    }
    float z = (-tol - p) / q;
    if (q > 0.f) lo = fmaxf(lo, z); else hi = fminf(hi, z);
}

template <int FMT>
__global__ void __launch_bounds__(256) integrate_kernel(const float *__restrict__ depth, void *__restrict__ vol,
                                                        const IntegrateParams P,
                                                        unsigned long long *__restrict__ stats) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const tde_round_buffer &rb = P.rb;
    __shared__ float s_pose[12];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid < 12) {
        if (P.dpose) s_pose[tid] = tid < 9 ? P.dpose->R_inv[tid] : P.dpose->t[tid - 9];
        else s_pose[tid] = tid < 9 ? P.R_inv[tid] : P.t[tid - 9];
    }
    __syncthreads();
    unsigned n_read = 0, n_written = 0;
    if (x < rb.voxels_size.x && y < rb.voxels_size.y) {
        float Ri[9];
        #pragma unroll
        for (int k = 0; k < 9; ++k) Ri[k] = s_pose[k];
        const float tx = s_pose[9], ty = s_pose[10], tz = s_pose[11];
        const float gx = ((float)x + 0.5f) * P.cell.x - tx;
        const float gy = ((float)y + 0.5f) * P.cell.y - ty;
        const int W = P.intr.cols, H = P.intr.rows;
        const int Nz = rb.voxels_size.z;

        // --- conservative z interval ------------------------------------
        // v(z) = c + z d  (camera frame), d = R_inv[:,2] * cell.z
        const float hz = 0.5f * P.cell.z - tz;
        float cxv = Ri[0] * gx + Ri[1] * gy + Ri[2] * hz;
        float cyv = Ri[3] * gx + Ri[4] * gy + Ri[5] * hz;
        float czv = Ri[6] * gx + Ri[7] * gy + Ri[8] * hz;
        float dxv = Ri[2] * P.cell.z, dyv = Ri[5] * P.cell.z, dzv = Ri[8] * P.cell.z;
        float lo = 0.f, hi = (float)(Nz - 1);
        const float scale = fabsf(cxv) + fabsf(cyv) + fabsf(czv) + (fabsf(dxv) + fabsf(dyv) + fabsf(dzv)) * (float)Nz;
        const float tol = 1e-4f * scale * (P.intr.fx + P.intr.fy + (float)(W + H)) + 1e-6f;
        bound_linear(czv, dzv, 1e-4f * scale + 1e-6f, lo, hi);                           // v.z > 0
        const float fx = P.intr.fx, fy = P.intr.fy, ccx = P.intr.cx, ccy = P.intr.cy;
        bound_linear(fx * cxv + (ccx + 0.5f) * czv, fx * dxv + (ccx + 0.5f) * dzv, tol, lo, hi);   // u >= -0.5
        bound_linear(-(fx * cxv + (ccx - (float)W + 0.5f) * czv), -(fx * dxv + (ccx - (float)W + 0.5f) * dzv), tol, lo, hi);
        bound_linear(fy * cyv + (ccy + 0.5f) * czv, fy * dyv + (ccy + 0.5f) * dzv, tol, lo, hi);
        bound_linear(-(fy * cyv + (ccy - (float)H + 0.5f) * czv), -(fy * dyv + (ccy - (float)H + 0.5f) * dzv), tol, lo, hi);
        int z0 = 0, z1 = -1;
        if (lo <= hi) {
            z0 = max(0, (int)floorf(lo) - 2);
            z1 = min(Nz - 1, (int)ceilf(hi) + 2);
        }

        const float ntrunc = -P.trunc;
        for (int zb = z0; zb <= z1; zb += kZBatch) {
            size_t idx[kZBatch];
            float sdfv[kZBatch];
            bool take[kZBatch];
            #pragma unroll
            for (int k = 0; k < kZBatch; ++k) {
                const int z = zb + k;
                take[k] = false;
                sdfv[k] = 0.f;
                idx[k] = 0;
                if (z > z1) continue;
                const float gz = ((float)z + 0.5f) * P.cell.z - tz;
                float vx = 0.f; vx += Ri[0] * gx; vx += Ri[1] * gy; vx += Ri[2] * gz;
                float vy = 0.f; vy += Ri[3] * gx; vy += Ri[4] * gy; vy += Ri[5] * gz;
                float vz = 0.f; vz += Ri[6] * gx; vz += Ri[7] * gy; vz += Ri[8] * gz;
                if (!(vz > 0.f)) continue;
                const int u = __float2int_rn(vx * fx / vz + ccx);
                const int v = __float2int_rn(vy * fy / vz + ccy);
                if (u < 0 || u >= W || v < 0 || v >= H) continue;
                const float Dp = __ldg(depth + (size_t)v * W + u);
                if (Dp == 0.f) continue;
                float n2 = 0.f; n2 += gx * gx; n2 += gy * gy; n2 += gz * gz;
                const float sdf = Dp - sqrtf(n2);
                if (!(sdf >= ntrunc)) continue;
                take[k] = true;
                sdfv[k] = sdf;
                idx[k] = voxel_address(x, y, z, rb);
            }
            typedef TsdfStore<FMT> S;
            typename S::Raw raw[kZBatch];
            #pragma unroll
            for (int k = 0; k < kZBatch; ++k)
                if (take[k]) raw[k] = S::load_raw(vol, idx[k], P.n);
            #pragma unroll
            for (int k = 0; k < kZBatch; ++k) {
                if (!take[k]) continue;
                ++n_read;
                float fo;
                int wo;
                S::decode(raw[k], fo, wo);
                const float tsdf = fminf(1.f, sdfv[k] / P.trunc);
                const float fw = (float)wo;
                const float fnew = (fo * fw + tsdf) / (fw + 1.f);
                const int wnew = min(wo + 1, P.max_weight);
                const typename S::Raw rn = S::encode(fnew, wnew);
                if (!S::same(rn, raw[k])) {
                    S::store_raw(vol, idx[k], P.n, rn);
                    ++n_written;
                }
            }
        }
    }
    if (stats) {
        unsigned r = n_read, w = n_written;
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r += __shfl_down_sync(0xffffffffu, r, off);
            w += __shfl_down_sync(0xffffffffu, w, off);
        }
        if ((threadIdx.x & 31) == 0 && (r | w)) {
            atomicAdd(stats, (unsigned long long)r);
            atomicAdd(stats + 1, (unsigned long long)w);
        }
    }
}

}  // namespace

int launch_integrate(const float *depth_scaled, void *volume, int format, const IntegrateParams &P,
                     unsigned long long *stats, cudaStream_t stream) {
    dim3 block(32, 8);
    dim3 grid(div_up(P.rb.voxels_size.x, 32), div_up(P.rb.voxels_size.y, 8));
    return dispatch_format(format, [&](auto F) {
        integrate_kernel<decltype(F)::value><<<grid, block, 0, stream>>>(depth_scaled, volume, P, stats);
        return check_launch("integrate_tsdf");
    });
}

}  // namespace tde
