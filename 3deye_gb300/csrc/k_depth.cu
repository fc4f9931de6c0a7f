// k_depth.cu -- depth preprocessing: bilateral filter, depth pyramid, scaled
// depth, vertex maps and PCA normal maps.
#include "tde_common.cuh"

namespace tde {
namespace {

constexpr int kBR = 6;   // bilateral radius, compute_bilateral_filtering.cl:19
constexpr int kBX = 32, kBY = 8;
constexpr int kTileW = kBX + 2 * kBR, kTileH = kBY + 2 * kBR;

// compute_bilateral_filtering.cl:8-57, intended output.  The window is
// [c-6, min(c+7, W-1)) on each axis exactly as the reference writes it, so the
// last column / row of the image never contributes.
__global__ void __launch_bounds__(kBX *kBY) bilateral_kernel(const uint16_t *__restrict__ src,
                                                             uint16_t *__restrict__ dst, int W, int H,
                                                             float inv_half_ss, float inv_half_sc,
                                                             uint32_t max_mm, float *__restrict__ vmap,
                                                             float fx, float fy, float cx, float cy) {
    // depths staged as floats: int->float conversion runs at a quarter of the
    // FMA rate, so it is done once per pixel instead of three times per tap
    __shared__ float tile[kTileH][kTileW + 1];
    __shared__ float s_space[2 * kBR + 1][2 * kBR + 1];
    const int bx0 = blockIdx.x * kBX - kBR, by0 = blockIdx.y * kBY - kBR;
    const int tid = threadIdx.y * kBX + threadIdx.x;
    for (int i = tid; i < kTileH * kTileW; i += kBX * kBY) {
        int ty = i / kTileW, tx = i - ty * kTileW;
        int gx = bx0 + tx, gy = by0 + ty;
        tile[ty][tx] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? (float)src[(size_t)gy * W + gx] : 0.f;
    }
    if (tid < (2 * kBR + 1) * (2 * kBR + 1)) {
        const int dy = tid / (2 * kBR + 1) - kBR, dx = tid % (2 * kBR + 1) - kBR;
        s_space[dy + kBR][dx + kBR] = (float)(dx * dx + dy * dy) * inv_half_ss;
    }
    __syncthreads();
    const int col = blockIdx.x * kBX + threadIdx.x, row = blockIdx.y * kBY + threadIdx.y;
    if (col >= W || row >= H) return;
    const float value = tile[threadIdx.y + kBR][threadIdx.x + kBR];
    const int max_x = min(col + kBR + 1, W - 1), max_y = min(row + kBR + 1, H - 1);
    const int min_x = max(col - kBR, 0), min_y = max(row - kBR, 0);
    float sum1 = 0.f, sum2 = 0.f;
    for (int cy = min_y; cy < max_y; ++cy) {
        const float *trow = &tile[cy - by0][0];
        const float *srow = &s_space[cy - row + kBR][0];
        for (int cx = min_x; cx < max_x; ++cx) {
            const float tmp = trow[cx - bx0];
            // |value - tmp| <= 65535: the square is exact in float up to 2^24,
            // beyond which the weight underflows to 0 either way
            const float d = value - tmp;
            const float w = __expf(-(srow[cx - col + kBR] + (d * d) * inv_half_sc));
            sum1 = fmaf(tmp, w, sum1);
            sum2 += w;
        }
    }
    int result = __float2int_rn(sum1 / sum2);
    int res = max(0, min(result, TDE_MAX_DEPTH_VALUE));
    if ((uint32_t)res > max_mm) res = 0;
    const size_t o = (size_t)row * W + col;
    dst[o] = (uint16_t)res;
    if (vmap) {
        const float qnan = __int_as_float(0x7fffffff);
        float z = (float)res / 1000.f;
        float vx = qnan, vy = qnan, vz = qnan;
        if (res != 0) { vx = z * (((float)col - cx) / fx); vy = z * (((float)row - cy) / fy); vz = z; }
        vmap[3 * o] = vx; vmap[3 * o + 1] = vy; vmap[3 * o + 2] = vz;
    }
}

// Depth pyramid level (restated; the reference kernel compute_depth_pyramid is
// absent): mean of the non-zero pixels of the 5x5 window around (2x, 2y) that
// differ from the centre by less than 3 sigma_color mm, rounded half up; 0
// when the centre is 0.  Optionally writes the level's vertex map.
__global__ void pyramid_kernel(const uint16_t *__restrict__ src, uint16_t *__restrict__ dst, int sW, int sH,
                               int thresh_mm, float *__restrict__ vmap, float fx, float fy, float cx, float cy) {
    const int dW = sW >> 1, dH = sH >> 1;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dW || y >= dH) return;
    const int center = src[(size_t)(2 * y) * sW + 2 * x];
    int out = 0;
    if (center != 0) {
        int sum = 0, cnt = 0;
        const int y0 = max(0, 2 * y - 2), y1 = min(sH, 2 * y + 3);
        const int x0 = max(0, 2 * x - 2), x1 = min(sW, 2 * x + 3);
        for (int cy = y0; cy < y1; ++cy)
            for (int cx2 = x0; cx2 < x1; ++cx2) {
                int v = src[(size_t)cy * sW + cx2];
                if (v != 0 && abs(v - center) < thresh_mm) { sum += v; ++cnt; }
            }
        out = (sum + cnt / 2) / cnt;  // cnt >= 1: the centre always qualifies
    }
    const size_t o = (size_t)y * dW + x;
    dst[o] = (uint16_t)out;
    if (vmap) {
        const float qnan = __int_as_float(0x7fffffff);
        float z = (float)out / 1000.f;
        float vx = qnan, vy = qnan, vz = qnan;
        if (out != 0) { vx = z * (((float)x - cx) / fx); vy = z * (((float)y - cy) / fy); vz = z; }
        vmap[3 * o] = vx; vmap[3 * o + 1] = vy; vmap[3 * o + 2] = vz;
    }
}

// scale_depth (absent from the reference; called at opencl_wrappers.cpp:37-43).
__global__ void scale_depth_kernel(const uint16_t *__restrict__ depth, float *__restrict__ scaled,
                                   const tde_intrinsics intr) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= intr.cols || y >= intr.rows) return;
    const size_t o = (size_t)y * intr.cols + x;
    float xl = ((float)x - intr.cx) / intr.fx;
    float yl = ((float)y - intr.cy) / intr.fy;
    float lambda = sqrtf(xl * xl + yl * yl + 1.f);
    scaled[o] = (float)depth[o] * lambda / 1000.f;
}

// compute_vertex_map (absent): back-projection with the level intrinsics.
__global__ void vertex_map_kernel(const uint16_t *__restrict__ depth, float *__restrict__ vmap,
                                  const tde_intrinsics intr) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= intr.cols || y >= intr.rows) return;
    const size_t o = (size_t)y * intr.cols + x;
    const float qnan = __int_as_float(0x7fffffff);
    int d = depth[o];
    float z = (float)d / 1000.f;
    float vx = qnan, vy = qnan, vz = qnan;
    if (d != 0) { vx = z * (((float)x - intr.cx) / intr.fx); vy = z * (((float)y - intr.cy) / intr.fy); vz = z; }
    vmap[3 * o] = vx; vmap[3 * o + 1] = vy; vmap[3 * o + 2] = vz;
}

// ---------------------------------------------------------------------------
// PCA normals.  The 7x7 window's vertices are staged in shared memory; each
// thread forms the window's covariance and takes the eigenvector of its
// smallest eigenvalue (closed-form eigenvalues, Smith 1961; eigenvector from
// the largest cross product of two rows of C - l I).
// ---------------------------------------------------------------------------
constexpr int kNR = 3;  // 7x7 window
constexpr int kNMin = 24;
constexpr int kNTW = kBX + 2 * kNR, kNTH = kBY + 2 * kNR;

__device__ __forceinline__ void smallest_eigvec(float c00, float c01, float c02, float c11, float c12,
                                                float c22, float &nx, float &ny, float &nz) {
    float scale = fmaxf(fmaxf(fmaxf(fabsf(c00), fabsf(c01)), fmaxf(fabsf(c02), fabsf(c11))),
                        fmaxf(fabsf(c12), fabsf(c22)));
    if (!(scale > 0.f)) { nx = ny = nz = __int_as_float(0x7fffffff); return; }
    float is = 1.f / scale;
    c00 *= is; c01 *= is; c02 *= is; c11 *= is; c12 *= is; c22 *= is;
    float q = (c00 + c11 + c22) * (1.f / 3.f);
    float p1 = c01 * c01 + c02 * c02 + c12 * c12;
    float a = c00 - q, b = c11 - q, c = c22 - q;
    float p2 = a * a + b * b + c * c + 2.f * p1;
    float p = sqrtf(p2 * (1.f / 6.f));
    float lmin;
    if (p < 1e-12f) {
        lmin = q;
    } else {
        float ip = 1.f / p;
        float b00 = a * ip, b11 = b * ip, b22 = c * ip, b01 = c01 * ip, b02 = c02 * ip, b12 = c12 * ip;
        float det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
        float r = fminf(1.f, fmaxf(-1.f, 0.5f * det));
        float phi = acosf(r) * (1.f / 3.f);
        lmin = q + 2.f * p * cosf(phi + 2.0943951023931953f);
    }
    float m00 = c00 - lmin, m11 = c11 - lmin, m22 = c22 - lmin;
    // rows r0 = (m00, c01, c02), r1 = (c01, m11, c12), r2 = (c02, c12, m22)
    float ax = c01 * c12 - c02 * m11, ay = c02 * c01 - m00 * c12, az = m00 * m11 - c01 * c01;  // r0 x r1
    float bx = c01 * m22 - c02 * c12, by = c02 * c02 - m00 * m22, bz = m00 * c12 - c01 * c02;  // r0 x r2
    float cx = m11 * m22 - c12 * c12, cy = c12 * c02 - c01 * m22, cz = c01 * c12 - m11 * c02;  // r1 x r2
    float da = ax * ax + ay * ay + az * az, db = bx * bx + by * by + bz * bz, dc = cx * cx + cy * cy + cz * cz;
    float ex = ax, ey = ay, ez = az, dm = da;
    if (db > dm) { ex = bx; ey = by; ez = bz; dm = db; }
    if (dc > dm) { ex = cx; ey = cy; ez = cz; dm = dc; }
    if (!(dm > 0.f)) { nx = ny = nz = __int_as_float(0x7fffffff); return; }
    float inv = rsqrtf(dm);
    nx = ex * inv; ny = ey * inv; nz = ez * inv;
}

__global__ void __launch_bounds__(kBX *kBY) normal_map_kernel(const float *__restrict__ vmap,
                                                              float *__restrict__ nmap, int W, int H) {
    __shared__ float sx[kNTH][kNTW + 1], sy[kNTH][kNTW + 1], sz[kNTH][kNTW + 1];
    const int bx0 = blockIdx.x * kBX - kNR, by0 = blockIdx.y * kBY - kNR;
    const int tid = threadIdx.y * kBX + threadIdx.x;
    const float qnan = __int_as_float(0x7fffffff);
    for (int i = tid; i < kNTH * kNTW; i += kBX * kBY) {
        int ty = i / kNTW, tx = i - ty * kNTW;
        int gx = bx0 + tx, gy = by0 + ty;
        float a = qnan, b = qnan, c = qnan;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            size_t o = 3 * ((size_t)gy * W + gx);
            a = vmap[o]; b = vmap[o + 1]; c = vmap[o + 2];
        }
        sx[ty][tx] = a; sy[ty][tx] = b; sz[ty][tx] = c;
    }
    __syncthreads();
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y;
    if (x >= W || y >= H) return;
    const int lx = threadIdx.x + kNR, ly = threadIdx.y + kNR;
    float nx = qnan, ny = qnan, nz = qnan;
    const float px = sx[ly][lx], py = sy[ly][lx], pz = sz[ly][lx];
    if (!isnan(px)) {
        // one pass over the window: first and second moments of the offsets
        // from the centre vertex (a window of a smooth surface is centred on
        // it, so the moments carry no large common part to cancel), then
        // C = S2 - S1 S1^T / n
        float s1x = 0.f, s1y = 0.f, s1z = 0.f;
        float c00 = 0.f, c01 = 0.f, c02 = 0.f, c11 = 0.f, c12 = 0.f, c22 = 0.f;
        int cnt = 0;
        #pragma unroll
        for (int dy = -kNR; dy <= kNR; ++dy)
            #pragma unroll
            for (int dx = -kNR; dx <= kNR; ++dx) {
                const float a = sx[ly + dy][lx + dx];
                if (!isnan(a)) {
                    const float ux = a - px, uy = sy[ly + dy][lx + dx] - py, uz = sz[ly + dy][lx + dx] - pz;
                    s1x += ux; s1y += uy; s1z += uz;
                    c00 = fmaf(ux, ux, c00); c01 = fmaf(ux, uy, c01); c02 = fmaf(ux, uz, c02);
                    c11 = fmaf(uy, uy, c11); c12 = fmaf(uy, uz, c12); c22 = fmaf(uz, uz, c22);
                    ++cnt;
                }
            }
        if (cnt >= kNMin) {
            const float ic = 1.f / (float)cnt;
            const float mx = s1x * ic, my = s1y * ic, mz = s1z * ic;
            c00 = fmaf(-mx, s1x, c00); c01 = fmaf(-mx, s1y, c01); c02 = fmaf(-mx, s1z, c02);
            c11 = fmaf(-my, s1y, c11); c12 = fmaf(-my, s1z, c12); c22 = fmaf(-mz, s1z, c22);
            smallest_eigvec(c00, c01, c02, c11, c12, c22, nx, ny, nz);
            if (nx * px + ny * py + nz * pz > 0.f) { nx = -nx; ny = -ny; nz = -nz; }
        }
    }
    size_t o = 3 * ((size_t)y * W + x);
    nmap[o] = nx; nmap[o + 1] = ny; nmap[o + 2] = nz;
}

}  // namespace

int launch_bilateral(const uint16_t *src, uint16_t *dst, int W, int H, float ss, float sc, uint32_t max_mm,
                     float *vmap, const tde_intrinsics *intr, cudaStream_t stream) {
    dim3 block(kBX, kBY), grid(div_up(W, kBX), div_up(H, kBY));
    float inv_ss = 0.5f / (ss * ss), inv_sc = 0.5f / (sc * sc);
    float fx = intr ? intr->fx : 1.f, fy = intr ? intr->fy : 1.f, cx = intr ? intr->cx : 0.f, cy = intr ? intr->cy : 0.f;
    bilateral_kernel<<<grid, block, 0, stream>>>(src, dst, W, H, inv_ss, inv_sc, max_mm, vmap, fx, fy, cx, cy);
    return check_launch("bilateral");
}

int launch_pyramid(const uint16_t *src, uint16_t *dst, int sW, int sH, float sigma_color, float *vmap,
                   const tde_intrinsics *intr_dst, cudaStream_t stream) {
    dim3 block(32, 8), grid(div_up(sW >> 1, 32), div_up(sH >> 1, 8));
    int thresh = (int)(3.f * sigma_color);
    float fx = intr_dst ? intr_dst->fx : 1.f, fy = intr_dst ? intr_dst->fy : 1.f;
    float cx = intr_dst ? intr_dst->cx : 0.f, cy = intr_dst ? intr_dst->cy : 0.f;
    pyramid_kernel<<<grid, block, 0, stream>>>(src, dst, sW, sH, thresh, vmap, fx, fy, cx, cy);
    return check_launch("depth_pyramid");
}

int launch_scale_depth(const uint16_t *depth, float *scaled, const tde_intrinsics &intr, cudaStream_t stream) {
    dim3 block(32, 8), grid(div_up(intr.cols, 32), div_up(intr.rows, 8));
    scale_depth_kernel<<<grid, block, 0, stream>>>(depth, scaled, intr);
    return check_launch("scale_depth");
}

int launch_vertex_map(const uint16_t *depth, float *vmap, const tde_intrinsics &intr, cudaStream_t stream) {
    dim3 block(32, 8), grid(div_up(intr.cols, 32), div_up(intr.rows, 8));
    vertex_map_kernel<<<grid, block, 0, stream>>>(depth, vmap, intr);
    return check_launch("vertex_map");
}

int launch_normal_map(const float *vmap, float *nmap, int W, int H, cudaStream_t stream) {
    dim3 block(kBX, kBY), grid(div_up(W, kBX), div_up(H, kBY));
    normal_map_kernel<<<grid, block, 0, stream>>>(vmap, nmap, W, H);
    return check_launch("normal_map");
}

}  // namespace tde
