// k_raycast.cu -- model prediction: TSDF ray march (raycast), model-map
// pyramid (resize) and rigid map transform.
//
// Built with -fmad=false: every float expression below is evaluated as the
// same sequence of IEEE-rounded multiplies and adds the reference kernel
// (GPU/opencl/raycast.cl) performs, so vertex/normal maps match the
// reference bit for bit on the same volume.
#include "tde_common.cuh"
#include "tde_launch.cuh"
#include "tde_integrate.cuh"

namespace tde {
namespace {

struct RayParams {
    tde_point3f t;          // ray origin (camera centre, volume frame)
    tde_matrix3f R;         // camera -> volume rotation
    float time_step;        // (float)((double)trunc * 0.8), raycast.cl:209
    float max_time;         // 3 * (Vx + Vy + Vz), raycast.cl:251
    tde_intrinsics intr;
    tde_round_buffer rb;
    tde_point3f cell;
    size_t n;               // voxel count (F32 plane offset)
    const CamPose *dpose;   // when set, t and R are read from here
    const uint8_t *neg_flags;  // per physical 8^3 brick: 0 = holds no negative value
    const uint8_t *super_flags;  // per physical 32^3 super-brick (null: no sample skipping)
    float inv_cell[3];
    float skip_margin;           // time margin kept from a super-brick's exit
};

struct f3 { float x, y, z; };

__device__ __forceinline__ f3 mat_vec(const tde_matrix3f &M, f3 v) {
    // multiply() in elementary_matrix_template.h:30-39: dot starting from 0.
    f3 r;
    float a = 0.f; a += M.row[0].x * v.x; a += M.row[0].y * v.y; a += M.row[0].z * v.z; r.x = a;
    float b = 0.f; b += M.row[1].x * v.x; b += M.row[1].y * v.y; b += M.row[1].z * v.z; r.y = b;
    float c = 0.f; c += M.row[2].x * v.x; c += M.row[2].y * v.y; c += M.row[2].z * v.z; r.z = c;
    return r;
}

__device__ __forceinline__ f3 normalized(f3 v) {
    float d = 0.f; d += v.x * v.x; d += v.y * v.y; d += v.z * v.z;
    float rs = 1.f / sqrtf(d);
    return f3{v.x * rs, v.y * rs, v.z * rs};
}

// ray_start + ray_dir * t, component-wise (add_3f after the scale).
__device__ __forceinline__ f3 along(const tde_point3f &o, f3 d, float t) {
    return f3{o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
}

__device__ __forceinline__ int floor_sat(float v) { return __float2int_rd(v); }  // convert_int_sat_rtn

// floor(v / c) with the IEEE quotient's result: v * (1/c) is within 2.5 ulp of
// v / c, so away from integer boundaries (and for |q| < 2048, where an ulp is
// below 2.5e-4) both floors agree; near a boundary the division is done.
__device__ __forceinline__ int floor_div(float v, float c, float inv_c) {
    const float q = v * inv_c;
    const float fr = q - floorf(q);
    if (fabsf(q) < 2048.f && fr > 2e-3f && fr < 1.f - 2e-3f) return __float2int_rd(q);
    return floor_sat(v / c);
}

template <int FMT>
__device__ __forceinline__ float read_tsdf(const void *vol, const RayParams &p, int x, int y, int z) {
    return TsdfStore<FMT>::value(vol, voxel_address(x, y, z, p.rb), p.n);
}

// interpolateTrilineary: raycast.cl:95-145.
template <int FMT>
__device__ __noinline__ float trilinear(const void *vol, const RayParams &p, f3 pt) {
    const tde_point3i &N = p.rb.voxels_size;
    int gx = floor_sat(pt.x / p.cell.x), gy = floor_sat(pt.y / p.cell.y), gz = floor_sat(pt.z / p.cell.z);
    if (gx <= 0 || gx >= N.x - 1) return __int_as_float(0x7fffffff);
    if (gy <= 0 || gy >= N.y - 1) return __int_as_float(0x7fffffff);
    if (gz <= 0 || gz >= N.z - 1) return __int_as_float(0x7fffffff);
    float vx = ((float)gx + 0.5f) * p.cell.x;
    float vy = ((float)gy + 0.5f) * p.cell.y;
    float vz = ((float)gz + 0.5f) * p.cell.z;
    gx = (pt.x < vx) ? gx - 1 : gx;
    gy = (pt.y < vy) ? gy - 1 : gy;
    gz = (pt.z < vz) ? gz - 1 : gz;
    float a = pt.x / p.cell.x - ((float)gx + 0.5f); if (a < 0) { gx--; a += 1.0f; }
    float b = pt.y / p.cell.y - ((float)gy + 0.5f); if (b < 0) { gy--; b += 1.0f; }
    float c = pt.z / p.cell.z - ((float)gz + 0.5f); if (c < 0) { gz--; c += 1.0f; }
    float r000 = read_tsdf<FMT>(vol, p, gx, gy, gz), r001 = read_tsdf<FMT>(vol, p, gx, gy, gz + 1);
    float r010 = read_tsdf<FMT>(vol, p, gx, gy + 1, gz), r011 = read_tsdf<FMT>(vol, p, gx, gy + 1, gz + 1);
    float r100 = read_tsdf<FMT>(vol, p, gx + 1, gy, gz), r101 = read_tsdf<FMT>(vol, p, gx + 1, gy, gz + 1);
    float r110 = read_tsdf<FMT>(vol, p, gx + 1, gy + 1, gz), r111 = read_tsdf<FMT>(vol, p, gx + 1, gy + 1, gz + 1);
    float one_a = 1.f - a, one_b = 1.f - b, one_c = 1.f - c;
    float x0 = one_b * (r000 * one_c + r001 * c) + b * (r010 * one_c + r011 * c);
    float x1 = one_b * (r100 * one_c + r101 * c) + b * (r110 * one_c + r111 * c);
    return one_a * x0 + a * x1;
}

// Zero crossing between time_curr and time_curr + step: secant refinement of
// the hit and central-difference normal (raycast.cl:280-401).  Kept out of
// line: it runs once per ray, and inlining it would bloat the march loop past
// the instruction cache.
template <int FMT>
__device__ __noinline__ void refine_surface(const void *vol, const RayParams &p, f3 dir, float time_curr,
                                            float &vx_out, float &vy_out, float &vz_out, float &nx_out,
                                            float &ny_out, float &nz_out) {
    const tde_point3i N = p.rb.voxels_size;
    const float step = p.time_step;
    float ct = time_curr + step;
    float Ftdt = trilinear<FMT>(vol, p, along(p.t, dir, ct));
    if (isnan(Ftdt)) return;
    float Ft = trilinear<FMT>(vol, p, along(p.t, dir, time_curr));
    if (isnan(Ft)) return;
    float Ts = time_curr - step * Ft / (Ftdt - Ft);
    f3 vf = along(p.t, dir, Ts);
    vx_out = vf.x; vy_out = vf.y; vz_out = vf.z;
    f3 p3 = along(p.t, dir, time_curr);
    int hx = floor_sat(p3.x / p.cell.x), hy = floor_sat(p3.y / p.cell.y), hz = floor_sat(p3.z / p.cell.z);
    if (hx > 1 && hy > 1 && hz > 1 && hx < N.x - 2 && hy < N.y - 2 && hz < N.z - 2) {
        float F[6];
        #pragma unroll 1
        for (int k = 0; k < 6; ++k) {
            f3 tt = vf;
            const int axis = k >> 1;
            const float d = axis == 0 ? p.cell.x : axis == 1 ? p.cell.y : p.cell.z;
            float &c = axis == 0 ? tt.x : axis == 1 ? tt.y : tt.z;
            c = (k & 1) ? c - d : c + d;
            F[k] = trilinear<FMT>(vol, p, tt);
        }
        f3 n = normalized(f3{F[0] - F[1], F[2] - F[3], F[4] - F[5]});
        nx_out = n.x; ny_out = n.y; nz_out = n.z;
    }
}

// Number of march samples whose addresses are issued together.  The samples
// are independent of each other's values, so their loads overlap; the
// zero-crossing logic then consumes them in order exactly as a one-sample
// loop would.
constexpr int kBatch = 4;

template <int FMT, bool SKIP>
__global__ void __launch_bounds__(256) raycast_kernel(const void *__restrict__ vol, float *__restrict__ vmap,
                                                     float *__restrict__ nmap, RayParams p) {
    // 16x16 pixels per block; each warp takes an 8x4 tile so its rays start
    // close together and sample neighbouring voxels.
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
    const int W = p.intr.cols, H = p.intr.rows;
    if (p.dpose) {
        __shared__ float s_pose[12];
        if (tid < 12) s_pose[tid] = tid < 9 ? p.dpose->R[tid] : p.dpose->t[tid - 9];
        __syncthreads();
        p.R = tde_matrix3f{{{s_pose[0], s_pose[1], s_pose[2]}, {s_pose[3], s_pose[4], s_pose[5]},
                            {s_pose[6], s_pose[7], s_pose[8]}}};
        p.t = tde_point3f{s_pose[9], s_pose[10], s_pose[11]};
    }
    if (x >= W || y >= H) return;
    const size_t pix = (size_t)W * y + x;
    const float qnan = __int_as_float(0x7fffffff);
    float vx_out = qnan, vy_out = qnan, vz_out = qnan;
    float nx_out = qnan, ny_out = qnan, nz_out = qnan;

    const tde_point3i N = p.rb.voxels_size;
    const tde_point3f V = p.rb.volume_size;
    const float step = p.time_step;
    const int nbx = (N.x + 7) >> 3, nby = (N.y + 7) >> 3;

    f3 rnu{((float)x - p.intr.cx) / p.intr.fx, ((float)y - p.intr.cy) / p.intr.fy, 1.f};
    f3 rn2 = mat_vec(p.R, rnu);
    f3 ray_next{rn2.x + p.t.x, rn2.y + p.t.y, rn2.z + p.t.z};
    f3 dir = normalized(f3{ray_next.x - p.t.x, ray_next.y - p.t.y, ray_next.z - p.t.z});
    dir.x = (dir.x == 0.f) ? 1e-15f : dir.x;
    dir.y = (dir.y == 0.f) ? 1e-15f : dir.y;
    dir.z = (dir.z == 0.f) ? 1e-15f : dir.z;

    // getMinTime / getMaxTime: raycast.cl:153-171
    float txmin = ((dir.x > 0 ? 0.f : V.x) - p.t.x) / dir.x;
    float tymin = ((dir.y > 0 ? 0.f : V.y) - p.t.y) / dir.y;
    float tzmin = ((dir.z > 0 ? 0.f : V.z) - p.t.z) / dir.z;
    float t_start = cl_fmax(cl_fmax(txmin, tymin), tzmin);
    float txmax = ((dir.x > 0 ? V.x : 0.f) - p.t.x) / dir.x;
    float tymax = ((dir.y > 0 ? V.y : 0.f) - p.t.y) / dir.y;
    float tzmax = ((dir.z > 0 ? V.z : 0.f) - p.t.z) / dir.z;
    float t_exit = cl_fmin(cl_fmin(txmax, tymax), tzmax);
    t_start = cl_fmax(t_start, 0.f);

    if (!(t_start >= t_exit)) {
        float time_curr = t_start;
        f3 pu = along(p.t, dir, time_curr);
        int gx = floor_sat(pu.x / p.cell.x), gy = floor_sat(pu.y / p.cell.y), gz = floor_sat(pu.z / p.cell.z);
        gx = max(0, min(gx, N.x - 1));
        gy = max(0, min(gy, N.y - 1));
        gz = max(0, min(gz, N.z - 1));
        // prev sample: its value when `known`, else only "non-negative"; its
        // sample time lets the value be fetched when it is needed after all
        float tsdf = read_tsdf<FMT>(vol, p, gx, gy, gz);
        bool known = true;
        float prev_ct = time_curr;
        const int nsx = (N.x + 31) >> 5, nsy = (N.y + 31) >> 5;

        bool done = false;
        while (!done && time_curr < p.max_time) {
            if (SKIP && p.super_flags && !(known && tsdf < 0.f)) {
                // Inside a 32^3 super-brick with no negative value and after a
                // non-negative sample, no test of the loop can fire: advance
                // time_curr by the same additions without evaluating samples,
                // stopping while the next sample is still clear of the exit.
                for (;;) {
                    if (!(time_curr < p.max_time)) break;
                    const float ct = time_curr + step;
                    const f3 q = along(p.t, dir, ct);
                    const int sx = floor_div(q.x, p.cell.x, p.inv_cell[0]);
                    const int sy = floor_div(q.y, p.cell.y, p.inv_cell[1]);
                    const int sz = floor_div(q.z, p.cell.z, p.inv_cell[2]);
                    if (!(sx >= 0 && sy >= 0 && sz >= 0 && sx < N.x && sy < N.y && sz < N.z)) break;
                    const int px = wrap_mod(sx + p.rb.origin_GRID.x, N.x);
                    const int py = wrap_mod(sy + p.rb.origin_GRID.y, N.y);
                    const int pz = wrap_mod(sz + p.rb.origin_GRID.z, N.z);
                    if (__ldg(p.super_flags + ((px >> 5) + nsx * ((py >> 5) + nsy * (pz >> 5))))) break;
                    // logical voxel box of this super-brick, in metres
                    const float lox = (float)(sx - (px & 31)) * p.cell.x, loy = (float)(sy - (py & 31)) * p.cell.y,
                                loz = (float)(sz - (pz & 31)) * p.cell.z;
                    const float hix = lox + 32.f * p.cell.x, hiy = loy + 32.f * p.cell.y, hiz = loz + 32.f * p.cell.z;
                    const float ex = ((dir.x > 0.f ? hix : lox) - p.t.x) / dir.x;
                    const float ey = ((dir.y > 0.f ? hiy : loy) - p.t.y) / dir.y;
                    const float ez = ((dir.z > 0.f ? hiz : loz) - p.t.z) / dir.z;
                    const float lim = fminf(fminf(ex, ey), ez) - p.skip_margin;
                    float tn = time_curr;
                    int m = 0;
                    while (tn < p.max_time && tn + step < lim) { tn = tn + step; ++m; }
                    if (m == 0) break;  // next sample near the exit: evaluate it normally
                    time_curr = tn;
                    known = false;
                    prev_ct = tn;
                }
                if (!(time_curr < p.max_time)) break;
            }
            float ts[kBatch];
            float vals[kBatch];
            size_t addr[kBatch];
            bool have[kBatch];
            int nvalid = 0;  // samples in range, in order; the first out-of-range one ends the ray
            {
                float tc = time_curr;
                #pragma unroll
                for (int k = 0; k < kBatch; ++k) {
                    ts[k] = tc;
                    vals[k] = 0.f;
                    have[k] = false;
                    addr[k] = 0;
                    tc = tc + step;
                }
            }
            bool stop_after = false;
            #pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                if (nvalid == k && !stop_after) {
                    if (!(ts[k] < p.max_time)) { stop_after = true; }
                    else {
                        const float ct = ts[k] + step;
                        const f3 q = along(p.t, dir, ct);
                        const int sx = floor_div(q.x, p.cell.x, p.inv_cell[0]);
                        const int sy = floor_div(q.y, p.cell.y, p.inv_cell[1]);
                        const int sz = floor_div(q.z, p.cell.z, p.inv_cell[2]);
                        if (sx >= 0 && sy >= 0 && sz >= 0 && sx < N.x && sy < N.y && sz < N.z) {
                            const int px = wrap_mod(sx + p.rb.origin_GRID.x, N.x);
                            const int py = wrap_mod(sy + p.rb.origin_GRID.y, N.y);
                            const int pz = wrap_mod(sz + p.rb.origin_GRID.z, N.z);
                            addr[k] = (size_t)px + (size_t)N.x * ((size_t)py + (size_t)N.y * (size_t)pz);
                            bool load = true;
                            if (SKIP)
                                load = __ldg(p.neg_flags + ((px >> 3) + nbx * ((py >> 3) + nby * (pz >> 3)))) != 0;
                            if (load) {
                                vals[k] = TsdfStore<FMT>::value(vol, addr[k], p.n);
                                have[k] = true;
                            }
                            nvalid = k + 1;
                        } else {
                            stop_after = true;
                        }
                    }
                }
            }
            // Consume the samples in order (raycast.cl:254-404).
            #pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                if (done) break;
                if (k >= nvalid) { done = true; break; }  // out of volume or out of time
                time_curr = ts[k];
                if (SKIP && !have[k]) {
                    if (!(known && tsdf < 0.f)) {
                        // a non-negative sample after a non-negative one: no test can fire
                        known = false;
                        prev_ct = ts[k] + step;
                        continue;
                    }
                    vals[k] = TsdfStore<FMT>::value(vol, addr[k], p.n);  // leaving a negative run
                }
                const float cur = vals[k];
                if (SKIP && !known) {
                    if (!(cur < 0.f)) {  // prev >= 0 and cur >= 0
                        tsdf = cur;
                        known = true;
                        prev_ct = ts[k] + step;
                        continue;
                    }
                    // the previous sample's sign decides a crossing: fetch it
                    const f3 q = along(p.t, dir, prev_ct);
                    tsdf = read_tsdf<FMT>(vol, p, floor_div(q.x, p.cell.x, p.inv_cell[0]),
                                          floor_div(q.y, p.cell.y, p.inv_cell[1]),
                                          floor_div(q.z, p.cell.z, p.inv_cell[2]));
                }
                const float tsdf_prev = tsdf;
                tsdf = cur;
                known = true;
                prev_ct = ts[k] + step;
                if (tsdf_prev < 0.f && tsdf > 0.f) { done = true; break; }
                if (tsdf_prev > 0.f && tsdf < 0.f) {
                    done = true;
                    refine_surface<FMT>(vol, p, dir, time_curr, vx_out, vy_out, vz_out, nx_out, ny_out, nz_out);
                    break;
                }
            }
            if (!done) {
                // every sample of the batch was consumed without a decision
                time_curr = ts[kBatch - 1] + step;
            }
        }
    }
    vmap[3 * pix + 0] = vx_out; vmap[3 * pix + 1] = vy_out; vmap[3 * pix + 2] = vz_out;
    nmap[3 * pix + 0] = nx_out; nmap[3 * pix + 1] = ny_out; nmap[3 * pix + 2] = nz_out;
}

// resize_vertex_map / resize_normal_map (absent from the reference; named at
// common/inc/constants.h:175-176): 2x2 block mean, all four valid.
template <bool NORMAL>
__global__ void resize_map_kernel(const float *__restrict__ src, float *__restrict__ dst, int sc, int sr) {
    const int dc = sc >> 1, dr = sr >> 1;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dc || y >= dr) return;
    const float qnan = __int_as_float(0x7fffffff);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    bool ok = true;
    #pragma unroll
    for (int dy = 0; dy < 2; ++dy)
        #pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
            size_t i = 3 * ((size_t)(2 * y + dy) * sc + (2 * x + dx));
            float a = src[i], b = src[i + 1], c = src[i + 2];
            ok = ok && !isnan(a);
            sx = sx + a; sy = sy + b; sz = sz + c;
        }
    float ox = qnan, oy = qnan, oz = qnan;
    if (ok) {
        if (NORMAL) {
            float d = 0.f; d += sx * sx; d += sy * sy; d += sz * sz;
            float rs = 1.f / sqrtf(d);
            ox = sx * rs; oy = sy * rs; oz = sz * rs;
        } else {
            ox = sx * 0.25f; oy = sy * 0.25f; oz = sz * 0.25f;
        }
    }
    size_t o = 3 * ((size_t)y * dc + x);
    dst[o] = ox; dst[o + 1] = oy; dst[o + 2] = oz;
}

// transform_map.cl:6-65
__global__ void transform_maps_kernel(const float *__restrict__ vs, const float *__restrict__ ns, float *vd,
                                      float *nd, const tde_matrix3f R, const tde_point3f t, int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float qnan = __int_as_float(0x7fffffff);
    size_t i = 3 * ((size_t)y * W + x);
    f3 v{vs[i], vs[i + 1], vs[i + 2]};
    f3 vo{qnan, qnan, qnan};
    if (!isnan(v.x)) {
        f3 r = mat_vec(R, v);
        vo = f3{r.x + t.x, r.y + t.y, r.z + t.z};
    }
    f3 n{ns[i], ns[i + 1], ns[i + 2]};
    f3 no{qnan, qnan, qnan};
    if (!isnan(n.x)) no = mat_vec(R, n);
    vd[i] = vo.x; vd[i + 1] = vo.y; vd[i + 2] = vo.z;
    nd[i] = no.x; nd[i + 1] = no.y; nd[i + 2] = no.z;
}

}  // namespace

int launch_raycast(const void *volume, int format, float *vmap, float *nmap, const tde_point3f &t,
                   const tde_matrix3f &R, float trunc, const tde_intrinsics &intr, const tde_round_buffer &rb,
                   const tde_point3f &cell, const CamPose *dpose, const uint8_t *neg_flags, cudaStream_t stream) {
    RayParams p;
    p.dpose = dpose;
    p.neg_flags = neg_flags;
    p.t = t; p.R = R;
    p.time_step = (float)((double)trunc * 0.8);
    p.max_time = 3.f * ((rb.volume_size.x + rb.volume_size.y) + rb.volume_size.z);
    p.intr = intr; p.rb = rb; p.cell = cell; p.n = voxel_count(rb);
    p.inv_cell[0] = 1.f / cell.x; p.inv_cell[1] = 1.f / cell.y; p.inv_cell[2] = 1.f / cell.z;
    // super-brick sample skipping needs whole 32^3 super-bricks on every axis
    const bool whole = rb.voxels_size.x % 32 == 0 && rb.voxels_size.y % 32 == 0 && rb.voxels_size.z % 32 == 0;
    p.super_flags = (neg_flags && whole) ? neg_flags + brick_count(rb) : nullptr;
    p.skip_margin = 1e-2f * fminf(fminf(cell.x, cell.y), cell.z);
    dim3 block(256);
    dim3 grid(div_up(intr.cols, 16), div_up(intr.rows, 16));
    return dispatch_format(format, [&](auto F) {
        if (neg_flags) raycast_kernel<decltype(F)::value, true><<<grid, block, 0, stream>>>(volume, vmap, nmap, p);
        else raycast_kernel<decltype(F)::value, false><<<grid, block, 0, stream>>>(volume, vmap, nmap, p);
        return check_launch("raycast");
    });
}

int launch_resize_map(const float *src, float *dst, int sc, int sr, bool normal, cudaStream_t stream) {
    dim3 block(32, 8);
    dim3 grid(div_up(sc >> 1, 32), div_up(sr >> 1, 8));
    if (normal) resize_map_kernel<true><<<grid, block, 0, stream>>>(src, dst, sc, sr);
    else resize_map_kernel<false><<<grid, block, 0, stream>>>(src, dst, sc, sr);
    return check_launch("resize_map");
}

int launch_transform_maps(const float *vs, const float *ns, float *vd, float *nd, const tde_matrix3f &R,
                          const tde_point3f &t, int W, int H, cudaStream_t stream) {
    dim3 block(32, 8);
    dim3 grid(div_up(W, 32), div_up(H, 8));
    transform_maps_kernel<<<grid, block, 0, stream>>>(vs, ns, vd, nd, R, t, W, H);
    return check_launch("transform_maps");
}

}  // namespace tde
