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
    unsigned *touched;      // measurement runs: one bit per voxel record read
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
__device__ __forceinline__ f3 along(f3 o, f3 d, float t) {
    return f3{o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
}

__device__ __forceinline__ int floor_sat(float v) { return __float2int_rd(v); }  // convert_int_sat_rtn

// A voxel record's value; measurement instantiations also mark the record.
template <int FMT, bool STATS>
__device__ __forceinline__ float load_rec(const void *vol, const RayParams &p, size_t addr) {
    if (STATS) atomicOr(p.touched + (addr >> 5), 1u << (addr & 31));
    return TsdfStore<FMT>::value_ro(vol, addr, p.n);
}

template <int FMT, bool STATS>
__device__ __forceinline__ float read_tsdf(const void *vol, const RayParams &p, int x, int y, int z) {
    return load_rec<FMT, STATS>(vol, p, voxel_address(x, y, z, p.rb));
}

// interpolateTrilineary (raycast.cl:95-145), split by axis: the lower corner
// along one axis, the upper corner's weight, and both corners' physical
// indices times the axis stride.  False when the base voxel lies on the
// volume border (the interpolation is then NaN).  The six normal samples of a
// hit share two of their three axes with the refined point, so those are
// formed once.
struct Axis {
    size_t i0, i1;
    float w;
};

__device__ __forceinline__ bool tri_axis(float pt, float q, float cell, int N, int origin, size_t stride, Axis &ax) {
    int g = floor_sat(q);
    if (g <= 0 || g >= N - 1) return false;
    const float v = ((float)g + 0.5f) * cell;
    g = (pt < v) ? g - 1 : g;
    float a = q - ((float)g + 0.5f);
    if (a < 0) { g--; a += 1.0f; }
    // the two corners g, g + 1 are inside [0, N) here
    ax.i0 = (size_t)wrap_mod(g + origin, N) * stride;
    ax.i1 = (size_t)wrap_mod(g + 1 + origin, N) * stride;
    ax.w = a;
    return true;
}

template <int FMT, bool STATS>
__device__ __forceinline__ float tri_corners(const void *vol, const RayParams &p, const Axis &X, const Axis &Y,
                                             const Axis &Z) {
    const size_t r00 = Y.i0 + Z.i0, r01 = Y.i0 + Z.i1, r10 = Y.i1 + Z.i0, r11 = Y.i1 + Z.i1;
    float v000 = load_rec<FMT, STATS>(vol, p, X.i0 + r00), v001 = load_rec<FMT, STATS>(vol, p, X.i0 + r01);
    float v010 = load_rec<FMT, STATS>(vol, p, X.i0 + r10), v011 = load_rec<FMT, STATS>(vol, p, X.i0 + r11);
    float v100 = load_rec<FMT, STATS>(vol, p, X.i1 + r00), v101 = load_rec<FMT, STATS>(vol, p, X.i1 + r01);
    float v110 = load_rec<FMT, STATS>(vol, p, X.i1 + r10), v111 = load_rec<FMT, STATS>(vol, p, X.i1 + r11);
    const float a = X.w, b = Y.w, c = Z.w;
    float one_a = 1.f - a, one_b = 1.f - b, one_c = 1.f - c;
    float xa = one_b * (v000 * one_c + v001 * c) + b * (v010 * one_c + v011 * c);
    float xb = one_b * (v100 * one_c + v101 * c) + b * (v110 * one_c + v111 * c);
    return one_a * xa + a * xb;
}

__device__ __forceinline__ bool axis_x(const RayParams &p, float pt, float q, Axis &ax) {
    return tri_axis(pt, q, p.cell.x, p.rb.voxels_size.x, p.rb.origin_GRID.x, 1, ax);
}
__device__ __forceinline__ bool axis_y(const RayParams &p, float pt, float q, Axis &ax) {
    return tri_axis(pt, q, p.cell.y, p.rb.voxels_size.y, p.rb.origin_GRID.y, (size_t)p.rb.voxels_size.x, ax);
}
__device__ __forceinline__ bool axis_z(const RayParams &p, float pt, float q, Axis &ax) {
    return tri_axis(pt, q, p.cell.z, p.rb.voxels_size.z, p.rb.origin_GRID.z,
                    (size_t)p.rb.voxels_size.x * (size_t)p.rb.voxels_size.y, ax);
}

template <int FMT, bool STATS>
__device__ __forceinline__ float trilinear(const void *vol, const RayParams &p, f3 pt) {
    Axis X, Y, Z;
    if (!axis_x(p, pt.x, pt.x / p.cell.x, X) || !axis_y(p, pt.y, pt.y / p.cell.y, Y) ||
        !axis_z(p, pt.z, pt.z / p.cell.z, Z))
        return __int_as_float(0x7fffffff);
    return tri_corners<FMT, STATS>(vol, p, X, Y, Z);
}

// Zero crossing between time_curr and time_curr + step: secant refinement of
// the hit and central-difference normal (raycast.cl:280-401).  Kept out of
// line: it runs once per ray, and inlining it would bloat the march loop past
// the instruction cache.
template <int FMT, bool STATS>
__device__ __noinline__ void refine_surface(const void *vol, const RayParams &p, f3 org, f3 dir, float time_curr,
                                            float &vx_out, float &vy_out, float &vz_out, float &nx_out,
                                            float &ny_out, float &nz_out) {
    const tde_point3i N = p.rb.voxels_size;
    const float step = p.time_step;
    float ct = time_curr + step;
    float Ftdt = trilinear<FMT, STATS>(vol, p, along(org, dir, ct));
    if (isnan(Ftdt)) return;
    float Ft = trilinear<FMT, STATS>(vol, p, along(org, dir, time_curr));
    if (isnan(Ft)) return;
    float Ts = time_curr - step * Ft / (Ftdt - Ft);
    f3 vf = along(org, dir, Ts);
    vx_out = vf.x; vy_out = vf.y; vz_out = vf.z;
    f3 p3 = along(org, dir, time_curr);
    int hx = floor_sat(p3.x / p.cell.x), hy = floor_sat(p3.y / p.cell.y), hz = floor_sat(p3.z / p.cell.z);
    if (hx > 1 && hy > 1 && hz > 1 && hx < N.x - 2 && hy < N.y - 2 && hz < N.z - 2) {
        // vf +- cell on one axis: the other two axes are vf's
        const float qnan = __int_as_float(0x7fffffff);
        Axis X, Y, Z, A1, A2;
        const bool okx = axis_x(p, vf.x, vf.x / p.cell.x, X);
        const bool oky = axis_y(p, vf.y, vf.y / p.cell.y, Y);
        const bool okz = axis_z(p, vf.z, vf.z / p.cell.z, Z);
        float t1 = vf.x + p.cell.x, t2 = vf.x - p.cell.x;
        const bool x1 = axis_x(p, t1, t1 / p.cell.x, A1), x2 = axis_x(p, t2, t2 / p.cell.x, A2);
        const float Fx1 = (x1 && oky && okz) ? tri_corners<FMT, STATS>(vol, p, A1, Y, Z) : qnan;
        const float Fx2 = (x2 && oky && okz) ? tri_corners<FMT, STATS>(vol, p, A2, Y, Z) : qnan;
        t1 = vf.y + p.cell.y; t2 = vf.y - p.cell.y;
        const bool y1 = axis_y(p, t1, t1 / p.cell.y, A1), y2 = axis_y(p, t2, t2 / p.cell.y, A2);
        const float Fy1 = (okx && y1 && okz) ? tri_corners<FMT, STATS>(vol, p, X, A1, Z) : qnan;
        const float Fy2 = (okx && y2 && okz) ? tri_corners<FMT, STATS>(vol, p, X, A2, Z) : qnan;
        t1 = vf.z + p.cell.z; t2 = vf.z - p.cell.z;
        const bool z1 = axis_z(p, t1, t1 / p.cell.z, A1), z2 = axis_z(p, t2, t2 / p.cell.z, A2);
        const float Fz1 = (okx && oky && z1) ? tri_corners<FMT, STATS>(vol, p, X, Y, A1) : qnan;
        const float Fz2 = (okx && oky && z2) ? tri_corners<FMT, STATS>(vol, p, X, Y, A2) : qnan;
        f3 n = normalized(f3{Fx1 - Fx2, Fy1 - Fy2, Fz1 - Fz2});
        nx_out = n.x; ny_out = n.y; nz_out = n.z;
    }
}

// Voxel of the sample at time ct: floor(pos / cell) with pos = t + dir * ct
// evaluated exactly as the reference does whenever it matters.  The fast
// estimate o/c + (d/c) ct is within ~4e-4 voxel of the exact quotient, so a
// fractional part clear of 4e-3 from an integer settles the floor; otherwise
// the position and the IEEE quotient are computed.
constexpr float kSkipMargin = 1e-2f;  // voxels

struct RayFast {
    float o[3], d[3];  // t / cell, dir / cell
    float inv_d[3];    // 1 / d
};

// Time at which the ray (fast coordinates) leaves the box [lo, lo + size)^3
// shrunk by kSkipMargin voxels on every side: the last time a sample may take
// and still lie inside the box (the fast coordinates' error is far below the
// margin).
__device__ __forceinline__ float box_exit(const RayFast &rf, float lox, float loy, float loz, float size) {
    const float ex = ((rf.d[0] > 0.f ? lox + (size - kSkipMargin) : lox + kSkipMargin) - rf.o[0]) * rf.inv_d[0];
    const float ey = ((rf.d[1] > 0.f ? loy + (size - kSkipMargin) : loy + kSkipMargin) - rf.o[1]) * rf.inv_d[1];
    const float ez = ((rf.d[2] > 0.f ? loz + (size - kSkipMargin) : loz + kSkipMargin) - rf.o[2]) * rf.inv_d[2];
    return fminf(fminf(ex, ey), ez);
}

__device__ __forceinline__ int axis_floor(float q, float o, float d, float cell, float ct) {
    const float fr = q - floorf(q);
    if (fabsf(q) < 2048.f && fr > 4e-3f && fr < 1.f - 4e-3f) return __float2int_rd(q);
    return floor_sat((o + d * ct) / cell);
}

__device__ __forceinline__ void sample_voxel(const RayParams &p, const f3 &org, const f3 &dir, const RayFast &rf,
                                             float ct, int &sx, int &sy, int &sz) {
    sx = axis_floor(fmaf(rf.d[0], ct, rf.o[0]), org.x, dir.x, p.cell.x, ct);
    sy = axis_floor(fmaf(rf.d[1], ct, rf.o[1]), org.y, dir.y, p.cell.y, ct);
    sz = axis_floor(fmaf(rf.d[2], ct, rf.o[2]), org.z, dir.z, p.cell.z, ct);
}

// A block takes 16 x kRayBlockRows pixels, a warp an 8 x 4 tile.
constexpr int kRayBlockRows = 16;
constexpr int kRayThreads = 16 * kRayBlockRows;

template <int FMT, bool SKIP, bool STATS>
__global__ void __launch_bounds__(kRayThreads) raycast_kernel(const void *__restrict__ vol, float *__restrict__ vmap,
                                                     float *__restrict__ nmap, const __grid_constant__ RayParams p) {
    // each warp takes an 8x4 tile so its rays start close together and
    // sample neighbouring voxels
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * kRayBlockRows + (warp >> 1) * 4 + (lane >> 3);
    const int W = p.intr.cols, H = p.intr.rows;
    // the pose: from the parameters, or read on the device
    tde_matrix3f R = p.R;
    f3 org{p.t.x, p.t.y, p.t.z};
    if (p.dpose) {
        __shared__ float s_pose[12];
        if (tid < 12) s_pose[tid] = tid < 9 ? p.dpose->R[tid] : p.dpose->t[tid - 9];
        __syncthreads();
        R = tde_matrix3f{{{s_pose[0], s_pose[1], s_pose[2]}, {s_pose[3], s_pose[4], s_pose[5]},
                          {s_pose[6], s_pose[7], s_pose[8]}}};
        org = f3{s_pose[9], s_pose[10], s_pose[11]};
    }
    const float qnan = __int_as_float(0x7fffffff);
    const tde_point3i N = p.rb.voxels_size;
    const tde_point3f V = p.rb.volume_size;
    const float step = p.time_step;
    // lanes outside the image stay (no early return): the warp reconverges
    // before the refinement
    const bool inside = x < W && y < H;
    float vx_out = qnan, vy_out = qnan, vz_out = qnan;
    float nx_out = qnan, ny_out = qnan, nz_out = qnan;

    f3 rnu{((float)x - p.intr.cx) / p.intr.fx, ((float)y - p.intr.cy) / p.intr.fy, 1.f};
    f3 rn2 = mat_vec(R, rnu);
    f3 ray_next{rn2.x + org.x, rn2.y + org.y, rn2.z + org.z};
    f3 dir = normalized(f3{ray_next.x - org.x, ray_next.y - org.y, ray_next.z - org.z});
    dir.x = (dir.x == 0.f) ? 1e-15f : dir.x;
    dir.y = (dir.y == 0.f) ? 1e-15f : dir.y;
    dir.z = (dir.z == 0.f) ? 1e-15f : dir.z;

    // getMinTime / getMaxTime: raycast.cl:153-171
    float txmin = ((dir.x > 0 ? 0.f : V.x) - org.x) / dir.x;
    float tymin = ((dir.y > 0 ? 0.f : V.y) - org.y) / dir.y;
    float tzmin = ((dir.z > 0 ? 0.f : V.z) - org.z) / dir.z;
    float t_start = cl_fmax(cl_fmax(txmin, tymin), tzmin);
    float txmax = ((dir.x > 0 ? V.x : 0.f) - org.x) / dir.x;
    float tymax = ((dir.y > 0 ? V.y : 0.f) - org.y) / dir.y;
    float tzmax = ((dir.z > 0 ? V.z : 0.f) - org.z) / dir.z;
    float t_exit = cl_fmin(cl_fmin(txmax, tymax), tzmax);
    t_start = cl_fmax(t_start, 0.f);

    // the march finds the zero crossing; the secant refinement and the normal
    // run after it, once per warp for all lanes that hit (lanes reaching the
    // crossing at different samples would otherwise refine one by one)
    bool hit = false;
    float hit_time = 0.f;
    if (inside && !(t_start >= t_exit)) {
        float time_curr = t_start;
        f3 pu = along(org, dir, time_curr);
        int gx = floor_sat(pu.x / p.cell.x), gy = floor_sat(pu.y / p.cell.y), gz = floor_sat(pu.z / p.cell.z);
        gx = max(0, min(gx, N.x - 1));
        gy = max(0, min(gy, N.y - 1));
        gz = max(0, min(gz, N.z - 1));
        RayFast rf;
        rf.o[0] = org.x * p.inv_cell[0]; rf.o[1] = org.y * p.inv_cell[1]; rf.o[2] = org.z * p.inv_cell[2];
        rf.d[0] = dir.x * p.inv_cell[0]; rf.d[1] = dir.y * p.inv_cell[1]; rf.d[2] = dir.z * p.inv_cell[2];
        rf.inv_d[0] = 1.f / rf.d[0]; rf.inv_d[1] = 1.f / rf.d[1]; rf.inv_d[2] = 1.f / rf.d[2];
        // previous sample: its value when `known`, else only "non-negative";
        // its time lets the value be fetched when it turns out to matter
        float tsdf = read_tsdf<FMT, STATS>(vol, p, gx, gy, gz);
        bool known = true;
        float prev_ct = time_curr;
        const int nbx = (N.x + 7) >> 3, nby = (N.y + 7) >> 3;
        const int nsx = (N.x + 31) >> 5, nsy = (N.y + 31) >> 5;
        int last_super = -1;

        // raycast.cl:254-404, one sample per iteration
        while (time_curr < p.max_time) {
            const float ct = time_curr + step;
            int sx, sy, sz;
            sample_voxel(p, org, dir, rf, ct, sx, sy, sz);
            if (!((unsigned)sx < (unsigned)N.x && (unsigned)sy < (unsigned)N.y && (unsigned)sz < (unsigned)N.z)) break;
            int px = sx + p.rb.origin_GRID.x; px -= px >= N.x ? N.x : 0;
            int py = sy + p.rb.origin_GRID.y; py -= py >= N.y ? N.y : 0;
            int pz = sz + p.rb.origin_GRID.z; pz -= pz >= N.z ? N.z : 0;
            bool have = true;
            if (SKIP) {
                if (p.super_flags && !(known && tsdf < 0.f)) {
                    const int sid = (px >> 5) + nsx * ((py >> 5) + nsy * (pz >> 5));
                    if (sid != last_super) {
                        last_super = sid;
                        if (!__ldg(p.super_flags + sid)) {
                            // A 32^3 super-brick with no negative value entered after a
                            // non-negative sample: no test can fire inside it, so time
                            // advances by the same additions without evaluating samples
                            // until the next one nears the exit.
                            const float lim = box_exit(rf, (float)(sx - (px & 31)), (float)(sy - (py & 31)),
                                                       (float)(sz - (pz & 31)), 32.f);
                            float tn = time_curr;
                            int m = 0;
                            while (tn < p.max_time && tn + step < lim) { tn = tn + step; ++m; }
                            if (m > 0) {
                                time_curr = tn;
                                known = false;
                                prev_ct = tn;
                                continue;
                            }
                        }
                    }
                }
                have = __ldg(p.neg_flags + ((px >> 3) + nbx * ((py >> 3) + nby * (pz >> 3)))) != 0;
            }
            const size_t addr = (size_t)px + (size_t)N.x * ((size_t)py + (size_t)N.y * (size_t)pz);
            float cur = 0.f;
            if (SKIP && !have) {
                if (!(known && tsdf < 0.f)) {
                    // a non-negative sample after a non-negative one: no test can
                    // fire, nor at the following samples inside this 8^3 brick,
                    // which advance by the same additions
                    const float lim = box_exit(rf, (float)(sx - (px & 7)), (float)(sy - (py & 7)),
                                               (float)(sz - (pz & 7)), 8.f);
                    float tn = ct;
                    while (tn < p.max_time && tn + step < lim) tn = tn + step;
                    known = false;
                    prev_ct = tn;
                    time_curr = tn;
                    continue;
                }
            }
            cur = load_rec<FMT, STATS>(vol, p, addr);
            if (SKIP && !known) {
                if (!(cur < 0.f)) {  // prev >= 0 and cur >= 0
                    tsdf = cur;
                    known = true;
                    prev_ct = ct;
                    time_curr = ct;
                    continue;
                }
                // the previous sample's sign decides a crossing: fetch it
                int qx, qy, qz;
                sample_voxel(p, org, dir, rf, prev_ct, qx, qy, qz);
                tsdf = read_tsdf<FMT, STATS>(vol, p, qx, qy, qz);
            }
            const float tsdf_prev = tsdf;
            tsdf = cur;
            known = true;
            prev_ct = ct;
            if (tsdf_prev < 0.f && tsdf > 0.f) break;
            if (tsdf_prev > 0.f && tsdf < 0.f) {
                hit = true;
                hit_time = time_curr;
                break;
            }
            time_curr = ct;
        }
    }
    __syncwarp();
    if (hit) refine_surface<FMT, STATS>(vol, p, org, dir, hit_time, vx_out, vy_out, vz_out, nx_out, ny_out, nz_out);
    if (inside) {
        const size_t pix = (size_t)W * y + x;
        vmap[3 * pix + 0] = vx_out; vmap[3 * pix + 1] = vy_out; vmap[3 * pix + 2] = vz_out;
        nmap[3 * pix + 0] = nx_out; nmap[3 * pix + 1] = ny_out; nmap[3 * pix + 2] = nz_out;
    }
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

// 2x2 mean of a vertex (NORMAL false) or normal map at destination pixel
// (x, y): the same IEEE operations as resize_map_kernel.
template <bool NORMAL>
__device__ __forceinline__ f3 resize_px(const float *__restrict__ src, int sc, int x, int y) {
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
    if (!ok) return f3{qnan, qnan, qnan};
    if (NORMAL) {
        float d = 0.f; d += sx * sx; d += sy * sy; d += sz * sz;
        float rs = 1.f / sqrtf(d);
        return f3{sx * rs, sy * rs, sz * rs};
    }
    return f3{sx * 0.25f, sy * 0.25f, sz * 0.25f};
}

// The same mean over four values already in registers (level 1 -> 2).
template <bool NORMAL>
__device__ __forceinline__ f3 mean4(const f3 (&q)[4]) {
    const float qnan = __int_as_float(0x7fffffff);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    bool ok = true;
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        ok = ok && !isnan(q[k].x);
        sx = sx + q[k].x; sy = sy + q[k].y; sz = sz + q[k].z;
    }
    if (!ok) return f3{qnan, qnan, qnan};
    if (NORMAL) {
        float d = 0.f; d += sx * sx; d += sy * sy; d += sz * sz;
        float rs = 1.f / sqrtf(d);
        return f3{sx * rs, sy * rs, sz * rs};
    }
    return f3{sx * 0.25f, sy * 0.25f, sz * 0.25f};
}

__device__ __forceinline__ void put3(float *dst, size_t i, f3 v) {
    dst[3 * i] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
}

// Model-map pyramid in one launch: thread (X, Y) makes level-1 pixels
// (2X..2X+1, 2Y..2Y+1) of the vertex and normal maps and, from those four
// values, level-2 pixel (X, Y) -- the values resize_map_kernel gives level
// by level.  v2/n2 null: level 1 only.
__global__ void resize_model_maps_kernel(const float *__restrict__ v0, const float *__restrict__ n0,
                                         float *__restrict__ v1, float *__restrict__ n1, float *__restrict__ v2,
                                         float *__restrict__ n2, int c0, int r0) {
    const int c1 = c0 >> 1, r1 = r0 >> 1, c2 = c1 >> 1, r2 = r1 >> 1;
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y * blockDim.y + threadIdx.y;
    if (2 * X >= c1 || 2 * Y >= r1) return;
    f3 qv[4], qn[4];
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = 2 * X + (k & 1), y = 2 * Y + (k >> 1);
        if (x >= c1 || y >= r1) { qv[k] = qn[k] = f3{0.f, 0.f, 0.f}; continue; }
        qv[k] = resize_px<false>(v0, c0, x, y);
        qn[k] = resize_px<true>(n0, c0, x, y);
        put3(v1, (size_t)y * c1 + x, qv[k]);
        put3(n1, (size_t)y * c1 + x, qn[k]);
    }
    if (v2 && X < c2 && Y < r2) {
        put3(v2, (size_t)Y * c2 + X, mean4<false>(qv));
        put3(n2, (size_t)Y * c2 + X, mean4<true>(qn));
    }
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
                   const tde_point3f &cell, const CamPose *dpose, const uint8_t *neg_flags, cudaStream_t stream,
                   unsigned *touched) {
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
    p.touched = touched;
    dim3 block(kRayThreads);
    dim3 grid(div_up(intr.cols, 16), div_up(intr.rows, kRayBlockRows));
    return dispatch_format(format, [&](auto F) {
        constexpr int FM = decltype(F)::value;
        if (touched) {
            if (neg_flags) raycast_kernel<FM, true, true><<<grid, block, 0, stream>>>(volume, vmap, nmap, p);
            else raycast_kernel<FM, false, true><<<grid, block, 0, stream>>>(volume, vmap, nmap, p);
        } else {
            if (neg_flags) raycast_kernel<FM, true, false><<<grid, block, 0, stream>>>(volume, vmap, nmap, p);
            else raycast_kernel<FM, false, false><<<grid, block, 0, stream>>>(volume, vmap, nmap, p);
        }
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

int launch_resize_model_maps(const float *v0, const float *n0, float *v1, float *n1, float *v2, float *n2, int c0,
                             int r0, cudaStream_t stream) {
    dim3 block(32, 8);
    dim3 grid(div_up(div_up(c0 >> 1, 2), 32), div_up(div_up(r0 >> 1, 2), 8));
    resize_model_maps_kernel<<<grid, block, 0, stream>>>(v0, n0, v1, n1, v2, n2, c0, r0);
    return check_launch("resize_model_maps");
}

int launch_transform_maps(const float *vs, const float *ns, float *vd, float *nd, const tde_matrix3f &R,
                          const tde_point3f &t, int W, int H, cudaStream_t stream) {
    dim3 block(32, 8);
    dim3 grid(div_up(W, 32), div_up(H, 8));
    transform_maps_kernel<<<grid, block, 0, stream>>>(vs, ns, vd, nd, R, t, W, H);
    return check_launch("transform_maps");
}

}  // namespace tde
