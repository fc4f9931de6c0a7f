// wrappers.cpp -- the reference's C++ API (include/3deye/) over the C-ABI.
//
// Compiled by the host C++ compiler without CUDA headers: the reference
// defines its own global `dim3`, so this layer reaches the GPU only through
// tde_capi.h.  Every function completes its GPU work before returning, as the
// reference's clFinish-after-launch does (common/src/opencl_helper.cpp:662-672).
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../../include/3deye/gpu_array.h"
#include "../../include/3deye/kernel_manager.h"
#include "../../include/3deye/matrix.h"
#include "../../include/3deye/opencl_wrappers.h"

namespace {

int g_tsdf_format = TDE_TSDF_I16;

void check(int status, const char *what) {
    if (status != TDE_OK) throw std::runtime_error(std::string(what) + ": " + tde_last_error());
}

void sync(const char *what) { check(tde_device_synchronize(), what); }

const tde_intrinsics *I(const intrinsics &in) { return reinterpret_cast<const tde_intrinsics *>(&in); }
const tde_matrix3f *M(const matrix_3f &m) { return reinterpret_cast<const tde_matrix3f *>(&m); }
const tde_point3f *V(const point_3f &p) { return reinterpret_cast<const tde_point3f *>(&p); }
tde_point3i P3(const point_3i &p) { return tde_point3i{p.x, p.y, p.z}; }
const tde_round_buffer *RB(const round_buffer *rb) {
    if (!rb) throw std::runtime_error("null round_buffer");
    return rb->c_abi();
}

void *dev(gpu_array_base *a, const char *what) {
    if (!a || !a->device()) throw std::runtime_error(std::string(what) + ": buffer not allocated on the device");
    return a->device();
}

const char *const kKnown[] = {
    "compute_bilateral_filtering", "compute_depth_pyramid", "compute_vertex_map", "compute_normal_map_eigen",
    "estimate_combined", "transform_estimation", "clean_buff", "scale_depth", "integrate_tsdf_volume", "raycast",
    "resize_vertex_map", "resize_normal_map", "transform_map", "scan_slice_of_both_volumes", "extract_slice_as_cloud",
    "scan_slice_of_tsdf_volume", "extract_tsdf_slice_as_cloud", "scan_pow2", "scan_subarrays", "clean_tsdf_slice",
    "clean_color_slice", "init_tsdf", "integrate_color_volume", "scan_the_whole_array", "extract_tsdf_cloud",
    "extract_colors", "generate_image", "scan_slice_of_color_volume", "extract_color_slice_as_cloud",
    "prepare_initial_frames_rgbd", "generate_intensity_and_depth_pyramid", "create_intensity_derivatives",
    "scan_for_interest_point", "extract_interest_points", "scan_list_of_valid_correspondence",
    "compute_least_squares_equation"};

string base_name(const string &n) {
    if (n.size() > 3 && n.compare(n.size() - 3, 3, ".cl") == 0) return n.substr(0, n.size() - 3);
    return n;
}

// Slab extraction through the C-ABI: count, size, extract (the reference
// counts, scans and extracts per chunk, opencl_wrappers.cpp:885-955).
// Count pass (capacity 0), then the scatter into a buffer of that size.
// `whole_cell` set: every voxel, no colour plane, metric points
// (Extract_Tsdf_Volume).
void extract(point_3i mn, point_3i mx, round_buffer *rb, gpu_array_base *vol, gpu_array_base *color,
             matrix<Point_XYZI> &pts_out, matrix<Point_Color> *cols_out, const point_3f *whole_cell = nullptr) {
    const bool whole = whole_cell != nullptr;
    const tde_round_buffer *r = RB(rb);
    size_t sb = whole ? tde_extract_tsdf_volume_scratch_bytes(r) : tde_extract_slice_scratch_bytes(r);
    if (!sb) throw std::runtime_error("Extract_Slice: bad round_buffer");
    void *scratch = nullptr, *cnt = nullptr, *pts = nullptr, *cols = nullptr;
    check(tde_device_malloc(&scratch, sb), "Extract_Slice");
    auto release = [&] {
        tde_device_free(scratch); tde_device_free(cnt); tde_device_free(pts); tde_device_free(cols);
    };
    try {
        check(tde_device_malloc(&cnt, sizeof(uint32_t)), "Extract_Slice");
        const tde_color *cv = color ? static_cast<const tde_color *>(dev(color, "Extract_Slice colour")) : nullptr;
        auto run = [&](tde_xyzi *p, tde_color *c, uint32_t cap) {
            if (whole)
                check(tde_extract_tsdf_volume(dev(vol, "Extract_Tsdf_Volume"), g_tsdf_format, r, *V(*whole_cell),
                                              scratch, sb, p, nullptr, cap, static_cast<uint32_t *>(cnt), nullptr),
                      "Extract_Tsdf_Volume");
            else
                check(tde_extract_slice(dev(vol, "Extract_Slice"), g_tsdf_format, cv, P3(mn), P3(mx), r, scratch, sb,
                                        p, c, nullptr, cap, static_cast<uint32_t *>(cnt), nullptr),
                      "Extract_Slice");
        };
        run(nullptr, nullptr, 0);
        uint32_t n = 0;
        check(tde_memcpy(&n, cnt, sizeof(n), 1), "Extract_Slice");
        if (n) {
            check(tde_device_malloc(&pts, (size_t)n * sizeof(tde_xyzi)), "Extract_Slice");
            if (cols_out) check(tde_device_malloc(&cols, (size_t)n * sizeof(tde_color)), "Extract_Slice");
            run(static_cast<tde_xyzi *>(pts), static_cast<tde_color *>(cols), n);
            matrix<Point_XYZI> part(n);
            check(tde_memcpy(part.data, pts, (size_t)n * sizeof(tde_xyzi), 1), "Extract_Slice");
            pts_out.extend_from(part);
            if (cols_out) {
                matrix<Point_Color> cpart(n);
                check(tde_memcpy(cpart.data, cols, (size_t)n * sizeof(tde_color), 1), "Extract_Slice");
                cols_out->extend_from(cpart);
            }
        }
    } catch (...) {
        release();
        throw;
    }
    release();
}

}  // namespace

void tde_cxx_throw_if(int status, const char *what) { check(status, what); }

// ---------------------------------------------------------------------------
// gpu_array_base (common/src/gpu_array_base.cpp:5-186)
// ---------------------------------------------------------------------------
gpu_array_base::~gpu_array_base() { dev_free(); }

void gpu_array_base::set_size(const dim3 &s) {
    if (s.x == 0 || s.y == 0 || s.z == 0) throw std::runtime_error("gpu_array::set_size: a dimension is zero");
    sizes = s;
    total_size = (unsigned)(s.x * s.y * s.z);
}

void gpu_array_base::dev_alloc() {
    if (device_ptr) return;
    check(tde_device_malloc(&device_ptr, bytes()), "gpu_array::dev_alloc");
    need_to_prepare = false;
}

void gpu_array_base::dev_free() {
    if (device_ptr) {
        tde_device_free(device_ptr);
        device_ptr = nullptr;
    }
}

void gpu_array_base::memcpy_to_dev(void *host_src) {
    check(tde_memcpy(device_ptr, host_src, bytes(), 0), "gpu_array::memcpy_to_dev");
}

void gpu_array_base::memcpy_from_dev(void *host_dst) {
    check(tde_memcpy(host_dst, device_ptr, bytes(), 1), "gpu_array::memcpy_from_dev");
}

void gpu_array_base::copy_to(gpu_array_base *dst) {
    if (!dst || dst->bytes() < bytes()) throw std::runtime_error("gpu_array::copy_to: destination too small");
    check(tde_memcpy(dst->device(), device_ptr, bytes(), 2), "gpu_array::copy_to");
}

// ---------------------------------------------------------------------------
// round_buffer (common/src/round_buffer.cpp:5-74)
// ---------------------------------------------------------------------------
round_buffer::round_buffer() { set_default_values(); }
round_buffer::round_buffer(const dim3 &d) {
    set_default_values();
    set_voxels_size(d.width, d.height, d.depth);
    set_memory_index();
}
round_buffer::round_buffer(size_t w, size_t h, size_t d) {
    set_default_values();
    set_voxels_size(w, h, d);
    set_memory_index();
}
round_buffer::round_buffer(point_3i voxels, point_3f metric) {
    set_default_values();
    voxels_size = voxels;
    volume_size = metric;
    set_memory_index();
}
void round_buffer::set_default_values() {
    origin_GRID = make_point_3i(0, 0, 0);
    origin_GRID_global = make_point_3f(0.f, 0.f, 0.f);
    origin_metric = origin_GRID_global;
    voxels_size = make_point_3i(512, 512, 512);
    volume_size = make_point_3f(3.f, 3.f, 3.f);
    end_index = 0;
    set_memory_index();
}
void round_buffer::set_voxels_size(size_t w, size_t h, size_t d) {
    voxels_size.x = (int)w;
    voxels_size.y = (int)h;
    voxels_size.z = (int)d;
}
void round_buffer::set_memory_index() {
    start_index = 0;
    buffer_length = voxels_size.x * voxels_size.y * voxels_size.z;
}

// ---------------------------------------------------------------------------
// kernel_manager / opencl_kernel
// ---------------------------------------------------------------------------
bool tde_kernel_known(const string &name) {
    string b = base_name(name);
    for (const char *k : kKnown)
        if (b == k) return true;
    return false;
}

opencl_kernel::opencl_kernel(const string &name, profiling_level) : kernel_name(base_name(name)) {
    if (!tde_kernel_known(kernel_name)) throw std::runtime_error("Kernel " + name + " Not found!");
}
opencl_kernel::~opencl_kernel() {}
void opencl_kernel::free_args() { num_args = 0; }

kernel_manager::kernel_manager(const string &p, vector<string> &names) : path(p) {
    for (const string &n : names) {
        string b = base_name(n);
        if (!kernels.count(b)) kernels[b] = new opencl_kernel(b);
    }
}
kernel_manager::~kernel_manager() {
    for (auto &kv : kernels) delete kv.second;
}
opencl_kernel *kernel_manager::Get_Kernel(string &name) {
    auto it = kernels.find(base_name(name));
    if (it == kernels.end()) throw std::runtime_error("Kernel " + name + " Not found!");
    it->second->free_args();
    return it->second;
}
opencl_kernel *kernel_manager::Get_Kernel(const char *name) {
    string s(name);
    return Get_Kernel(s);
}

// ---------------------------------------------------------------------------
// opencl_wrappers (common/src/opencl_wrappers.cpp)
// ---------------------------------------------------------------------------
void Set_Tsdf_Storage_Format(int f) {
    if (f != TDE_TSDF_I16 && f != TDE_TSDF_F16 && f != TDE_TSDF_F32)
        throw std::runtime_error("Set_Tsdf_Storage_Format: unknown format");
    g_tsdf_format = f;
}
int Get_Tsdf_Storage_Format() { return g_tsdf_format; }

// opencl_wrappers.cpp:21-64
void Integrate_Tsdf_Data(gpu_array_base *gDepth_Frame, gpu_array_base *gDepth_Frame_Scaled,
                         gpu_array_base *gTsdf_Volume, intrinsics &Intr, matrix_3f &Rotation_Inverse,
                         vector_3f &Translation, float Truncation_Distance, point_3f &Cell_Size,
                         round_buffer *Tsdf_Buffer, kernel_manager *, int) {
    check(tde_scale_depth(static_cast<const uint16_t *>(dev(gDepth_Frame, "Integrate_Tsdf_Data")),
                          static_cast<float *>(dev(gDepth_Frame_Scaled, "Integrate_Tsdf_Data")), I(Intr), nullptr),
          "Integrate_Tsdf_Data");
    check(tde_integrate_tsdf(static_cast<const float *>(gDepth_Frame_Scaled->device()),
                             dev(gTsdf_Volume, "Integrate_Tsdf_Data"), g_tsdf_format, Truncation_Distance,
                             M(Rotation_Inverse), V(Translation), I(Intr), V(Cell_Size), RB(Tsdf_Buffer),
                             MAX_TSDF_WEIGHT, nullptr),
          "Integrate_Tsdf_Data");
    sync("Integrate_Tsdf_Data");
}

// opencl_wrappers.cpp:66-95
void Raycast(gpu_array_base *gTsdf_Volume, gpu_array_base *Vertex_Map, gpu_array_base *Normal_Map,
             round_buffer *Round_Buffer, vector_3f &Translation, matrix_3f &Rotation, float Truncation_Distance,
             intrinsics &Intr, point_3f &Cell_Size, opencl_kernel *) {
    check(tde_raycast(dev(gTsdf_Volume, "Raycast"), g_tsdf_format, static_cast<float *>(dev(Vertex_Map, "Raycast")),
                      static_cast<float *>(dev(Normal_Map, "Raycast")), V(Translation), M(Rotation),
                      Truncation_Distance, I(Intr), RB(Round_Buffer), V(Cell_Size), nullptr),
          "Raycast");
    sync("Raycast");
}

// opencl_wrappers.cpp:97-146; Intr describes the source (finer) level.
void Resize_Vertex_Map(gpu_array_base *in, gpu_array_base *out, intrinsics &Intr, opencl_kernel *) {
    check(tde_resize_vertex_map(static_cast<const float *>(dev(in, "Resize_Vertex_Map")),
                                static_cast<float *>(dev(out, "Resize_Vertex_Map")), Intr.cols, Intr.rows, nullptr),
          "Resize_Vertex_Map");
    sync("Resize_Vertex_Map");
}

void Resize_Normal_Map(gpu_array_base *in, gpu_array_base *out, intrinsics &Intr, opencl_kernel *) {
    check(tde_resize_normal_map(static_cast<const float *>(dev(in, "Resize_Normal_Map")),
                                static_cast<float *>(dev(out, "Resize_Normal_Map")), Intr.cols, Intr.rows, nullptr),
          "Resize_Normal_Map");
    sync("Resize_Normal_Map");
}

// opencl_wrappers.cpp:148-179
void Transform_Maps(gpu_array_base *vs, gpu_array_base *ns, gpu_array_base *vd, gpu_array_base *nd,
                    matrix_3f &Rotation, vector_3f &Translation, intrinsics &Intr, opencl_kernel *) {
    check(tde_transform_maps(static_cast<const float *>(dev(vs, "Transform_Maps")),
                             static_cast<const float *>(dev(ns, "Transform_Maps")),
                             static_cast<float *>(dev(vd, "Transform_Maps")), static_cast<float *>(dev(nd, "Transform_Maps")),
                             M(Rotation), V(Translation), Intr.cols, Intr.rows, nullptr),
          "Transform_Maps");
    sync("Transform_Maps");
}

// opencl_wrappers.cpp:181-214.  gRGB_Frame: cols x rows pixels of 3 bytes (r, g, b);
// Vertex_Map: the model surface raycast from the same pose.
void Integrate_Colors(gpu_array_base *gTsdf_Color_Volume, gpu_array_base *gRGB_Frame, gpu_array_base *Vertex_Map,
                      intrinsics &Intr, matrix_3f &Rotation_Inverse, vector_3f &Translation, float Truncation_Distance,
                      int Max_Weight, point_3f Cell_Size, round_buffer *Round_Buffer, opencl_kernel *) {
    check(tde_integrate_colors(static_cast<tde_color *>(dev(gTsdf_Color_Volume, "Integrate_Colors")),
                               static_cast<const uint8_t *>(dev(gRGB_Frame, "Integrate_Colors")),
                               static_cast<const float *>(dev(Vertex_Map, "Integrate_Colors")), I(Intr),
                               M(Rotation_Inverse), V(Translation), Truncation_Distance, Max_Weight, V(Cell_Size),
                               RB(Round_Buffer), nullptr),
          "Integrate_Colors");
    sync("Integrate_Colors");
}

// opencl_wrappers.cpp:216-235; Trunc_Dist is the maximum depth in millimetres.
void Apply_Billateral_Filtration(gpu_array_base *gDepth, const intrinsics &Intr, float Trunc_Dist, opencl_kernel *,
                                 gpu_array_base *gDepth_Filtered) {
    uint32_t maxd = Trunc_Dist > 0.f ? (uint32_t)Trunc_Dist : 0u;
    check(tde_bilateral_filter(static_cast<const uint16_t *>(dev(gDepth, "Apply_Billateral_Filtration")),
                               static_cast<uint16_t *>(dev(gDepth_Filtered, "Apply_Billateral_Filtration")), Intr.cols,
                               Intr.rows, DEFAULT_SIGMA_SPACE, DEFAULT_SIGMA_COLOR, maxd, nullptr),
          "Apply_Billateral_Filtration");
    sync("Apply_Billateral_Filtration");
}

// opencl_wrappers.cpp:245-271
void Create_Pyramid(vector<gpu_array_base *> &pyr, int levels, intrinsics Intr, kernel_manager *) {
    if ((int)pyr.size() < levels) throw std::runtime_error("Create_Pyramid: fewer buffers than levels");
    for (int i = 1; i < levels; ++i)
        check(tde_depth_pyramid_level(static_cast<const uint16_t *>(dev(pyr[i - 1], "Create_Pyramid")),
                                      static_cast<uint16_t *>(dev(pyr[i], "Create_Pyramid")), Intr.cols >> (i - 1),
                                      Intr.rows >> (i - 1), DEFAULT_SIGMA_COLOR, nullptr),
              "Create_Pyramid");
    sync("Create_Pyramid");
}

// opencl_wrappers.cpp:281-305
void Create_Vertex_Maps(vector<gpu_array_base *> &depths, vector<gpu_array_base *> &vertexes, intrinsics Intr,
                        int levels, kernel_manager *) {
    for (int i = 0; i < levels; ++i) {
        intrinsics li = Intr(i);
        check(tde_vertex_map(static_cast<const uint16_t *>(dev(depths.at(i), "Create_Vertex_Maps")),
                             static_cast<float *>(dev(vertexes.at(i), "Create_Vertex_Maps")), I(li), nullptr),
              "Create_Vertex_Maps");
    }
    sync("Create_Vertex_Maps");
}

// opencl_wrappers.cpp:315-343
void Create_Normal_Maps(vector<gpu_array_base *> &vertexes, vector<gpu_array_base *> &normals, intrinsics Intr,
                        int levels, kernel_manager *) {
    for (int i = 0; i < levels; ++i)
        check(tde_normal_map(static_cast<const float *>(dev(vertexes.at(i), "Create_Normal_Maps")),
                             static_cast<float *>(dev(normals.at(i), "Create_Normal_Maps")), Intr.cols >> i,
                             Intr.rows >> i, nullptr),
              "Create_Normal_Maps");
    sync("Create_Normal_Maps");
}

// opencl_wrappers.cpp:364-438: sums on the GPU, 27 floats back, unpacked
// into the symmetric A (6x6) and b (6) exactly as the reference does.
void Estimate_Combined(matrix_3f &Rotation_Current, vector_3f &Translation_Current, gpu_array_base *vcur,
                       gpu_array_base *ncur, matrix_3f &Rotation_Previous_Inverse, vector_3f &Translation_Previous,
                       intrinsics &Intr, gpu_array_base *vprev, gpu_array_base *nprev, float Distance_Threshold,
                       float Angle_Threshold, gpu_array_base *gbuf, gpu_array_base *gMBuf, double *A, double *b,
                       kernel_manager *) {
    const size_t need = tde_estimate_combined_gbuf_floats(Intr.cols, Intr.rows) * sizeof(float);
    if (!gbuf || gbuf->bytes() < need)
        throw std::runtime_error("Estimate_Combined: gbuf smaller than tde_estimate_combined_gbuf_floats()");
    if (!gMBuf || gMBuf->bytes() < 27 * sizeof(float)) throw std::runtime_error("Estimate_Combined: gMBuf < 27 floats");
    check(tde_estimate_combined(static_cast<const float *>(dev(vcur, "Estimate_Combined")),
                                static_cast<const float *>(dev(ncur, "Estimate_Combined")),
                                static_cast<const float *>(dev(vprev, "Estimate_Combined")),
                                static_cast<const float *>(dev(nprev, "Estimate_Combined")), M(Rotation_Current),
                                V(Translation_Current), M(Rotation_Previous_Inverse), V(Translation_Previous), I(Intr),
                                Distance_Threshold, Angle_Threshold, static_cast<float *>(dev(gbuf, "Estimate_Combined")),
                                static_cast<float *>(dev(gMBuf, "Estimate_Combined")), nullptr),
          "Estimate_Combined");
    float mbuf[27];
    check(tde_memcpy(mbuf, gMBuf->device(), sizeof(mbuf), 1), "Estimate_Combined");
    int shift = 0;
    for (int k = 0; k < 6; ++k)
        for (int j = k; j < 7; ++j) {
            float value = mbuf[shift++];
            if (j == 6) b[k] = value;
            else A[j * 6 + k] = A[k * 6 + j] = value;
        }
}

// opencl_wrappers.cpp:440-543: every zero crossing as the metric centre of
// the voxel it names; appends to the cloud, as extend_from does there.
void Extract_Tsdf_Volume(round_buffer *Round_Buffer, const point_3f &Cell_Size, gpu_array_base *gTsdf_Volume,
                         kernel_manager *, matrix<Point_XYZI> &Resulting_Cloud_Parallel) {
    extract(point_3i{}, point_3i{}, Round_Buffer, gTsdf_Volume, nullptr, Resulting_Cloud_Parallel, nullptr,
            &Cell_Size);
}

// opencl_wrappers.cpp:545-581: the colour of the voxel holding each point of
// Vertex_Point_Cloud, into Resulting_Color_Point_Cloud (sized like the cloud
// by the caller, as there).
void Extract_Color_Volume(gpu_array_base *gColor_Volume, round_buffer *Round_Buffer,
                          matrix<Point_XYZI> &Vertex_Point_Cloud, point_3f Cell_Size, opencl_kernel *,
                          matrix<Point_Color> &Resulting_Color_Point_Cloud) {
    const uint32_t n = Vertex_Point_Cloud.Get_Num_Of_Elem();
    if (Resulting_Color_Point_Cloud.Get_Num_Of_Elem() < n)
        throw std::runtime_error("Extract_Color_Volume: colour cloud smaller than the vertex cloud");
    if (!n) return;
    void *pts = nullptr, *cols = nullptr;
    auto release = [&] { tde_device_free(pts); tde_device_free(cols); };
    try {
        check(tde_device_malloc(&pts, (size_t)n * sizeof(tde_xyzi)), "Extract_Color_Volume");
        check(tde_device_malloc(&cols, (size_t)n * sizeof(tde_color)), "Extract_Color_Volume");
        check(tde_memcpy(pts, Vertex_Point_Cloud.data, (size_t)n * sizeof(tde_xyzi), 0), "Extract_Color_Volume");
        check(tde_extract_color_volume(static_cast<const tde_color *>(dev(gColor_Volume, "Extract_Color_Volume")),
                                       RB(Round_Buffer), static_cast<const tde_xyzi *>(pts), n, *V(Cell_Size),
                                       static_cast<tde_color *>(cols), nullptr),
              "Extract_Color_Volume");
        check(tde_memcpy(Resulting_Color_Point_Cloud.data, cols, (size_t)n * sizeof(tde_color), 1),
              "Extract_Color_Volume");
    } catch (...) {
        release();
        throw;
    }
    release();
}

// opencl_wrappers.cpp:583-683 (three planes: +x, +y, +z)
void Extract_Tsdf_Slice(point_3i Min_Bounds, point_3i Max_Bounds, round_buffer *Round_Buffer, point_3f &,
                        gpu_array_base *gTsdf_Volume, kernel_manager *, matrix<Point_XYZI> &cloud) {
    extract(Min_Bounds, Max_Bounds, Round_Buffer, gTsdf_Volume, nullptr, cloud, nullptr);
}

// opencl_wrappers.cpp:856-964
void Extract_Slice(point_3i Min_Bounds, point_3i Max_Bounds, round_buffer *Round_Buffer, gpu_array_base *gTsdf_Volume,
                   gpu_array_base *gColor_Volume, point_3f, kernel_manager *, matrix<Point_XYZI> &Vertex_Slice,
                   matrix<Point_Color> &Color_Slice) {
    extract(Min_Bounds, Max_Bounds, Round_Buffer, gTsdf_Volume, gColor_Volume, Vertex_Slice, &Color_Slice);
}

// opencl_wrappers.cpp:687-782: count, then the colours, appended to the cloud
void Extract_Color_Slice(point_3i Min_Bounds, point_3i Max_Bounds, round_buffer *Round_Buffer,
                         gpu_array_base *gColor_Volume, kernel_manager *, matrix<Point_Color> &cloud) {
    const tde_round_buffer *r = RB(Round_Buffer);
    const size_t sb = tde_extract_slice_scratch_bytes(r);
    if (!sb) throw std::runtime_error("Extract_Color_Slice: bad round_buffer");
    const tde_color *cv = static_cast<const tde_color *>(dev(gColor_Volume, "Extract_Color_Slice"));
    void *scratch = nullptr, *cnt = nullptr, *cols = nullptr;
    auto release = [&] { tde_device_free(scratch); tde_device_free(cnt); tde_device_free(cols); };
    try {
        check(tde_device_malloc(&scratch, sb), "Extract_Color_Slice");
        check(tde_device_malloc(&cnt, sizeof(uint32_t)), "Extract_Color_Slice");
        check(tde_extract_color_slice(cv, P3(Min_Bounds), P3(Max_Bounds), r, scratch, sb, nullptr, 0,
                                      static_cast<uint32_t *>(cnt), nullptr),
              "Extract_Color_Slice");
        uint32_t n = 0;
        check(tde_memcpy(&n, cnt, sizeof(n), 1), "Extract_Color_Slice");
        if (n) {
            check(tde_device_malloc(&cols, (size_t)n * sizeof(tde_color)), "Extract_Color_Slice");
            check(tde_extract_color_slice(cv, P3(Min_Bounds), P3(Max_Bounds), r, scratch, sb,
                                          static_cast<tde_color *>(cols), n, static_cast<uint32_t *>(cnt), nullptr),
                  "Extract_Color_Slice");
            matrix<Point_Color> part(n);
            check(tde_memcpy(part.data, cols, (size_t)n * sizeof(tde_color), 1), "Extract_Color_Slice");
            cloud.extend_from(part);
        }
    } catch (...) {
        release();
        throw;
    }
    release();
}

// opencl_wrappers.cpp:967-992: Image_Out holds cols*rows RGB8 pixels.
void Generate_Image(gpu_array_base *Vertex_Map, gpu_array_base *Normal_Map, intrinsics &Intr, light_source &light,
                    gpu_array_base *Image_Out, opencl_kernel *) {
    if (!Image_Out || Image_Out->bytes() < (size_t)Intr.cols * Intr.rows * 3)
        throw std::runtime_error("Generate_Image: Image_Out smaller than cols*rows*3 bytes");
    check(tde_generate_image(static_cast<const float *>(dev(Vertex_Map, "Generate_Image")),
                             static_cast<const float *>(dev(Normal_Map, "Generate_Image")), Intr.cols, Intr.rows,
                             reinterpret_cast<const tde_light_source *>(&light),
                             static_cast<uint8_t *>(dev(Image_Out, "Generate_Image")), nullptr),
          "Generate_Image");
    sync("Generate_Image");
}

// opencl_wrappers.cpp:835-854
void Clean_Tsdf_Slice(point_3i Min_Bounds, point_3i Max_Bounds, round_buffer *Round_Buffer,
                      gpu_array_base *gTsdf_Volume, opencl_kernel *) {
    check(tde_clean_tsdf_slice(dev(gTsdf_Volume, "Clean_Tsdf_Slice"), g_tsdf_format, P3(Min_Bounds), P3(Max_Bounds),
                               RB(Round_Buffer), nullptr),
          "Clean_Tsdf_Slice");
    sync("Clean_Tsdf_Slice");
}

// opencl_wrappers.cpp:814-833
void Clean_Color_Slice(point_3i Min_Bounds, point_3i Max_Bounds, round_buffer *Round_Buffer,
                       gpu_array_base *gColor_Volume, opencl_kernel *) {
    check(tde_clean_color_slice(static_cast<tde_color *>(dev(gColor_Volume, "Clean_Color_Slice")), P3(Min_Bounds),
                                P3(Max_Bounds), RB(Round_Buffer), nullptr),
          "Clean_Color_Slice");
    sync("Clean_Color_Slice");
}

// opencl_wrappers.cpp:994-1006: zero 27 rows of gPtr->height() floats.
void Clean_Buff(gpu_array_base *gPtr, opencl_kernel *) {
    int width = (int)gPtr->height();
    check(tde_clean_buff(static_cast<float *>(dev(gPtr, "Clean_Buff")), width, nullptr), "Clean_Buff");
    sync("Clean_Buff");
}

// ---- dense RGB-D odometry (opencl_wrappers.cpp:345-362, 1008-1466) ----
namespace {

void need_bytes(gpu_array_base *a, size_t bytes, const char *what) {
    if (!a || !a->device() || a->bytes() < bytes)
        throw std::runtime_error(std::string(what) + ": buffer missing or smaller than " + std::to_string(bytes) +
                                 " bytes");
}

const int16_t *deriv(gpu_array_base *a, size_t n, const char *what) {
    if (a && a->elem_size() != sizeof(int16_t))
        throw std::runtime_error(std::string(what) + ": derivatives must be short (signed Sobel responses)");
    need_bytes(a, n * sizeof(int16_t), what);
    return static_cast<const int16_t *>(a->device());
}

// pose12 (R row-major, t) of a matrix_3f / vector_3f pair and back
void to_pose(const matrix_3f &R, const vector_3f &t, double *p) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) p[3 * r + c] = R.data[r].data[c];
    for (int k = 0; k < 3; ++k) p[9 + k] = t.data[k];
}

}  // namespace

void Prepare_Data_For_RGBD(gpu_array_base *gDepth_Frame, gpu_array_base *gRGB_Frame, gpu_array_base *gIntensity_Image,
                           gpu_array_base *gMetric_Depth, opencl_kernel *) {
    const char *what = "Prepare_Data_For_RGBD";
    if (!gDepth_Frame) throw std::runtime_error("Prepare_Data_For_RGBD: no depth frame");
    const int W = (int)gDepth_Frame->width(), H = (int)std::max(1u, gDepth_Frame->height());
    const size_t n = (size_t)W * H;
    need_bytes(gDepth_Frame, n * sizeof(uint16_t), what);
    need_bytes(gRGB_Frame, n * 3, what);
    need_bytes(gIntensity_Image, n, what);
    need_bytes(gMetric_Depth, n * sizeof(float), what);
    check(tde_rgbd_prepare(static_cast<const uint16_t *>(gDepth_Frame->device()),
                           static_cast<const uint8_t *>(gRGB_Frame->device()),
                           W, H, static_cast<uint8_t *>(gIntensity_Image->device()),
                           static_cast<float *>(gMetric_Depth->device()), nullptr),
          what);
    sync(what);
}

void Generate_Intensity_And_Depth_Pyramid(vector<gpu_array_base *> &ip, vector<gpu_array_base *> &dp, intrinsics Intr,
                                          int levels, kernel_manager *) {
    const char *what = "Generate_Intensity_And_Depth_Pyramid";
    if ((int)ip.size() < levels || (int)dp.size() < levels) throw std::runtime_error(std::string(what) + ": fewer buffers than levels");
    for (int i = 1; i < levels; ++i) {
        const int W = Intr.cols >> (i - 1), H = Intr.rows >> (i - 1);
        const size_t n2 = (size_t)(W >> 1) * (H >> 1);
        need_bytes(ip[i - 1], (size_t)W * H, what);
        need_bytes(dp[i - 1], (size_t)W * H * sizeof(float), what);
        need_bytes(ip[i], n2, what);
        need_bytes(dp[i], n2 * sizeof(float), what);
        check(tde_rgbd_pyramid(static_cast<const uint8_t *>(ip[i - 1]->device()),
                               static_cast<const float *>(dp[i - 1]->device()), W, H,
                               static_cast<uint8_t *>(ip[i]->device()), static_cast<float *>(dp[i]->device()), nullptr),
              what);
    }
    sync(what);
}

void Create_Intensity_Derivatives(vector<gpu_array_base *> &ip, vector<gpu_array_base *> &DI_dx,
                                  vector<gpu_array_base *> &DI_dy, intrinsics Intr, int levels, kernel_manager *) {
    const char *what = "Create_Intensity_Derivatives";
    if ((int)ip.size() < levels || (int)DI_dx.size() < levels || (int)DI_dy.size() < levels)
        throw std::runtime_error(std::string(what) + ": fewer buffers than levels");
    for (int i = 0; i < levels; ++i) {
        const int W = Intr.cols >> i, H = Intr.rows >> i;
        const size_t n = (size_t)W * H;
        need_bytes(ip[i], n, what);
        deriv(DI_dx[i], n, what);
        deriv(DI_dy[i], n, what);
        check(tde_rgbd_derivatives(static_cast<const uint8_t *>(ip[i]->device()), W, H,
                                   static_cast<int16_t *>(DI_dx[i]->device()),
                                   static_cast<int16_t *>(DI_dy[i]->device()), nullptr),
              what);
    }
    sync(what);
}

void Accumulate_Points_Of_Interest_For_RGBD(gpu_array_base *DI_dx, gpu_array_base *DI_dy, float Depth_Scale,
                                            gpu_array_base *Points_Of_Interest, gpu_array_base *Num_Of_Points,
                                            int &num_of_points, kernel_manager *) {
    const char *what = "Accumulate_Points_Of_Interest_For_RGBD";
    if (!DI_dx) throw std::runtime_error(std::string(what) + ": no derivatives");
    const int W = (int)DI_dx->width(), H = (int)std::max(1u, DI_dx->height());
    const size_t n = (size_t)W * H;
    const int16_t *dx = deriv(DI_dx, n, what), *dy = deriv(DI_dy, n, what);
    need_bytes(Num_Of_Points, sizeof(uint32_t), what);
    uint32_t capacity = 0;
    if (Points_Of_Interest) {
        need_bytes(Points_Of_Interest, sizeof(tde_point2i), what);
        capacity = (uint32_t)(Points_Of_Interest->bytes() / sizeof(tde_point2i));
    }
    const size_t sb = tde_rgbd_points_scratch_bytes(W, H);
    void *scratch = nullptr;
    check(tde_device_malloc(&scratch, sb), what);
    const int st = tde_rgbd_points_of_interest(dx, dy, W, H, Depth_Scale, scratch, sb,
                                               capacity ? static_cast<tde_point2i *>(Points_Of_Interest->device())
                                                        : nullptr,
                                               capacity, static_cast<uint32_t *>(Num_Of_Points->device()), nullptr);
    const int st2 = tde_device_synchronize();
    tde_device_free(scratch);
    check(st, what);
    check(st2, what);
    uint32_t cnt = 0;
    check(tde_memcpy(&cnt, Num_Of_Points->device(), sizeof(cnt), 1), what);
    num_of_points = (int)cnt;
}

namespace {

void fill_pairs(gpu_array_base *I_Prev, gpu_array_base *D_Prev, gpu_array_base *I_Curr, gpu_array_base *D_Curr,
                gpu_array_base *points, float Depth_Threshold, int npoints, const matrix_3f &R, const vector_3f &t,
                gpu_array_base *cprev, gpu_array_base *ccurr, gpu_array_base *diff, gpu_array_base *count,
                int *h_count, float *sigma_squared) {
    const char *what = "Fill_List_Of_Valid_Correspondence_RGBD";
    if (!I_Prev || npoints < 0) throw std::runtime_error(std::string(what) + ": bad arguments");
    const int W = (int)I_Prev->width(), H = (int)std::max(1u, I_Prev->height());
    const size_t n = (size_t)W * H;
    need_bytes(I_Prev, n, what);
    need_bytes(D_Prev, n * sizeof(float), what);
    need_bytes(I_Curr, n, what);
    need_bytes(D_Curr, n * sizeof(float), what);
    need_bytes(count, sizeof(uint32_t), what);
    const size_t np = (size_t)npoints;
    if (np) {
        need_bytes(points, np * sizeof(tde_point2i), what);
        need_bytes(cprev, np * sizeof(tde_point2i), what);
        need_bytes(ccurr, np * sizeof(tde_point2i), what);
        need_bytes(diff, np * sizeof(float), what);
    }
    float proj[12];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) proj[3 * r + c] = R.data[r].data[c];
    for (int k = 0; k < 3; ++k) proj[9 + k] = t.data[k];
    void *sum = nullptr;
    check(tde_device_malloc(&sum, sizeof(double)), what);
    const int st = np ? tde_rgbd_correspondences(
                            static_cast<const uint8_t *>(I_Prev->device()), static_cast<const float *>(D_Prev->device()),
                            static_cast<const uint8_t *>(I_Curr->device()), static_cast<const float *>(D_Curr->device()),
                            nullptr, nullptr, W, H, static_cast<const tde_point2i *>(points->device()), (uint32_t)np,
                            proj, Depth_Threshold, 35.f, 0.f, static_cast<tde_point2i *>(cprev->device()),
                            static_cast<tde_point2i *>(ccurr->device()), static_cast<float *>(diff->device()),
                            static_cast<uint32_t *>(count->device()), static_cast<double *>(sum), nullptr)
                      : tde_memset(count->device(), 0, sizeof(uint32_t));
    double s2 = 0.0;
    int st2 = tde_device_synchronize();
    if (st == TDE_OK && st2 == TDE_OK && np) st2 = tde_memcpy(&s2, sum, sizeof(s2), 1);
    tde_device_free(sum);
    check(st, what);
    check(st2, what);
    if (h_count) {
        uint32_t c = 0;
        check(tde_memcpy(&c, count->device(), sizeof(c), 1), what);
        *h_count = (int)c;
    }
    if (sigma_squared) *sigma_squared = (float)s2;
}

}  // namespace

void Fill_List_Of_Valid_Correspondence_RGBD(gpu_array_base *I_Prev, gpu_array_base *D_Prev, gpu_array_base *I_Curr,
                                            gpu_array_base *D_Curr, gpu_array_base *Points_Of_Interest,
                                            float Depth_Threshold, int Num_Of_Points_Of_Interest, matrix_3f R,
                                            vector_3f t, gpu_array_base *cprev, gpu_array_base *ccurr,
                                            gpu_array_base *diff, gpu_array_base *Num_Of_Correspondence,
                                            int &hNum_Of_Correspondence, float &sigma_squared, opencl_kernel *) {
    fill_pairs(I_Prev, D_Prev, I_Curr, D_Curr, Points_Of_Interest, Depth_Threshold, Num_Of_Points_Of_Interest, R, t,
               cprev, ccurr, diff, Num_Of_Correspondence, &hNum_Of_Correspondence, &sigma_squared);
}

void Fill_List_Of_Valid_Correspondence_RGBD(gpu_array_base *I_Prev, gpu_array_base *D_Prev, gpu_array_base *I_Curr,
                                            gpu_array_base *D_Curr, gpu_array_base *Points_Of_Interest,
                                            float Depth_Threshold, int Num_Of_Points_Of_Interest, matrix_3f R,
                                            vector_3f t, gpu_array_base *cprev, gpu_array_base *ccurr,
                                            gpu_array_base *diff, gpu_array_base *Num_Of_Correspondence, float,
                                            opencl_kernel *) {
    fill_pairs(I_Prev, D_Prev, I_Curr, D_Curr, Points_Of_Interest, Depth_Threshold, Num_Of_Points_Of_Interest, R, t,
               cprev, ccurr, diff, Num_Of_Correspondence, nullptr, nullptr);
}

bool Estimate_Isometry_By_RGBD(vector<gpu_array_base *> &I_Prev, vector<gpu_array_base *> &D_Prev,
                               vector<gpu_array_base *> &I_Curr, vector<gpu_array_base *> &D_Curr,
                               vector<gpu_array_base *> &DI_dx, vector<gpu_array_base *> &DI_dy, intrinsics Intr,
                               float RGBD_Depth_Threshold, int levels, matrix_3f Init_R, vector_3f Init_t,
                               matrix_3f &Estimated_Rotation, vector_3f &Estimated_Translation, kernel_manager *) {
    const char *what = "Estimate_Isometry_By_RGBD";
    if (levels < 1 || levels > TDE_RGBD_MAX_LEVELS)
        throw std::runtime_error(std::string(what) + ": 1 to 4 pyramid levels");
    if ((int)I_Prev.size() < levels || (int)D_Prev.size() < levels || (int)I_Curr.size() < levels ||
        (int)D_Curr.size() < levels || (int)DI_dx.size() < levels || (int)DI_dy.size() < levels)
        throw std::runtime_error(std::string(what) + ": fewer buffers than levels");
    tde_rgbd_frame prev = {}, curr = {};
    for (int l = 0; l < levels; ++l) {
        const size_t n = (size_t)(Intr.cols >> l) * (Intr.rows >> l);
        need_bytes(I_Prev[l], n, what);
        need_bytes(D_Prev[l], n * sizeof(float), what);
        need_bytes(I_Curr[l], n, what);
        need_bytes(D_Curr[l], n * sizeof(float), what);
        prev.intensity[l] = static_cast<const uint8_t *>(I_Prev[l]->device());
        prev.depth[l] = static_cast<const float *>(D_Prev[l]->device());
        curr.intensity[l] = static_cast<const uint8_t *>(I_Curr[l]->device());
        curr.depth[l] = static_cast<const float *>(D_Curr[l]->device());
        curr.dx[l] = deriv(DI_dx[l], n, what);
        curr.dy[l] = deriv(DI_dy[l], n, what);
    }
    tde_rgbd_params params;
    tde_rgbd_default_params(&params);
    params.levels = levels;
    params.max_depth_diff = RGBD_Depth_Threshold;
    double init[12], pose[12];
    to_pose(Init_R, Init_t, init);
    const size_t sb = tde_rgbd_odometry_scratch_bytes(Intr.cols, Intr.rows);
    void *scratch = nullptr, *dpose = nullptr;
    check(tde_device_malloc(&scratch, sb), what);
    if (tde_device_malloc(&dpose, 16 * sizeof(double)) != TDE_OK) {
        tde_device_free(scratch);
        check(TDE_ERR_OOM, what);
    }
    int *dstatus = reinterpret_cast<int *>(static_cast<double *>(dpose) + 12);
    int st = tde_rgbd_odometry(&prev, &curr, I(Intr), &params, init, static_cast<double *>(dpose), dstatus, scratch,
                               sb, nullptr);
    int status = 0;
    if (st == TDE_OK) st = tde_device_synchronize();
    if (st == TDE_OK) st = tde_memcpy(pose, dpose, sizeof(pose), 1);
    if (st == TDE_OK) st = tde_memcpy(&status, dstatus, sizeof(status), 1);
    tde_device_free(scratch);
    tde_device_free(dpose);
    check(st, what);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Estimated_Rotation.data[r].data[c] = (float)pose[3 * r + c];
    for (int k = 0; k < 3; ++k) Estimated_Translation.data[k] = (float)pose[9 + k];
    return (status & 2) != 0;
}
