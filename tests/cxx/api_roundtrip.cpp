// A caller written against the reference's C++ API (common/inc/opencl_wrappers.h
// and friends), built only with -I include/3deye and linked to
// lib3deye_gb300.so.  Reads a depth frame and a pose from argv[1]/input.bin,
// runs Integrate_Tsdf_Data -> Raycast -> Resize maps -> Extract_Slice ->
// Extract_Tsdf_Volume -> Extract_Color_Volume -> Extract_Color_Slice -> Generate_Image ->
// Clean_Tsdf_Slice -> Estimate_Combined, and writes every result to
// argv[1]/output.bin for the Python test to compare with the CPU oracle.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <kernel_manager.h>
#include <opencl_wrappers.h>

template <class T> static void rd(FILE *f, T *p, size_t n) {
    if (fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
template <class T> static void wr(FILE *f, const T *p, size_t n) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    std::string dir = argv[1];
    FILE *in = fopen((dir + "/input.bin").c_str(), "rb");
    if (!in) return 3;
    int hdr[5];  // cols rows voxels use_color ... format
    rd(in, hdr, 5);
    const int W = hdr[0], H = hdr[1], N = hdr[2], fmt = hdr[4];
    float f[8];  // fx fy cx cy volume trunc dist angle
    rd(in, f, 8);
    float pose[12], pose2[12];
    rd(in, pose, 12);
    rd(in, pose2, 12);
    std::vector<unsigned short> depth((size_t)W * H), depth2((size_t)W * H);
    rd(in, depth.data(), depth.size());
    rd(in, depth2.data(), depth2.size());
    int bounds[6];
    rd(in, bounds, 6);
    fclose(in);

    Set_Tsdf_Storage_Format(fmt);
    vector<string> names = {"scale_depth.cl", "integrate_tsdf_volume.cl", "raycast.cl", "resize_vertex_map.cl",
                            "resize_normal_map.cl", "estimate_combined.cl", "transform_estimation.cl",
                            "compute_bilateral_filtering.cl", "compute_vertex_map.cl", "compute_normal_map_eigen.cl",
                            "clean_tsdf_slice.cl", "scan_the_whole_array.cl", "extract_tsdf_cloud.cl",
                            "extract_colors.cl", "generate_image.cl", "scan_slice_of_color_volume.cl",
                            "extract_color_slice_as_cloud.cl"};
    kernel_manager gm("ignored/path", names);
    bool threw = false;
    try { gm.Get_Kernel("no_such_kernel.cl"); } catch (const std::exception &) { threw = true; }
    if (!threw) { fprintf(stderr, "unknown kernel accepted\n"); return 4; }

    intrinsics intr = {f[0], f[1], f[2], f[3], W, H};
    point_3i vox = make_point_3i(N, N, N);
    point_3f metric = make_point_3f(f[4], f[4], f[4]);
    round_buffer rb(vox, metric);
    point_3f cell = make_point_3f(f[4] / N, f[4] / N, f[4] / N);
    float trunc = f[5];

    matrix_3f R, Rinv, R2;
    vector_3f t, t2;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            R.data[r].data[c] = pose[3 * r + c];
            Rinv.data[r].data[c] = pose[3 * c + r];
            R2.data[r].data[c] = pose2[3 * r + c];
        }
    t = make_point_3f(pose[9], pose[10], pose[11]);
    t2 = make_point_3f(pose2[9], pose2[10], pose2[11]);

    size_t vbytes = tde_tsdf_volume_bytes(fmt, rb.c_abi());
    gpu_array<unsigned char> vol(dim3((unsigned)vbytes), true);
    if (tde_tsdf_init(vol.device(), fmt, rb.c_abi(), nullptr) != 0) return 5;
    gpu_array<Point_Depth> gdepth((Point_Depth *)depth.data(), dim3(W, H), TO_GPU);
    gpu_array<float> gscaled(dim3(W, H), true);
    Integrate_Tsdf_Data(&gdepth, &gscaled, &vol, intr, Rinv, t, trunc, cell, &rb, &gm, 0);

    gpu_array<Point_XYZ> vmap(dim3(W, H)), nmap(dim3(W, H));
    Raycast(&vol, &vmap, &nmap, &rb, t, R, trunc, intr, cell, gm.Get_Kernel("raycast"));
    gpu_array<Point_XYZ> vmap1(dim3(W / 2, H / 2)), nmap1(dim3(W / 2, H / 2));
    Resize_Vertex_Map(&vmap, &vmap1, intr, gm.Get_Kernel("resize_vertex_map"));
    Resize_Normal_Map(&nmap, &nmap1, intr, gm.Get_Kernel("resize_normal_map"));

    // current frame maps from the second depth frame
    gpu_array<Point_Depth> gdepth2((Point_Depth *)depth2.data(), dim3(W, H), TO_GPU);
    gpu_array<Point_Depth> gfilt(dim3(W, H));
    Apply_Billateral_Filtration(&gdepth2, intr, 4000.f, gm.Get_Kernel("compute_bilateral_filtering"), &gfilt);
    vector<gpu_array_base *> depths = {&gfilt}, verts, norms;
    gpu_array<Point_XYZ> vc(dim3(W, H)), nc(dim3(W, H));
    verts.push_back(&vc);
    norms.push_back(&nc);
    Create_Vertex_Maps(depths, verts, intr, 1, &gm);
    Create_Normal_Maps(verts, norms, intr, 1, &gm);

    gpu_array<float> gbuf((unsigned)tde_estimate_combined_gbuf_floats(W, H));
    gpu_array<float> gmbuf(27u);
    double A[36], b[6];
    float dist = f[6], angle = f[7];
    Estimate_Combined(R2, t2, &vc, &nc, Rinv, t, intr, &vmap, &nmap, dist, angle, &gbuf, &gmbuf, A, b, &gm);

    point_3i mn = make_point_3i(bounds[0], bounds[1], bounds[2]);
    point_3i mx = make_point_3i(bounds[3], bounds[4], bounds[5]);
    matrix<Point_XYZI> cloud;
    Extract_Tsdf_Slice(mn, mx, &rb, cell, &vol, &gm, cloud);
    // whole-model export, colour lookup and the shaded image, before cleaning
    matrix<Point_XYZI> whole;
    Extract_Tsdf_Volume(&rb, cell, &vol, &gm, whole);
    const size_t nvox = (size_t)N * N * N;
    std::vector<Point_Color> hcol(nvox);
    for (size_t i = 0; i < nvox; ++i) {
        hcol[i].data.r = (unsigned char)(i * 7);
        hcol[i].data.g = (unsigned char)(i * 13);
        hcol[i].data.b = (unsigned char)(i * 29);
        hcol[i].data.w = (unsigned char)(i % 5 == 0 ? 0 : 200);
    }
    gpu_array<Point_Color> gcol(hcol.data(), dim3((unsigned)nvox), TO_GPU);
    matrix<Point_Color> wcols(whole.Get_Num_Of_Elem());
    Extract_Color_Volume(&gcol, &rb, whole, cell, gm.Get_Kernel("extract_colors"), wcols);
    // colour slab of the same bounds, appended to a cloud that holds one entry
    matrix<Point_Color> cslab(1);
    cslab.data[0].data.r = 1; cslab.data[0].data.g = 2; cslab.data[0].data.b = 3; cslab.data[0].data.w = 4;
    Extract_Color_Slice(mn, mx, &rb, &gcol, &gm, cslab);
    light_source light;
    light.pos = t;
    light.number = 1;
    gpu_array<unsigned char> img(dim3((unsigned)(W * H * 3)));
    Generate_Image(&vmap, &nmap, intr, light, &img, gm.Get_Kernel("generate_image"));
    std::vector<unsigned char> himg((size_t)W * H * 3);
    img.memcpy_to_host(himg.data());
    Clean_Tsdf_Slice(mn, mx, &rb, &vol, gm.Get_Kernel("clean_tsdf_slice"));

    std::vector<float> hv((size_t)W * H * 3), hn((size_t)W * H * 3), hv1((size_t)W * H * 3 / 4), hn1(hv1.size());
    vmap.memcpy_to_host(hv.data());
    nmap.memcpy_to_host(hn.data());
    vmap1.memcpy_to_host(hv1.data());
    nmap1.memcpy_to_host(hn1.data());
    std::vector<unsigned char> hvol(vbytes);
    vol.memcpy_to_host(hvol.data());
    std::vector<float> hvc((size_t)W * H * 3), hnc((size_t)W * H * 3);
    vc.memcpy_to_host(hvc.data());
    nc.memcpy_to_host(hnc.data());

    FILE *out = fopen((dir + "/output.bin").c_str(), "wb");
    unsigned n = cloud.Get_Num_Of_Elem();
    wr(out, hv.data(), hv.size());
    wr(out, hn.data(), hn.size());
    wr(out, hv1.data(), hv1.size());
    wr(out, hn1.data(), hn1.size());
    wr(out, A, 36);
    wr(out, b, 6);
    wr(out, &n, 1);
    if (n) wr(out, (const float *)cloud.data, (size_t)n * 4);
    wr(out, hvol.data(), hvol.size());
    wr(out, hvc.data(), hvc.size());
    wr(out, hnc.data(), hnc.size());
    unsigned nw = whole.Get_Num_Of_Elem();
    wr(out, &nw, 1);
    if (nw) wr(out, (const float *)whole.data, (size_t)nw * 4);
    if (nw) wr(out, (const unsigned char *)wcols.data, (size_t)nw * 4);
    wr(out, himg.data(), himg.size());
    unsigned nc_slab = cslab.Get_Num_Of_Elem();
    wr(out, &nc_slab, 1);
    wr(out, (const unsigned char *)cslab.data, (size_t)nc_slab * 4);
    fclose(out);
    printf("ok points=%u\n", n);
    return 0;
}
