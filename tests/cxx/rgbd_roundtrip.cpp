// A caller of the reference's RGB-D odometry API (common/inc/opencl_wrappers.h:
// 99-103, 227-292), built only with -I include/3deye and linked to
// lib3deye_gb300.so.  Reads two depth + RGB frames and the camera from
// argv[1]/rgbd_in.bin, runs Prepare_Data_For_RGBD ->
// Generate_Intensity_And_Depth_Pyramid -> Create_Intensity_Derivatives ->
// Accumulate_Points_Of_Interest_For_RGBD -> Fill_List_Of_Valid_Correspondence_RGBD
// -> Estimate_Isometry_By_RGBD and writes the results to argv[1]/rgbd_out.bin
// for the Python test to compare with the CPU oracle.
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
    FILE *in = fopen((dir + "/rgbd_in.bin").c_str(), "rb");
    if (!in) return 3;
    int hdr[3];  // cols rows levels
    rd(in, hdr, 3);
    const int W = hdr[0], H = hdr[1], L = hdr[2];
    float f[5];  // fx fy cx cy depth threshold
    rd(in, f, 5);
    const size_t n = (size_t)W * H;
    std::vector<unsigned short> d0(n), d1(n);
    std::vector<unsigned char> c0(3 * n), c1(3 * n);
    rd(in, d0.data(), n);
    rd(in, c0.data(), 3 * n);
    rd(in, d1.data(), n);
    rd(in, c1.data(), 3 * n);
    fclose(in);

    vector<string> names = {"prepare_initial_frames_rgbd.cl", "generate_intensity_and_depth_pyramid.cl",
                            "create_intensity_derivatives.cl", "scan_for_interest_point.cl",
                            "extract_interest_points.cl", "scan_list_of_valid_correspondence.cl",
                            "compute_least_squares_equation.cl"};
    kernel_manager gm("ignored/path", names);
    intrinsics intr = {f[0], f[1], f[2], f[3], W, H};

    gpu_array<unsigned short> gd0(d0.data(), dim3(W, H), TO_GPU), gd1(d1.data(), dim3(W, H), TO_GPU);
    gpu_array<unsigned char> gc0(c0.data(), dim3(3 * W, H), TO_GPU), gc1(c1.data(), dim3(3 * W, H), TO_GPU);
    vector<gpu_array_base *> I0, D0, I1, D1, DX, DY;
    for (int l = 0; l < L; ++l) {
        dim3 s(W >> l, H >> l);
        I0.push_back(new gpu_array<unsigned char>(s));
        D0.push_back(new gpu_array<float>(s));
        I1.push_back(new gpu_array<unsigned char>(s));
        D1.push_back(new gpu_array<float>(s));
        DX.push_back(new gpu_array<short>(s));
        DY.push_back(new gpu_array<short>(s));
    }
    Prepare_Data_For_RGBD(&gd0, &gc0, I0[0], D0[0], gm.Get_Kernel("prepare_initial_frames_rgbd.cl"));
    Prepare_Data_For_RGBD(&gd1, &gc1, I1[0], D1[0], gm.Get_Kernel("prepare_initial_frames_rgbd.cl"));
    Generate_Intensity_And_Depth_Pyramid(I0, D0, intr, L, &gm);
    Generate_Intensity_And_Depth_Pyramid(I1, D1, intr, L, &gm);
    Create_Intensity_Derivatives(I1, DX, DY, intr, L, &gm);

    FILE *out = fopen((dir + "/rgbd_out.bin").c_str(), "wb");
    if (!out) return 4;
    for (int l = 0; l < L; ++l) {  // previous frame's pyramid, current frame's derivatives
        const size_t m = (size_t)(W >> l) * (H >> l);
        std::vector<unsigned char> i8(m);
        std::vector<float> dm(m);
        std::vector<short> gx(m), gy(m);
        I0[l]->memcpy_to_host(i8.data());
        D0[l]->memcpy_to_host(dm.data());
        DX[l]->memcpy_to_host(gx.data());
        DY[l]->memcpy_to_host(gy.data());
        wr(out, i8.data(), m);
        wr(out, dm.data(), m);
        wr(out, gx.data(), m);
        wr(out, gy.data(), m);
    }

    // points of interest of the current frame at level 0, then their pairs
    // at the identity pose (R' = I, t' = 0)
    const float scale = (10.f / 0.125f) * (10.f / 0.125f);
    gpu_array<point_2i> pts(dim3(W, H));
    gpu_array<int> npts(1u), ncorr(1u);
    int num_points = -1;
    Accumulate_Points_Of_Interest_For_RGBD(DX[0], DY[0], scale, &pts, &npts, num_points, &gm);
    std::vector<point_2i> hp(n);
    pts.memcpy_to_host(hp.data());
    wr(out, &num_points, 1);
    wr(out, hp.data(), (size_t)num_points);

    matrix_3f Rid = {{{{1.f, 0.f, 0.f}}, {{0.f, 1.f, 0.f}}, {{0.f, 0.f, 1.f}}}};
    vector_3f tz = {{0.f, 0.f, 0.f}};
    gpu_array<point_2i> cp(dim3(W, H)), cc(dim3(W, H));
    gpu_array<float> diff(dim3(W, H));
    int num_corr = -1;
    float sigma2 = -1.f;
    Fill_List_Of_Valid_Correspondence_RGBD(I0[0], D0[0], I1[0], D1[0], &pts, f[4], num_points, Rid, tz, &cp, &cc,
                                           &diff, &ncorr, num_corr, sigma2,
                                           gm.Get_Kernel("scan_list_of_valid_correspondence.cl"));
    std::vector<float> hd(n);
    diff.memcpy_to_host(hd.data());
    wr(out, &num_corr, 1);
    wr(out, &sigma2, 1);
    wr(out, hd.data(), (size_t)num_points);

    matrix_3f R;
    vector_3f t;
    const bool ok = Estimate_Isometry_By_RGBD(I0, D0, I1, D1, DX, DY, intr, f[4], L, Rid, tz, R, t, &gm);
    const int okv = ok ? 1 : 0;
    wr(out, &okv, 1);
    for (int r = 0; r < 3; ++r) wr(out, R.data[r].data, 3);
    wr(out, t.data, 3);
    fclose(out);

    // derivatives declared as the reference does (unsigned char) are refused
    vector<gpu_array_base *> DX8, DY8;
    for (int l = 0; l < L; ++l) {
        DX8.push_back(new gpu_array<unsigned char>(dim3(W >> l, H >> l)));
        DY8.push_back(new gpu_array<unsigned char>(dim3(W >> l, H >> l)));
    }
    bool threw = false;
    try {
        Create_Intensity_Derivatives(I1, DX8, DY8, intr, L, &gm);
    } catch (const std::exception &) {
        threw = true;
    }
    for (int l = 0; l < L; ++l) {
        delete DX8[l];
        delete DY8[l];
    }
    if (!threw) {
        fprintf(stderr, "unsigned char derivatives accepted\n");
        return 5;
    }
    for (int l = 0; l < L; ++l) {
        delete I0[l]; delete D0[l]; delete I1[l]; delete D1[l]; delete DX[l]; delete DY[l];
    }
    return 0;
}
