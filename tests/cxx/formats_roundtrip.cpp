// Text formats of include/3deye/ (header-only: no library, no GPU).
// argv[1] = a directory holding input.bin:
//   int32 n_poses, n_points; float R[n_poses][9], t[n_poses][3];
//   float points[n_points][4]; uint8 colors[n_points][4]
// Writes trajectory.txt, cloud.txt, colors.txt there with the C++ writers,
// reads both clouds back with Fill_From_File and writes readback.bin
// (int32 status pair, counts, then the points and colours read); with two
// more arguments, reads those text clouds into golden.bin likewise.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "matrix.h"
#include "string_utils.h"

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    FILE *f = std::fopen((dir + "/input.bin").c_str(), "rb");
    if (!f) return 3;
    int32_t np = 0, nq = 0;
    if (std::fread(&np, 4, 1, f) != 1 || std::fread(&nq, 4, 1, f) != 1) return 4;
    std::vector<matrix_3f> R(np);
    std::vector<vector_3f> t(np);
    for (int i = 0; i < np; ++i)
        if (std::fread(&R[i], sizeof(float), 9, f) != 9) return 5;
    for (int i = 0; i < np; ++i)
        if (std::fread(&t[i], sizeof(float), 3, f) != 3) return 5;
    matrix<Point_XYZI> cloud(nq);
    matrix<Point_Color> colors(nq);
    if (nq && std::fread(cloud.data, sizeof(Point_XYZI), nq, f) != (size_t)nq) return 6;
    if (nq && std::fread(colors.data, sizeof(Point_Color), nq, f) != (size_t)nq) return 6;
    std::fclose(f);

    write_isometry_to_file((dir + "/trajectory.txt").c_str(), R.data(), t.data(), R.size());
    cloud.Save_To_File(dir + "/cloud.txt");
    colors.Save_To_File(dir + "/colors.txt");

    matrix<Point_XYZI> cloud_in;
    matrix<Point_Color> colors_in;
    int32_t st[2] = {cloud_in.Fill_From_File(dir + "/cloud.txt"), colors_in.Fill_From_File(dir + "/colors.txt")};
    FILE *o = std::fopen((dir + "/readback.bin").c_str(), "wb");
    if (!o) return 7;
    std::fwrite(st, 4, 2, o);
    int32_t n_in[2] = {(int32_t)cloud_in.Get_Num_Of_Elem(), (int32_t)colors_in.Get_Num_Of_Elem()};
    std::fwrite(n_in, 4, 2, o);
    if (n_in[0]) std::fwrite(cloud_in.data, sizeof(Point_XYZI), n_in[0], o);
    if (n_in[1]) std::fwrite(colors_in.data, sizeof(Point_Color), n_in[1], o);
    std::fclose(o);
    // a round buffer record, written and read back into rb.bin
    {
        // the record's fields only (round_buffer's constructors live in the library)
        alignas(round_buffer) unsigned char store[2][sizeof(round_buffer)] = {};
        round_buffer &rb = *reinterpret_cast<round_buffer *>(store[0]);
        round_buffer &back = *reinterpret_cast<round_buffer *>(store[1]);
        rb.origin_GRID = make_point_3i(3, 500, 7);
        rb.origin_GRID_global = make_point_3f(3.f, -12.f, 7.f);
        rb.origin_metric = make_point_3f(0.0175781f, -0.0703125f, 0.0410156f);
        rb.volume_size = make_point_3f(3.f, 3.f, 3.f);
        rb.voxels_size = make_point_3i(512, 512, 512);
        rb.start_index = 0;
        rb.buffer_length = 512 * 512 * 512;
        {
            std::ofstream f((dir + "/rb.txt").c_str());
            f << rb;
        }
        std::ifstream f((dir + "/rb.txt").c_str());
        f >> back;
        FILE *b = std::fopen((dir + "/rb.bin").c_str(), "wb");
        if (!b) return 9;
        int32_t ok = f ? 1 : 0;
        std::fwrite(&ok, 4, 1, b);
        std::fwrite(&back, sizeof(back), 1, b);
        std::fclose(b);
    }
    // argv[2], argv[3] (optional): a point cloud and a colour cloud in the
    // reference's text format, read with Fill_From_File into golden.bin
    if (argc >= 4) {
        matrix<Point_XYZI> gp;
        matrix<Point_Color> gc;
        int32_t gs[2] = {gp.Fill_From_File(argv[2]), gc.Fill_From_File(argv[3])};
        FILE *g = std::fopen((dir + "/golden.bin").c_str(), "wb");
        if (!g) return 8;
        int32_t gn[2] = {(int32_t)gp.Get_Num_Of_Elem(), (int32_t)gc.Get_Num_Of_Elem()};
        std::fwrite(gs, 4, 2, g);
        std::fwrite(gn, 4, 2, g);
        if (gn[0]) std::fwrite(gp.data, sizeof(Point_XYZI), gn[0], g);
        if (gn[1]) std::fwrite(gc.data, sizeof(Point_Color), gn[1], g);
        std::fclose(g);
    }
    return 0;
}
