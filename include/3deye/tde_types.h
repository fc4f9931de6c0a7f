/*
 * tde_types.h -- the reference's shared POD types and enums, byte-identical
 * (static_assert-pinned) to common/inc/elementary_points.h,
 * common/inc/types/{intrinsics,round_buffer,base_points,dim3}.h and
 * common/inc/enums.h, so code written against 3deye's C++ API compiles
 * unchanged.  The C-ABI twins live in ../tde_capi.h.
 */
#ifndef TDE_3DEYE_TYPES_H
#define TDE_3DEYE_TYPES_H

#include <cstddef>
#include <cstdint>
#include <iostream>

#include "../tde_capi.h"

/* ---- elementary points: common/inc/elementary_points.h:32-87 ---------- */
typedef struct point_3f { union { float data[3]; struct { float x, y, z; }; }; } point_3f;
typedef point_3f vector_3f;
typedef struct point_3i { union { int data[3]; struct { int x, y, z; }; }; } point_3i;
/* `us` is unsigned int in the reference (elementary_points.h:34) */
typedef struct point_3us { union { unsigned int data[3]; struct { unsigned int x, y, z; }; }; } point_3us;
typedef struct point_2i { union { int data[2]; struct { int x, y; }; }; } point_2i;
typedef struct point_2us { union { unsigned int data[2]; struct { unsigned int x, y; }; }; } point_2us;
typedef struct matrix_3f { point_3f data[3]; } matrix_3f;

inline point_3f make_point_3f(float x, float y, float z) { point_3f p; p.x = x; p.y = y; p.z = z; return p; }
inline point_3i make_point_3i(int x, int y, int z) { point_3i p; p.x = x; p.y = y; p.z = z; return p; }

/* ---- dim3: common/inc/types/dim3.h:12-38 ------------------------------- */
struct dim3 {
    union {
        size_t data[3];
        struct { size_t x, y, z; };
        struct { size_t width, height, depth; };
    };
    dim3(size_t nx = 1, size_t ny = 1, size_t nz = 1) : x(nx), y(ny), z(nz) {}
};

/* ---- intrinsics: common/inc/types/intrinsics.h:8-26 -------------------- */
typedef struct intrinsics {
    float fx, fy, cx, cy;
    int cols, rows;
    /* pyramid level: fx/2^l, cx/2^l, cols>>l (common/src/intrinsics.cpp:7-18) */
    intrinsics operator()(int level_index) const {
        int div = 1 << level_index;
        intrinsics r = {fx / div, fy / div, cx / div, cy / div, cols >> level_index, rows >> level_index};
        return r;
    }
} intrinsics;

/* ---- enums: common/inc/enums.h:8-77 ------------------------------------ */
enum Types_Of_Scan { INCLUSIVE, EXCLUSIVE };
enum size_dimensions { WIDTH, HEIGHT, DEPTH };
enum gpu_mem_type { LOCAL, GLOBAL, PRIVATE, CONSTANT, IMAGE };
enum gpu_transfer_type { TO_NONE, TO_CPU, TO_GPU, TO_GPU_AND_BACK, IN_GPU_USE_ONLY };
enum gpu_data_type { TYPE_NONE, BUFFER_1D, IMAGE_2D, CONSTANT_BUFFER };
enum profiling_level { DISABLE_PROFILING, ENABLE_PROFILING };

/* ---- round_buffer: common/inc/types/round_buffer.h:25-63 --------------- */
typedef struct round_buffer {
    int start_index;
    int end_index;
    int buffer_length;
    point_3i origin_GRID;
    point_3f origin_GRID_global;
    point_3f origin_metric;
    point_3f volume_size;
    point_3i voxels_size;

    /* constructors of common/src/round_buffer.cpp:5-74 */
    round_buffer();
    round_buffer(const dim3 &dimensions);
    round_buffer(size_t width, size_t height, size_t depth);
    round_buffer(point_3i voxels_size, point_3f metric_size);
    void set_default_values();
    void set_voxels_size(size_t new_width, size_t new_height, size_t new_depth);
    void set_memory_index();
    const tde_round_buffer *c_abi() const { return reinterpret_cast<const tde_round_buffer *>(this); }
} round_buffer;

/* ---- base points: common/inc/types/base_points.h:17-214 ---------------- */
typedef struct Depth { unsigned short value; } Depth;
typedef struct Tsdf { short value; short weight; } Tsdf;
typedef struct Color { unsigned char r, g, b, w; } Color;
typedef struct XYZ { float x, y, z; } XYZ;
typedef XYZ NXYZ;
typedef struct XYZI { union { float value[4]; struct { float x, y, z, w; }; }; } XYZI;
typedef XYZI NXYZI;

/* Point<T>: the C++ form of BASE_TYPE Point (base_point_template.h:49-56):
 * a single `data` member, so arrays of Point<T> have T's layout. */
template <class T> class Point {
  public:
    T data;
};
typedef Point<Depth> Point_Depth;
typedef Point<Tsdf> Point_Tsdf;
typedef Point<Color> Point_Color;
typedef Point<XYZ> Point_XYZ;
typedef Point<NXYZ> Point_NXYZ;
typedef Point<XYZI> Point_XYZI;

/* ---- light_source: common/inc/types/light_source.h:4-8 ----------------- */
typedef struct light_source {
    point_3f pos;
    int number;
} light_source;

/* ---- constants: common/inc/common_defines.h / constants.h -------------- */
#ifndef DEFAULT_STRIDE
#define DEFAULT_STRIDE 256
#define MAX_DEPTH_VALUE 32767
#define MAX_TSDF_WEIGHT (1 << 7)
#define DEFAULT_NUM_OF_ICP_PYRAMID_LEVELS 3
#define DEFAULT_SIGMA_COLOR 30.f
#define DEFAULT_SIGMA_SPACE 4.5f
#define DEFAULT_TRUNCATION_DISTANCE 0.03f
#define DEFAULT_DISTANCE_THRESHOLD 0.1f
#define DEFAULT_VOLUME_SHIFTING_THRESHOLD 1.5f
#define DEFAULT_ANGLE_THRESHOLD 0.34202014332566873f /* sin(20 deg) */
#define DIVUP(TOTAL, DIVISOR) (((TOTAL) + (DIVISOR)-1) / DIVISOR)
#endif

static_assert(sizeof(point_3f) == 12 && sizeof(point_3i) == 12 && sizeof(matrix_3f) == 36, "point layouts");
static_assert(sizeof(point_2us) == 8, "point_2us holds two unsigned ints");
static_assert(sizeof(intrinsics) == 24 && sizeof(round_buffer) == 72, "intrinsics / round_buffer");
static_assert(sizeof(Point_Tsdf) == 4 && sizeof(Point_Color) == 4 && sizeof(Point_XYZ) == 12 &&
                  sizeof(Point_XYZI) == 16 && sizeof(Point_Depth) == 2,
              "point record layouts");
static_assert(sizeof(round_buffer) == sizeof(tde_round_buffer), "round_buffer is the C-ABI record");
static_assert(sizeof(light_source) == sizeof(tde_light_source), "light_source is the C-ABI record");

#endif
