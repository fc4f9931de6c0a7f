/*
 * ref_launch.c -- NDRange launchers for the reference's OpenCL kernels compiled
 * as C through ref_shim.h.  TEST INFRASTRUCTURE ONLY: built by
 * oracle/build_ref.sh into oracle/_ref/ref_<kernel>.so and loaded only by
 * tests/golden/make_golden.py.
 *
 * One kernel per translation unit: the build passes -DREF_<KERNEL> and
 * -DREF_CL_PATH="<path to the .cl file>".  Kernels that call barrier() run each
 * work-group as a set of ucontext fibers that are resumed round-robin, so a
 * barrier is a point every fiber of the group reaches before any continues.
 */
#define _GNU_SOURCE
#include "ref_shim.h"
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

_Thread_local tde_ref_workitem *tde_ref_wi;
_Thread_local float *tde_ref_capture_rte;

#include REF_CL_PATH

#define TDE_REF_EXPORT __attribute__((visibility("default")))

/* ---------------------------------------------------------------------------
 * Plain loop over a 2-D NDRange (kernels without barriers).
 * ------------------------------------------------------------------------- */
typedef void (*tde_ref_item_fn)(void);

static void tde_ref_run_plain(tde_ref_item_fn fn, size_t gx, size_t gy, size_t lx, size_t ly) {
    tde_ref_workitem wi;
    memset(&wi, 0, sizeof(wi));
    wi.gsz[0] = gx; wi.gsz[1] = gy; wi.gsz[2] = 1;
    wi.lsz[0] = lx; wi.lsz[1] = ly; wi.lsz[2] = 1;
    tde_ref_wi = &wi;
    for (size_t y = 0; y < gy; ++y)
        for (size_t x = 0; x < gx; ++x) {
            wi.gid[0] = x; wi.gid[1] = y;
            wi.lid[0] = x % lx; wi.lid[1] = y % ly;
            wi.grp[0] = x / lx; wi.grp[1] = y / ly;
            fn();
        }
    tde_ref_wi = NULL;
}

/* ---------------------------------------------------------------------------
 * Fiber scheduler for kernels with barrier().
 * ------------------------------------------------------------------------- */
#define TDE_REF_MAX_GROUP 1024
#define TDE_REF_STACK (64 * 1024)

static ucontext_t tde_ref_sched_ctx;
static ucontext_t tde_ref_item_ctx[TDE_REF_MAX_GROUP];
static tde_ref_workitem tde_ref_items[TDE_REF_MAX_GROUP];
static int tde_ref_done[TDE_REF_MAX_GROUP];
static int tde_ref_cur;
static tde_ref_item_fn tde_ref_cur_fn;
static char *tde_ref_stacks;

void tde_ref_barrier(void) {
    swapcontext(&tde_ref_item_ctx[tde_ref_cur], &tde_ref_sched_ctx);
}

static void tde_ref_fiber_entry(void) {
    tde_ref_cur_fn();
    tde_ref_done[tde_ref_cur] = 1;
    /* returning resumes uc_link == scheduler */
}

static int tde_ref_run_fibers(tde_ref_item_fn fn, size_t gx, size_t gy, size_t lx, size_t ly) {
    size_t n = lx * ly;
    if (n > TDE_REF_MAX_GROUP || gx % lx || gy % ly) return -1;
    if (!tde_ref_stacks) tde_ref_stacks = (char *)malloc((size_t)TDE_REF_MAX_GROUP * TDE_REF_STACK);
    if (!tde_ref_stacks) return -2;
    tde_ref_cur_fn = fn;
    for (size_t by = 0; by < gy / ly; ++by)
        for (size_t bx = 0; bx < gx / lx; ++bx) {
            for (size_t i = 0; i < n; ++i) {
                tde_ref_workitem *w = &tde_ref_items[i];
                memset(w, 0, sizeof(*w));
                w->gsz[0] = gx; w->gsz[1] = gy; w->gsz[2] = 1;
                w->lsz[0] = lx; w->lsz[1] = ly; w->lsz[2] = 1;
                w->lid[0] = i % lx; w->lid[1] = i / lx;
                w->grp[0] = bx; w->grp[1] = by;
                w->gid[0] = bx * lx + w->lid[0];
                w->gid[1] = by * ly + w->lid[1];
                tde_ref_done[i] = 0;
                getcontext(&tde_ref_item_ctx[i]);
                tde_ref_item_ctx[i].uc_stack.ss_sp = tde_ref_stacks + i * TDE_REF_STACK;
                tde_ref_item_ctx[i].uc_stack.ss_size = TDE_REF_STACK;
                tde_ref_item_ctx[i].uc_link = &tde_ref_sched_ctx;
                makecontext(&tde_ref_item_ctx[i], tde_ref_fiber_entry, 0);
            }
            for (;;) {
                int alive = 0;
                for (size_t i = 0; i < n; ++i) {
                    if (tde_ref_done[i]) continue;
                    tde_ref_cur = (int)i;
                    tde_ref_wi = &tde_ref_items[i];
                    swapcontext(&tde_ref_sched_ctx, &tde_ref_item_ctx[i]);
                    if (!tde_ref_done[i]) alive++;
                }
                if (!alive) break;
            }
        }
    tde_ref_wi = NULL;
    return 0;
}

/* ===========================================================================
 * Per-kernel entry points
 * ========================================================================= */
#if defined(REF_RAYCAST)
static struct {
    Point_Tsdf *vol; Point_XYZ *vmap; Point_NXYZ *nmap;
    point_3f t; matrix_3f R; float trunc; intrinsics intr; round_buffer rb; point_3f cell;
} A;
static void item(void) { raycast(A.vol, A.vmap, A.nmap, A.t, A.R, A.trunc, A.intr, A.rb, A.cell); }

TDE_REF_EXPORT int ref_raycast(void *vol, void *vmap, void *nmap, const float *t, const float *R,
                               float trunc, const void *intr, const void *rb, const float *cell) {
    A.vol = (Point_Tsdf *)vol; A.vmap = (Point_XYZ *)vmap; A.nmap = (Point_NXYZ *)nmap;
    memcpy(&A.t, t, sizeof(A.t)); memcpy(&A.R, R, sizeof(A.R)); A.trunc = trunc;
    memcpy(&A.intr, intr, sizeof(A.intr)); memcpy(&A.rb, rb, sizeof(A.rb));
    memcpy(&A.cell, cell, sizeof(A.cell));
    tde_ref_run_plain(item, (size_t)A.intr.cols, (size_t)A.intr.rows, 32, 8);
    return 0;
}
TDE_REF_EXPORT int ref_sizes(int *out) {
    out[0] = (int)sizeof(round_buffer); out[1] = (int)sizeof(intrinsics);
    out[2] = (int)sizeof(Point_Tsdf); out[3] = (int)sizeof(Point_XYZ); out[4] = (int)sizeof(matrix_3f);
    return 0;
}

#elif defined(REF_BILATERAL)
static struct { Point_Depth *src, *dst; point_2us sz; uint maxd; float *cap; } A;
static void item(void) {
    float slot = NAN;
    tde_ref_capture_rte = &slot;
    compute_bilateral_filtering(A.src, A.dst, A.sz, A.maxd);
    tde_ref_capture_rte = NULL;
    A.cap[get_global_id(1) * A.sz.x + get_global_id(0)] = slot;
}
/* dst receives the kernel's literal output; intended[] receives sum1/sum2 */
TDE_REF_EXPORT int ref_bilateral(const void *src, void *dst, int cols, int rows, unsigned maxd,
                                 float *intended) {
    A.src = (Point_Depth *)src; A.dst = (Point_Depth *)dst;
    A.sz.x = (us)cols; A.sz.y = (us)rows; A.maxd = maxd; A.cap = intended;
    tde_ref_run_plain(item, (size_t)cols, (size_t)rows, 32, 8);
    return 0;
}

#elif defined(REF_TRANSFORM_MAP)
static struct { Point_XYZ *vs; Point_NXYZ *ns; matrix_3f R; point_3f t; point_2us sz; Point_XYZ *vd; Point_NXYZ *nd; } A;
static void item(void) { transform_map(A.vs, A.ns, A.R, A.t, A.sz, A.vd, A.nd); }
TDE_REF_EXPORT int ref_transform_map(const void *vs, const void *ns, const float *R, const float *t,
                                     int cols, int rows, void *vd, void *nd) {
    A.vs = (Point_XYZ *)vs; A.ns = (Point_NXYZ *)ns; memcpy(&A.R, R, sizeof(A.R));
    memcpy(&A.t, t, sizeof(A.t)); A.sz.x = (us)cols; A.sz.y = (us)rows;
    A.vd = (Point_XYZ *)vd; A.nd = (Point_NXYZ *)nd;
    tde_ref_run_plain(item, (size_t)cols, (size_t)rows, 32, 8);
    return 0;
}

#elif defined(REF_TRANSFORM_ESTIMATION)
static struct { float *gbuf, *out; int len; } A;
static void item(void) { transform_estimation(A.gbuf, A.out, A.len); }
TDE_REF_EXPORT int ref_transform_estimation(const float *gbuf, float *out, int buf_length) {
    A.gbuf = (float *)gbuf; A.out = out; A.len = buf_length;
    return tde_ref_run_fibers(item, (size_t)DEFAULT_STRIDE * 27, 1, DEFAULT_STRIDE, 1);
}

#elif defined(REF_CLEAN_BUFF)
static struct { float *p; int w; } A;
static void item(void) { clean_buff(A.p, A.w); }
TDE_REF_EXPORT int ref_clean_buff(float *p, int width) {
    A.p = p; A.w = width;
    tde_ref_run_plain(item, (size_t)width, 1, (size_t)width, 1);
    return 0;
}

#elif defined(REF_SCAN_SLICE)
static struct { Point_Tsdf *t; Point_Color *c; point_3i mn, mx; uint lo, hi; round_buffer rb; uint *pred; uint *num; } A;
static void item(void) {
    scan_slice_of_both_volumes(A.t, A.c, A.mn, A.mx, A.lo, A.hi, A.rb, A.pred, A.num);
}
TDE_REF_EXPORT int ref_scan_slice(const void *tsdf, const void *color, const int *mn, const int *mx,
                                  unsigned lo, unsigned hi, const void *rb, unsigned *pred, unsigned *num) {
    A.t = (Point_Tsdf *)tsdf; A.c = (Point_Color *)color;
    memcpy(&A.mn, mn, sizeof(A.mn)); memcpy(&A.mx, mx, sizeof(A.mx));
    A.lo = lo; A.hi = hi; memcpy(&A.rb, rb, sizeof(A.rb)); A.pred = pred; A.num = num;
    return tde_ref_run_fibers(item, (size_t)A.rb.voxels_size.x, (size_t)A.rb.voxels_size.y, 32, 8);
}

#elif defined(REF_EXTRACT_SLICE)
static struct { uint *pred; Point_Tsdf *t; Point_Color *c; uint lo, hi; point_3f cell; point_3i mn, mx; round_buffer rb; Point_XYZI *pv; Point_Color *pc; } A;
static void item(void) {
    extract_slice_as_cloud(A.pred, A.t, A.c, A.lo, A.hi, A.cell, A.mn, A.mx, A.rb, A.pv, A.pc);
}
TDE_REF_EXPORT int ref_extract_slice(const unsigned *slots, const void *tsdf, const void *color, unsigned lo,
                                     unsigned hi, const float *cell, const int *mn, const int *mx,
                                     const void *rb, void *points, void *colors) {
    A.pred = (uint *)slots; A.t = (Point_Tsdf *)tsdf; A.c = (Point_Color *)color; A.lo = lo; A.hi = hi;
    memcpy(&A.cell, cell, sizeof(A.cell)); memcpy(&A.mn, mn, sizeof(A.mn)); memcpy(&A.mx, mx, sizeof(A.mx));
    memcpy(&A.rb, rb, sizeof(A.rb)); A.pv = (Point_XYZI *)points; A.pc = (Point_Color *)colors;
    tde_ref_run_plain(item, (size_t)A.rb.voxels_size.x, (size_t)A.rb.voxels_size.y, 32, 8);
    return 0;
}

#elif defined(REF_CLEAN_COLOR_SLICE)
static struct { Point_Color *c; point_3i mn, mx; round_buffer rb; } A;
static void item(void) { clean_color_slice(A.c, A.mn, A.mx, A.rb); }
TDE_REF_EXPORT int ref_clean_color_slice(void *color, const int *mn, const int *mx, const void *rb) {
    A.c = (Point_Color *)color; memcpy(&A.mn, mn, sizeof(A.mn)); memcpy(&A.mx, mx, sizeof(A.mx));
    memcpy(&A.rb, rb, sizeof(A.rb));
    tde_ref_run_plain(item, (size_t)A.rb.voxels_size.x, (size_t)A.rb.voxels_size.y, 32, 8);
    return 0;
}
#elif defined(REF_LSM)
/* compute_least_squares_equation over n correspondences.  Each item writes
 * Indexes[id + 0..5] (overlapping its neighbours' entries for n > 1), so the
 * per-correspondence row is read with n = 1. */
static struct {
    Point_Intensity *ip; float *dp; Point_Intensity *ic; unsigned char *dx, *dy; point_2i *cp, *cc; float *diff;
    float sigma; matrix_3f R; vector_3f t; intrinsics intr; int n; float *idx, *vec;
} A;
static void item(void) {
    compute_least_squares_equation(A.ip, A.dp, A.ic, A.dx, A.dy, A.cp, A.cc, A.diff, A.sigma, A.R, A.t, A.intr,
                                   A.n, A.idx, A.vec);
}
TDE_REF_EXPORT int ref_lsm(const void *i_prev, const float *d_prev, const void *i_curr, const unsigned char *dx,
                           const unsigned char *dy, const int *corr_prev, const int *corr_curr, const float *diff,
                           float sigma, const float *R, const float *t, const void *intr, int n, float *indexes,
                           float *indexes_vector) {
    A.ip = (Point_Intensity *)i_prev; A.dp = (float *)d_prev; A.ic = (Point_Intensity *)i_curr;
    A.dx = (unsigned char *)dx; A.dy = (unsigned char *)dy;
    A.cp = (point_2i *)corr_prev; A.cc = (point_2i *)corr_curr; A.diff = (float *)diff; A.sigma = sigma;
    memcpy(&A.R, R, sizeof(A.R)); memcpy(&A.t, t, sizeof(A.t)); memcpy(&A.intr, intr, sizeof(A.intr));
    A.n = n; A.idx = indexes; A.vec = indexes_vector;
    tde_ref_run_plain(item, (size_t)n, 1, 1, 1);
    return 0;
}
TDE_REF_EXPORT int ref_lsm_sizes(int *out) {
    out[0] = (int)sizeof(Point_Intensity); out[1] = (int)sizeof(point_2i); out[2] = (int)sizeof(intrinsics);
    out[3] = (int)sizeof(matrix_3f);
    return 0;
}
#else
#error "define one REF_<KERNEL>"
#endif
