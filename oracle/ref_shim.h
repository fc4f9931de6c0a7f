/*
 * ref_shim.h -- OpenCL C 1.x work-item shim for compiling the reference's
 * GPU/opencl/*.cl kernels as plain C (gcc -x c -std=gnu11).
 *
 * TEST INFRASTRUCTURE ONLY.  The shared objects built with this shim live in
 * oracle/_ref/ and are used solely by tests/golden/make_golden.py to pin the
 * oracle restatement and to produce the committed golden vectors.  Nothing in
 * the product links or loads them.
 *
 * Semantics emulated (OpenCL C 1.2, section 6):
 *   - address-space qualifiers vanish; `local` arrays become `static` so that
 *     every work-item of a work-group shares them (work-groups run one at a
 *     time on one OS thread when a kernel uses barrier()).
 *   - get_global_id / get_local_id / get_group_id / get_local_size read a
 *     per-thread work-item record that the launcher fills.
 *   - barrier() yields to a ucontext fiber scheduler (see ref_launch.c); the
 *     kernels that never call it run as plain loops.
 *   - builtin math on float arguments is the float overload (sqrt -> sqrtf,
 *     exp -> expf), as OpenCL's overloads are; min/max follow the OpenCL
 *     definitions for integer and float arguments.
 *   - convert_<int|ushort>[_sat]_<rte|rtz|rtn> follow the rounding-mode
 *     suffix; the non-saturating forms are made saturating, which only fixes
 *     behaviour the OpenCL specification leaves undefined.
 */
#ifndef TDE_REF_SHIM_H
#define TDE_REF_SHIM_H

#include <float.h> /* FLT_/DBL_EPSILON: OpenCL C 6.12.2.1 macros */
#include <math.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <limits.h>

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;

typedef struct { float x, y, z, w; } float4;

/* ---- qualifiers ---------------------------------------------------------- */
#define __kernel
#define kernel
#define __global
#define global
#define __constant const
#define constant const
#define __read_only
#define read_only
#define __write_only
#define write_only
#define __local static
#define local static
#define __private
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

/* ---- work-item state ------------------------------------------------------ */
typedef struct {
    size_t gid[3], lid[3], grp[3], lsz[3], gsz[3];
} tde_ref_workitem;

extern _Thread_local tde_ref_workitem *tde_ref_wi;

static inline size_t get_global_id(uint d) { return tde_ref_wi->gid[d]; }
static inline size_t get_local_id(uint d) { return tde_ref_wi->lid[d]; }
static inline size_t get_group_id(uint d) { return tde_ref_wi->grp[d]; }
static inline size_t get_local_size(uint d) { return tde_ref_wi->lsz[d]; }
static inline size_t get_global_size(uint d) { return tde_ref_wi->gsz[d]; }

void tde_ref_barrier(void);
#define barrier(flags) tde_ref_barrier()

/* ---- atomics (kernels using them run single-threaded) --------------------- */
static inline uint tde_ref_atomic_add(volatile uint *p, uint v) { uint o = *p; *p = o + v; return o; }
#define atomic_add(p, v) tde_ref_atomic_add((volatile uint *)(p), (uint)(v))
#define atom_add(p, v) tde_ref_atomic_add((volatile uint *)(p), (uint)(v))

/* ---- min / max (OpenCL 6.12.3 integer, 6.12.4 float) ---------------------- */
static inline int tde_ref_imin(int a, int b) { return b < a ? b : a; }
static inline int tde_ref_imax(int a, int b) { return a < b ? b : a; }
static inline uint tde_ref_umin(uint a, uint b) { return b < a ? b : a; }
static inline uint tde_ref_umax(uint a, uint b) { return a < b ? b : a; }
static inline long tde_ref_lmin(long a, long b) { return b < a ? b : a; }
static inline long tde_ref_lmax(long a, long b) { return a < b ? b : a; }
static inline ulong tde_ref_ulmin(ulong a, ulong b) { return b < a ? b : a; }
static inline ulong tde_ref_ulmax(ulong a, ulong b) { return a < b ? b : a; }
/* float max: "returns y if x < y, otherwise x" */
static inline float tde_ref_fmin(float a, float b) { return b < a ? b : a; }
static inline float tde_ref_fmax(float a, float b) { return a < b ? b : a; }
static inline double tde_ref_dmin(double a, double b) { return b < a ? b : a; }
static inline double tde_ref_dmax(double a, double b) { return a < b ? b : a; }

#define TDE_REF_SEL(a, b, F, D, I, U, L, UL)                                       \
    _Generic((a) + (b), float: F, double: D, int: I, unsigned int: U, long: L,     \
             unsigned long: UL, default: I)
#define min(a, b) TDE_REF_SEL(a, b, tde_ref_fmin, tde_ref_dmin, tde_ref_imin, tde_ref_umin, \
                              tde_ref_lmin, tde_ref_ulmin)((a), (b))
#define max(a, b) TDE_REF_SEL(a, b, tde_ref_fmax, tde_ref_dmax, tde_ref_imax, tde_ref_umax, \
                              tde_ref_lmax, tde_ref_ulmax)((a), (b))

/* ---- float builtins: float overloads ------------------------------------- */
#define sqrt(x) sqrtf((float)(x))
#define exp(x) expf((float)(x))

/* ---- conversions ----------------------------------------------------------- */
static inline int tde_ref_sat_i32(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}
static inline ushort tde_ref_sat_u16(double v) {
    if (v != v) return 0;
    if (v >= 65535.0) return 65535;
    if (v <= 0.0) return 0;
    return (ushort)v;
}

/* Capture hook: the bilateral kernel's intended result is the argument of its
 * convert_int_rte (sum1/sum2); the harness records it per work-item. */
extern _Thread_local float *tde_ref_capture_rte;

static inline int tde_ref_int_rte(float v) {
    if (tde_ref_capture_rte) *tde_ref_capture_rte = v;
    return tde_ref_sat_i32(nearbyintf(v));
}
#define convert_int_rte(x) tde_ref_int_rte((float)(x))
#define convert_int_sat_rte(x) tde_ref_sat_i32(nearbyintf((float)(x)))
#define convert_int_rtz(x) tde_ref_sat_i32(truncf((float)(x)))
#define convert_int_sat_rtz(x) tde_ref_sat_i32(truncf((float)(x)))
#define convert_int_rtn(x) tde_ref_sat_i32(floorf((float)(x)))
#define convert_int_sat_rtn(x) tde_ref_sat_i32(floorf((float)(x)))
#define convert_ushort_rte(x) tde_ref_sat_u16(nearbyintf((float)(x)))
#define convert_ushort_sat_rte(x) tde_ref_sat_u16(nearbyintf((float)(x)))

#endif /* TDE_REF_SHIM_H */
