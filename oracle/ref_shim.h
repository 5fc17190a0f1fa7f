/*
 * ref_shim.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Lets gcc compile the reference's OpenCL C kernels
 * (SvoTracer/SvoTracer.Kernel/wavefront.cl) for the host CPU so that the
 * restatement in svo_oracle.c can be checked against the reference's own
 * code. build_ref.py rewrites only OpenCL syntax that C lacks (vector
 * literals become compound literals, .x/.y/.z become [0]/[1]/[2]); this
 * header supplies the OpenCL types and built-ins.
 *
 * Execution model: every kernel runs with work-groups of one work-item, so
 * work_group_barrier is a no-op; work-items of a pass may run on several host
 * threads, so the atomics are real (relaxed) atomics.
 *
 * OpenCL's implementation-defined built-ins follow the parity contract:
 * native_divide is IEEE division, native_sin/cos are (float)sin((double)x),
 * fast_length is sqrtf((x*x + y*y) + z*z), and half_log2 returns a value
 * whose comparisons with integers (the only way wavefront.cl reads
 * ConeDepth = -half_log2(c)) are exact: floor(log2 x) + 0.5 when x is not a
 * power of two, log2 x exactly when it is. length and normalize (kernel.cl)
 * use the same correctly rounded sqrtf((x*x + y*y) + z*z); normalize returns
 * its argument when every element is zero, as the OpenCL C specification
 * defines it. floatToUlong's out-of-range and NaN conversions saturate
 * (NaN -> 0), as on the GPU.
 */
#ifndef REF_SHIM_H
#define REF_SHIM_H

#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <string.h>

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;

typedef float float2 __attribute__((vector_size(8)));
typedef float float3 __attribute__((vector_size(16)));
typedef float float4 __attribute__((vector_size(16)));
typedef int int2 __attribute__((vector_size(8)));
typedef uint uint2 __attribute__((vector_size(8)));
typedef uint uint3 __attribute__((vector_size(16)));
typedef ulong ulong3 __attribute__((vector_size(32)));

#define global
#define local
#define constant const
#define kernel
#define __write_only
typedef float *image2d_t;

#ifndef ULONG_MAX
#define ULONG_MAX 0xFFFFFFFFFFFFFFFFul
#endif
#ifndef UINT_MAX
#define UINT_MAX 0xFFFFFFFFu
#endif
#ifndef USHRT_MAX
#define USHRT_MAX 65535
#endif
#ifndef UCHAR_MAX
#define UCHAR_MAX 255
#endif
#define M_PI_F 3.14159274101257324219f
#define M_PI_2_F 1.57079637050628662109f
#define CLK_LOCAL_MEM_FENCE 1

/* Work-item identity, set by the harness before each kernel call. */
extern _Thread_local size_t ref_gid[2];
extern size_t ref_gsize[2];
extern uint ref_image_width;
static inline size_t get_global_id(int d) { return ref_gid[d]; }
static inline size_t get_global_size(int d) { return ref_gsize[d]; }
static inline size_t get_local_id(int d) {
  (void)d;
  return 0;
}
static inline void work_group_barrier(int f) { (void)f; }

#define atomic_inc(p) __atomic_fetch_add((p), 1, __ATOMIC_RELAXED)
#define atomic_dec(p) __atomic_fetch_sub((p), 1, __ATOMIC_RELAXED)
#define atomic_add(p, v) __atomic_fetch_add((p), (v), __ATOMIC_RELAXED)
#define atomic_xchg(p, v) __atomic_exchange_n((p), (v), __ATOMIC_RELAXED)

static inline float nd_s(float a, float b) { return a / b; }
static inline float3 nd_v3(float a, float3 b) { return a / b; }
#define native_divide(a, b) _Generic((b), float3: nd_v3, default: nd_s)((a), (b))

/* floatToUlong's conversion (rewritten by build_ref.py): saturating, NaN -> 0. */
static inline ulong ref_float_to_ulong(double v) {
  if (v != v || v <= 0.0) return 0;
  if (v >= 18446744073709551616.0) return ULONG_MAX;
  return (ulong)v;
}

/* (uchar)x of the material stage (rewritten by build_ref.py): truncation inside
 * [0, 255], saturating outside, NaN -> 0. */
static inline uchar ref_float_to_uchar(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 255.0f) return 255;
  return (uchar)v;
}

static inline float native_sin(float x) { return (float)sin((double)x); }
static inline float native_cos(float x) { return (float)cos((double)x); }

static inline float half_log2(float x) {
  if (x != x || x < 0.0f) return NAN;
  if (x == 0.0f) return -INFINITY;
  if (isinf(x)) return INFINITY;
  int e;
  float f = frexpf(x, &e); /* x = f * 2^e, f in [0.5, 1) */
  return f == 0.5f ? (float)(e - 1) : (float)(e - 1) + 0.5f;
}

static inline float fast_length(float3 v) { return sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static inline float dot(float3 a, float3 b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline float length(float3 v) { return sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static inline float3 normalize(float3 v) {
  if (v[0] == 0.0f && v[1] == 0.0f && v[2] == 0.0f) return v;
  float l = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  return v / l;
}
static inline float3 cross(float3 a, float3 b) {
  return (float3){a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0], 0.0f};
}

#define max(a, b) ({ __typeof__(a) _a = (a); __typeof__(b) _b = (b); _a < _b ? _b : _a; })
#define min(a, b) ({ __typeof__(a) _a = (a); __typeof__(b) _b = (b); _b < _a ? _b : _a; })
static inline uint abs_diff(uint a, uint b) { return a > b ? a - b : b - a; }

static inline void write_imagef(image2d_t img, int2 coord, float4 c) {
  float *p = img + 4 * ((size_t)coord[1] * ref_image_width + (size_t)coord[0]);
  p[0] = c[0];
  p[1] = c[1];
  p[2] = c[2];
  p[3] = c[3];
}

#endif
