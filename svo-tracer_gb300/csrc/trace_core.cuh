// Device code shared by the trace and the differentiable kernels: the
// fixed-point stepping of wavefront.cl (traverseChunk, comparePositions,
// roundUlong, floatToUlong/ulongToFloat), the ray setup (setupInitialTrace,
// traceIntoVolume) and one runBaseTrace/runBlockTrace step.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "svo_internal.h"

namespace svo {
namespace {

namespace cg = cooperative_groups;

constexpr unsigned kFull = 0xffffffffu;
constexpr uint64_t kAll = ~0ull;

// powSum (wavefront.cl:224): base chunks of levels 1..depth, depth 0..10, by
// the reference's shift of a repeating octal pattern (no table: lanes at
// different depths would serialise on a constant-memory read).
__device__ __forceinline__ uint32_t pow_sum(int depth) {
  return (uint32_t)((0b1001001001001001001001001001001000ull >> ((11 - depth) * 3)) - 1);
}

// The fixed-point conversions exist in two exact forms: the 64-bit conversion
// instructions, which run on this GPU's FP64 pipe at 1/64 of the FP32 rate, and
// integer forms (more instructions, no FP64 pipe). The step code is bound by
// instruction issue, and by the FP64 pipe once it carries most conversions, so
// the fastest mix splits them between the two; measured on GB300 with
// identical outputs (1080p frame / 64 views / megakernel frame):
//  * ulong_to_float (SVO_CVT_INTEGER): the integer form, except where
//    SVO_CVT_HW_TRAVERSE and SVO_CVT_HW_CONE give the number of traverseChunk's
//    three boundary distances and coneSize's three coordinates converted by the
//    instruction. Counts (traverse, cone) 0,0: 1.451 / 8.12 / 14.60 ms;
//    2,2: 1.371 / 7.61 / 13.85 ms; 2,1: 1.384 / 7.72 / 13.95; 2,3: 1.386 / 7.65
//    / 13.92; 1,2: 1.398 / 7.80 / 14.04; 3,0: 1.409 / 7.77 / 14.08; 3,3 (the
//    instruction everywhere): 1.445 / 7.91 / 14.29. An integer form without
//    the 32-bit conversion (normalise, round by guard and sticky bits) at 2,2:
//    1.470 / 8.16 / 14.55 ms.
//  * unit_to_ulong (SVO_CVT_INTEGER_F2U): the instruction unless set. The
//    integer form for one of traverseChunk's two moves at 2,2: 1.415 / 7.90 /
//    14.26 ms; for both: 1.467 / 8.17 / 14.71 ms.
#ifndef SVO_CVT_INTEGER
#define SVO_CVT_INTEGER 1
#endif
#ifndef SVO_CVT_INTEGER_F2U
#define SVO_CVT_INTEGER_F2U 0
#endif

// (float)x of a 64-bit fixed-point value, rounded to nearest even
// (ulongToFloat, wavefront.cl:209, without the 2^-64 scaling). Integer form:
// the top 32 significant bits of x with every lower bit folded into a sticky
// LSB (which leaves the rounding decision unchanged), the 32-bit conversion,
// and the scale 2^(32 - n) added to the exponent field; x = 0 gives 0.
__device__ __forceinline__ float ulong_to_float(uint64_t x) {
  if (!SVO_CVT_INTEGER) return __ull2float_rn(x);
  const uint32_t hi = (uint32_t)(x >> 32), lo = (uint32_t)x;
  const uint32_t n = __clz(hi);                       // 32 when hi == 0
  const uint32_t top = __funnelshift_lc(lo, hi, n);   // bits 63..32 of x << n
  const uint32_t rest = __funnelshift_lc(0u, lo, n);  // bits 31..0 of x << n
  const float f = __uint2float_rn(top | (rest != 0u ? 1u : 0u));
  return __int_as_float(__float_as_int(f) + (int)((32u - n) << 23));
}
// ulongToFloat (wavefront.cl:209): (float)x * 2^-64, the scaling exact.
__device__ __forceinline__ float ulong_to_unit(uint64_t x) { return __fmul_rn(ulong_to_float(x), 0x1p-64f); }
// The same conversion by the 64-bit instruction (kHw) or the integer form.
template <bool kHw>
__device__ __forceinline__ float ulong_to_float_by(uint64_t x) { return kHw ? __ull2float_rn(x) : ulong_to_float(x); }
#ifndef SVO_CVT_HW_CONE
#define SVO_CVT_HW_CONE 2
#endif
#ifndef SVO_CVT_HW_TRAVERSE
#define SVO_CVT_HW_TRAVERSE 2
#endif

// floatToUlong (wavefront.cl:200-207); out-of-range products saturate, NaN -> 0.
// Integer form: |x| * 2^64 is exact (a power-of-two scale of a float below the
// overflow range), so its truncation is the 24-bit significand m shifted by
// e = exponent(|x|) + 64 - 150: m << e for e >= 0, m >> -e for e in (-24, 0),
// 0 below; |x| >= 1 saturates to 2^64 - 1 as the instruction does.
__device__ __forceinline__ uint64_t unit_to_ulong(float x) {
  if (x >= 0.999999911f) return kAll;
  if (SVO_CVT_INTEGER_F2U) {
    const uint32_t u = __float_as_uint(x) & 0x7fffffffu;
    if (u > 0x7f800000u) return 0;       // NaN
    if (u >= 0x3f800000u) return kAll;   // |x| >= 1 (and infinity)
    const int e = (int)(u >> 23) - 86;   // exponent + 64 - 150, at most 40
    const uint32_t m = (u & 0x7fffffu) | 0x800000u;
    if (e >= 0) return (uint64_t)m << e;
    return e > -24 ? (uint64_t)(m >> -e) : 0ull;
  }
  const float v = __fmul_rn(fabsf(x), 0x1p64f);
  // the conversion clamps v >= 2^64 to kAll, but turns NaN into 2^63
  return v != v ? 0 : __float2ull_rz(v);
}

// Locations in travel space. A ray keeps each 64-bit fixed-point coordinate v
// as w = v for a positive direction and w = ~v for a negative one, so that a
// step in the travel direction always increases w. Then, with
// low = kAll >> (d + 1) (the bits below level d+1), the reference's rules of
// both directions become one:
//   roundUlong (wavefront.cl:211-221): the distance to the next level-(d+1)
//     boundary is (~w & low) + 1, except for a negative direction in the lowest
//     cell ((w | low) == kAll), where the reference's subtraction wraps and its
//     comparison returns v = ~w;
//   traverseChunk's move and clamp (:440-497): w += d, and a sum of 0 becomes
//     kAll (v + d giving 0 becomes ULONG_MAX; v - d giving ULONG_MAX becomes 0);
//   leaving (:433-437): some w == kAll, so after a move: some sum is 0 or kAll;
//   comparePositions (:413-426): the bits that flipped against the travel
//     direction are w_before & ~w_after.
// Real coordinates (octants, cell indices, float conversions, requests) are
// w ^ dir_mask.
__device__ __forceinline__ uint64_t dir_mask(bool positive) { return positive ? 0ull : kAll; }

// low = kAll >> (d + 1) for a level d below 32: its low word is all ones, so
// only its high word low_hi is passed. In the negative-direction case ~w has no
// bit above low, so ~w & low is ~w itself.
__device__ __forceinline__ uint64_t boundary_distance(uint64_t w, uint32_t low_hi, bool positive) {
  const uint32_t wh = (uint32_t)(w >> 32);
  const uint64_t t = ((uint64_t)(~wh & low_hi) << 32) | (uint32_t)~(uint32_t)w;  // ~w & low
  return t + ((!positive && (wh | low_hi) == ~0u) ? 0u : 1u);
}

// A coordinate after a move that leaves the cube: w == 0 (the reference clamps it
// to kAll) or w == kAll.
__device__ __forceinline__ bool leaves_cube(uint64_t w) {
  const uint32_t lo = (uint32_t)w, hi = (uint32_t)(w >> 32);
  return lo == hi && hi + 1u <= 1u;
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// spread3 of every 10-bit value, in shared memory: filled by each CTA of the
// kernels that step rays (fill_spread_table before their first __syncthreads).
__shared__ uint32_t s_spread3[1024];

__device__ __forceinline__ void fill_spread_table() {
  for (uint32_t i = threadIdx.x; i < 1024; i += blockDim.x) s_spread3[i] = spread3(i);
}

// baseLocation (wavefront.cl:405-411) for 1 <= depth <= 10 from travel-space
// coordinates: the Morton index of the top `depth` bits of each real coordinate
// (all within the high 32 bits; `flip` bit k set for a negative axis k).
__device__ __forceinline__ uint32_t cell_index(int depth, uint64_t wx, uint64_t wy, uint64_t wz, uint32_t flip) {
  const uint32_t s = 32 - depth;
  const uint32_t cx = ((uint32_t)(wx >> 32) ^ (0u - (flip & 1u))) >> s;
  const uint32_t cy = ((uint32_t)(wy >> 32) ^ (0u - ((flip >> 1) & 1u))) >> s;
  const uint32_t cz = ((uint32_t)(wz >> 32) ^ (0u - ((flip >> 2) & 1u))) >> s;
  return s_spread3[cx] | (s_spread3[cy] << 1) | (s_spread3[cz] << 2);
}

// Levels 1..31 are bits 63..32 of a coordinate, so the stepping helpers below
// read only the high words (trees are at most SVO_MAX_TREE_DEPTH = 24 deep).
__device__ __forceinline__ uint32_t hi32(uint64_t w) { return (uint32_t)(w >> 32); }

// chunkPosition (wavefront.cl:428-430) from travel-space coordinates, depth 0..31.
__device__ __forceinline__ uint32_t octant(int depth, uint64_t wx, uint64_t wy, uint64_t wz, uint32_t flip) {
  const uint32_t s = 31u - (uint32_t)depth;
  return (((hi32(wx) >> s) & 1u) | (((hi32(wy) >> s) & 1u) << 1) | (((hi32(wz) >> s) & 1u) << 2)) ^ flip;
}

__device__ __forceinline__ float pow2_neg(int k) { return __int_as_float((127 - k) << 23); }

struct Ray {
  uint64_t wx, wy, wz;  // location in travel space (see dir_mask)
  float dx, dy, dz;
  float ix, iy, iz;
  float ox, oy, oz;
  float fov;
  uint32_t id;   // pixel index within its view
  int view;
  int depth;
  int steps;
  bool sx, sy, sz;
  uint32_t flip;  // bit k: axis k travels towards 0
  bool fresh;     // megakernel primary: no move yet, so kernel.cl's ConeDepth is still 0
  float cone;     // coneSize at the current location, < 0 until computed there
  uint32_t cell;  // baseLocation(depth) while depth <= B (SVO_TRACE_CELL_CACHE)
};

// SVO_TRACE_CELL_CACHE: a ray at a base level keeps baseLocation(depth) in a
// register. A descent extends it by the octant the step just read
// (baseLocation(d + 1) = 8 baseLocation(d) + chunkPosition(d)), an ascent to
// level B takes it from the level-(B+2) path entry (>> 6), and only a move (or
// the ray's start) computes it from the location. Identical results; measured
// on GB300 (1080p frame / 64 views / megakernel frame): 1.520 vs 1.520 ms, 8.47
// vs 8.65 ms, 14.91 vs 15.05 ms.
#ifndef SVO_TRACE_CELL_CACHE
#define SVO_TRACE_CELL_CACHE 1
#endif
// SVO_TRACE_BASE_RUN: a base-level step that descends runs the ray's following
// base-level steps in the same call while they descend (with the cell cache
// only). Identical results; measured on GB300 (1080p frame / 64 views /
// megakernel frame): 1.453 vs 1.464 ms, 8.12 vs 8.43 ms, 14.69 vs 14.91 ms, and
// 56 instead of 59 registers in the trace kernel.
#ifndef SVO_TRACE_BASE_RUN
#define SVO_TRACE_BASE_RUN 1
#endif
// (The same for block-level descents, where the next step loads the child node,
// measured much slower: 1.82 vs 1.46 ms, 10.5 vs 8.1 ms, 18.7 vs 14.7 ms.)


__device__ __forceinline__ uint64_t loc_x(const Ray &r) { return r.wx ^ dir_mask(r.sx); }
__device__ __forceinline__ uint64_t loc_y(const Ray &r) { return r.wy ^ dir_mask(r.sy); }
__device__ __forceinline__ uint64_t loc_z(const Ray &r) { return r.wz ^ dir_mask(r.sz); }
__device__ __forceinline__ void set_loc(Ray &r, uint64_t x, uint64_t y, uint64_t z) {
  r.wx = x ^ dir_mask(r.sx);
  r.wy = y ^ dir_mask(r.sy);
  r.wz = z ^ dir_mask(r.sz);
  r.cone = -1.0f;
}

struct Node {
  uint32_t child;
  uint32_t chunk;
};

__device__ __forceinline__ uint4 load_node(const uint4 *blocks, uint32_t n_blocks, uint32_t addr) {
  if (addr >= n_blocks) return make_uint4(0, 0, 0, 0);
  return __ldg(blocks + addr);
}

// traverseChunk (wavefront.cl:440-497) without the trailing setConeDepth,
// returning leaving (:433-437) of the new location. A sum that the reference
// clamps (0 to kAll) always leaves, so the clamp is left to the caller's
// leaving branch.
// SVO_TRACE_AXIS_BOUNDS (off): traverseChunk's axis chosen from bounds on the
// three boundary distances, one exact 64-bit conversion instead of three when
// the choice is clear. Identical results; measured on GB300 (1080p frame / 64
// views / megakernel frame): 1.536 vs 1.522 ms, 8.54 vs 8.66 ms, 16.96 vs 15.07
// ms, so the FP64-pipe conversions it saves do not bound these kernels.
#ifndef SVO_TRACE_AXIS_BOUNDS
#define SVO_TRACE_AXIS_BOUNDS 0
#endif
__device__ __forceinline__ bool traverse(Ray &r, int depth) {
  const uint32_t low_hi = 0xffffffffu >> (depth + 1);  // kAll >> (depth + 1), depth < 31
  uint64_t d0 = boundary_distance(r.wx, low_hi, r.sx);
  uint64_t d1 = boundary_distance(r.wy, low_hi, r.sy);
  uint64_t d2 = boundary_distance(r.wz, low_hi, r.sz);
  int ax = -1;
  float fa = 0.0f;
  if (SVO_TRACE_AXIS_BOUNDS) {
    // The axis from bounds. A distance d with high word h >= 1 lies in
    // [h, h + 1) * 2^32, so fl(d) lies in [RZ(h), RU(h + 1)] * 2^32 (floats
    // below and above d), and a = fl(fl(d) * |inv|) lies between the rounded
    // products of those bounds (the rounded product is monotone). An axis whose
    // upper bound is below both other lower bounds is the strict minimum, the
    // reference's choice whatever its tie rule; only its distance is then
    // converted exactly. Otherwise all three are (below).
    const uint32_t h0 = hi32(d0), h1 = hi32(d1), h2 = hi32(d2);
    if (h0 && h1 && h2) {
      const float i0 = fabsf(r.ix), i1 = fabsf(r.iy), i2 = fabsf(r.iz);
      const float l0 = __fmul_rn(__fmul_rn(__uint2float_rz(h0), 0x1p32f), i0);
      const float l1 = __fmul_rn(__fmul_rn(__uint2float_rz(h1), 0x1p32f), i1);
      const float l2 = __fmul_rn(__fmul_rn(__uint2float_rz(h2), 0x1p32f), i2);
      const float u0 = __fmul_rn(__fmul_rn(__uint2float_ru(h0 + (h0 != 0xffffffffu)), 0x1p32f), i0);
      const float u1 = __fmul_rn(__fmul_rn(__uint2float_ru(h1 + (h1 != 0xffffffffu)), 0x1p32f), i1);
      const float u2 = __fmul_rn(__fmul_rn(__uint2float_ru(h2 + (h2 != 0xffffffffu)), 0x1p32f), i2);
      ax = (u0 < l1 && u0 < l2) ? 0 : ((u1 < l0 && u1 < l2) ? 1 : ((u2 < l0 && u2 < l1) ? 2 : -1));
      if (ax >= 0) fa = ulong_to_float(ax == 0 ? d0 : (ax == 1 ? d1 : d2));
    }
  }
  if (ax < 0) {
    const float f0 = ulong_to_float_by<(SVO_CVT_HW_TRAVERSE >= 1)>(d0);
    const float f1 = ulong_to_float_by<(SVO_CVT_HW_TRAVERSE >= 2)>(d1);
    const float f2 = ulong_to_float_by<(SVO_CVT_HW_TRAVERSE >= 3)>(d2);
    float a0 = fabsf(__fmul_rn(f0, r.ix));
    float a1 = fabsf(__fmul_rn(f1, r.iy));
    float a2 = fabsf(__fmul_rn(f2, r.iz));
    ax = (a0 <= a1 && a0 <= a2) ? 0 : ((a1 <= a0 && a1 <= a2) ? 1 : 2);
    fa = ax == 0 ? f0 : (ax == 1 ? f1 : f2);
  }
  float inv = ax == 0 ? r.ix : (ax == 1 ? r.iy : r.iz);
  // ulongToFloat of the chosen distance: its float conversion times 2^-64 (exact)
  float u = __fmul_rn(fa, 0x1p-64f);
  // the two other axes' moves, exactly two conversions per lane: A is x unless x
  // was chosen (then y), B is z unless z was chosen (then y)
  const bool c0 = ax == 0, c2 = ax == 2;
  const uint64_t eA = unit_to_ulong(__fmul_rn(__fmul_rn(c0 ? r.dy : r.dx, inv), u));
  const uint64_t eB = unit_to_ulong(__fmul_rn(__fmul_rn(c2 ? r.dy : r.dz, inv), u));
  d1 = c0 ? eA : (c2 ? eB : d1);
  if (!c0) d0 = eA;
  if (!c2) d2 = eB;
  r.wx += d0;
  r.wy += d1;
  r.wz += d2;
  return leaves_cube(r.wx) | leaves_cube(r.wy) | leaves_cube(r.wz);
}

// comparePositions (wavefront.cl:413-426): the loop pops one level for every
// consecutive level, counted upwards from `depth`, whose octant bit flipped
// against the travel direction on some axis; it stops at level 1.
// px, py, pz: the travel-space location before the step.
__device__ __forceinline__ int pop_depth(const Ray &r, int depth, uint64_t px, uint64_t py, uint64_t pz) {
  const uint32_t m = (hi32(px) & ~hi32(r.wx)) | (hi32(py) & ~hi32(r.wy)) | (hi32(pz) & ~hi32(r.wz));
  const uint32_t run = ~(m >> (31 - depth));  // bit k: level depth - k kept its octant bit
  const int ones = run ? __ffs((int)run) - 1 : 32;
  return ones < depth ? depth - ones : 1;
}

// coneSize (wavefront.cl:387-391) at the distance setConeDepth uses (:394-399).
__device__ __forceinline__ float cone_at(const Ray &r, float dof0, float dof1) {
  float x = __fsub_rn(r.ox, __fmul_rn(ulong_to_float_by<(SVO_CVT_HW_CONE >= 1)>(loc_x(r)), 0x1p-64f));
  float y = __fsub_rn(r.oy, __fmul_rn(ulong_to_float_by<(SVO_CVT_HW_CONE >= 2)>(loc_y(r)), 0x1p-64f));
  float z = __fsub_rn(r.oz, __fmul_rn(ulong_to_float_by<(SVO_CVT_HW_CONE >= 3)>(loc_z(r)), 0x1p-64f));
  float m = fabsf(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z))));
  float eye = __fmul_rn(r.fov, m);
  float f = fabsf(__fmul_rn(dof0, __fsub_rn(dof1, m)));
  return eye < f ? f : eye;
}

// traceIntoVolume (wavefront.cl:639-1088, kernel.cl:546-995): enter the unit
// cube on the face of the outside slab with the largest entry distance (ties x,
// then y); reject when the entry point is outside the cube grown by the cone
// size. The DoF of the cone size is the TraceData's: zero for the wavefront's
// fresh TraceData, the input's for kernel.cl's setupInitialTrace.
__device__ __forceinline__ bool enter_volume(Ray &r, float dof0 = 0.0f, float dof1 = 0.0f) {
  const float o[3] = {r.ox, r.oy, r.oz};
  const float d[3] = {r.dx, r.dy, r.dz};
  const float iv[3] = {r.ix, r.iy, r.iz};
  bool lo[3], hi[3], any = false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    lo[k] = o[k] < 0.0f;
    hi[k] = o[k] > 1.0f;
    any |= lo[k] | hi[k];
  }
  if (!any) {
    set_loc(r, unit_to_ulong(o[0]), unit_to_ulong(o[1]), unit_to_ulong(o[2]));
    return true;
  }
#pragma unroll
  for (int k = 0; k < 3; k++)
    if ((lo[k] || hi[k]) && d[k] == 0.0f) return false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    bool pos = d[k] >= 0.0f;
    if ((lo[k] && !pos) || (hi[k] && pos)) return false;
  }
  float mk[3];
#pragma unroll
  for (int k = 0; k < 3; k++) mk[k] = (lo[k] || hi[k]) ? fabsf(__fmul_rn(__fsub_rn(hi[k] ? 1.0f : 0.0f, o[k]), iv[k])) : 0.0f;
  bool ox = lo[0] || hi[0], oy = lo[1] || hi[1], oz = lo[2] || hi[2];
  int axis;
  if (ox && oy && oz)
    axis = (mk[0] >= mk[1] && mk[0] >= mk[2]) ? 0 : ((mk[1] >= mk[0] && mk[1] >= mk[2]) ? 1 : 2);
  else if (ox && oy)
    axis = mk[0] >= mk[1] ? 0 : 1;
  else if (ox && oz)
    axis = mk[0] >= mk[2] ? 0 : 2;
  else if (oy && oz)
    axis = mk[1] >= mk[2] ? 1 : 2;
  else
    axis = ox ? 0 : (oy ? 1 : 2);
  float m = mk[axis];
  float p[3];
#pragma unroll
  for (int k = 0; k < 3; k++) p[k] = (k == axis) ? (hi[k] ? 1.0f : 0.0f) : __fadd_rn(o[k], __fmul_rn(d[k], m));
  set_loc(r, unit_to_ulong(p[0]), unit_to_ulong(p[1]), unit_to_ulong(p[2]));
  float eye = __fmul_rn(r.fov, m);
  float f = fabsf(__fmul_rn(dof0, __fsub_rn(dof1, m)));
  float c = eye < f ? f : eye;
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (p[k] < -c || p[k] > __fadd_rn(1.0f, c)) return false;
  return true;
}

struct Stats {
  unsigned long long rays, hits, base_steps, block_reads, block_steps, requests, limited;
};

// Claims `per_lane` consecutive slots of a device counter for every lane of `g`
// with one atomic; returns this lane's first slot. Only the lanes present in `g`
// take part, so lanes may arrive here (or leave the kernel) independently.
__device__ __forceinline__ uint32_t claim(cg::coalesced_group &g, uint32_t *counter, uint32_t per_lane) {
  uint32_t base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, g.size() * per_lane);
  return g.shfl(base, 0) + g.thread_rank();
}

// SVO_CHECKED (a debugging build, off by default): every index of the step code
// into the path cache, the base chunks and the per-pixel outputs is checked
// before the access. A failed check records SVO_ERR_INTERNAL with the check's
// number and the index in the kernel error record (the next synchronising call
// reports it) and the access is skipped: the ray ends as background. Nothing
// traps. With the option off the checks compile to nothing.
#ifndef SVO_CHECKED
#define SVO_CHECKED 0
#endif
#if SVO_CHECKED
__device__ __noinline__ inline void checked_fail(uint32_t *error, uint32_t check, uint32_t index) {
  if (error && atomicCAS(error, 0u, (unsigned)SVO_ERR_INTERNAL) == 0u) {
    error[1] = blockIdx.x;
    error[2] = threadIdx.x;
    error[3] = check;
    error[4] = index;
    error[5] = 0;
  }
}
// True when `cond` holds; false after recording the failed check.
#define SVO_CHECK(err, cond, check, index) ((cond) || (checked_fail((err), (check), (index)), false))
#else
#define SVO_CHECK(err, cond, check, index) true
#endif

// Per-thread traversal state besides the ray itself.
struct Walk {
  uint32_t *path;  // path[level * stride]: node address of each level below B+2
  int stride;
  uint32_t cur_addr, cur_child, cur_chunk;  // last node read
  uint32_t last_group;                      // last usage group stamped
  uint32_t v_block, v_base;                 // reference-walk counters (stats launches)
};

enum : int { kStepOn = 0, kStepBackground = 1, kStepHit = 2, kStepEmpty = 3 };

// The first part of one runBaseTrace (wavefront.cl:1400-1463) or runBlockTrace
// (:1465-1566) step: read the 2-bit octant pair from a chunk (a base chunk or
// the current node's) and, when the octant holds geometry, descend or take the
// cone LOD decision. An empty octant returns kStepEmpty: the step ends with
// advance() (the traverseChunk / comparePositions part), which callers can run
// for the lanes of a warp together.
// kMega: kernel.cl's traceBase/traceBlock (kernel.cl:1002-1073), which differ
// in two points: ConeDepth keeps its initial 0 until the first move (r.fresh),
// and a request carries the frame's Tick and TreeSize 1.
template <bool kStats, bool kSmemBases, bool kMega = false>
__device__ __forceinline__ int probe(const TraceLaunch &a, const ViewParams &v, const uint16_t *s_bases,
                                    const uint4 *blocks, int B, Ray &r, Walk &w, Stats &st) {
  if (r.depth == 0) return kStepBackground;
  if (a.max_steps > 0 && r.steps >= a.max_steps) {
    if (kStats) st.limited++;
    return kStepBackground;
  }
  r.steps++;
  const bool block = r.depth > B;
  const int lvl = r.depth - (B + 2);
  uint32_t chunk;
  if (!block) {
    uint32_t idx = pow_sum(r.depth - 1) + (SVO_TRACE_CELL_CACHE ? r.cell : cell_index(r.depth, r.wx, r.wy, r.wz, r.flip));
    if (!SVO_CHECK(a.error, idx < a.n_bases, 1, idx)) return kStepBackground;
    chunk = kSmemBases ? s_bases[idx] : __ldg(a.bases + idx);
    if (kStats) w.v_base++;
  } else {
    if (!SVO_CHECK(a.error, lvl >= 0 && lvl < a.path_levels, 3, (uint32_t)lvl)) return kStepBackground;
    uint32_t addr = w.path[lvl * w.stride];
    if (addr != w.cur_addr) {
      uint4 nd = load_node(blocks, a.n_blocks, addr);
      w.cur_addr = addr;
      w.cur_child = nd.x;
      w.cur_chunk = nd.y & 0xffffu;
    }
    chunk = w.cur_chunk;
    if (kStats) {
      w.v_block += (uint32_t)(r.depth - B - 1);
      st.block_steps++;
    }
    uint32_t group = addr >> 3;
    if (a.usage && group != w.last_group && group < a.n_groups) {
      // updateUsage (wavefront.cl:377-381)
      uint16_t *tick = reinterpret_cast<uint16_t *>(a.usage + group);
      uint16_t cur = *tick;
      if (cur < 65534 && cur != v.tick) *tick = v.tick;
      w.last_group = group;
    }
  }
  uint32_t oct = octant(r.depth, r.wx, r.wy, r.wz, r.flip);
  if (((chunk >> (oct * 2)) & 2) == 0) return kStepEmpty;
  if (!block) {
    // geometry below a base cell: descend, jumping from level B to B+2
#if SVO_TRACE_BASE_RUN && SVO_TRACE_CELL_CACHE
    // the following base-level steps of the ray run here while they descend:
    // each is the step the next call would take (same step count, limit and
    // order), without the call's dispatch
    while (r.depth < B) {
      r.depth++;
      r.cell = r.cell * 8u + oct;
      if (a.max_steps > 0 && r.steps >= a.max_steps) return kStepOn;  // the next call ends the ray
      r.steps++;
      if (!SVO_CHECK(a.error, pow_sum(r.depth - 1) + r.cell < a.n_bases, 2, pow_sum(r.depth - 1) + r.cell))
        return kStepBackground;
      const uint32_t c2 = kSmemBases ? s_bases[pow_sum(r.depth - 1) + r.cell] : __ldg(a.bases + pow_sum(r.depth - 1) + r.cell);
      if (kStats) w.v_base++;
      oct = octant(r.depth, r.wx, r.wy, r.wz, r.flip);
      if (((c2 >> (oct * 2)) & 2) == 0) return kStepEmpty;
    }
    r.depth = B + 2;
    w.path[0] = (r.cell * 8u + oct) * 8u + octant(B + 1, r.wx, r.wy, r.wz, r.flip);
#else
    if (r.depth < B) {
      r.depth++;
      if (SVO_TRACE_CELL_CACHE) r.cell = r.cell * 8u + oct;
    } else {
      r.depth = B + 2;
      w.path[0] = SVO_TRACE_CELL_CACHE ? (r.cell * 8u + oct) * 8u + octant(B + 1, r.wx, r.wy, r.wz, r.flip)
                                       : cell_index(B + 2, r.wx, r.wy, r.wz, r.flip);
    }
#endif
    return kStepOn;
  }
  // geometry below a node: the cone LOD decision (ConeDepth = -half_log2(c));
  // ConeDepth 0 compares like c = 1. Descents and ascents keep the location, so
  // the cone size computed there is reused until the next move.
  float c = 1.0f;
  if (!(kMega && r.fresh)) {
    if (r.cone < 0.0f) r.cone = cone_at(r, v.dof[0], v.dof[1]);
    c = r.cone;
  }
  if (c > pow2_neg(B + 2)) {
    r.depth = B + 2;
    return kStepHit;
  }
  if (c > pow2_neg(r.depth)) {
    r.depth--;
    if (r.depth == B + 1) {
      r.depth = B;
      if (SVO_TRACE_CELL_CACHE) r.cell = w.path[0] >> 6;  // baseLocation(B + 2) without its last two levels
    }
    return kStepOn;
  }
  if (w.cur_child == SVO_NO_CHILD) {
    // requestChild (wavefront.cl:362-375). Pixel order: the record goes to the
    // ray's pixel slot and the queue is built after the trace. Arrival order:
    // one atomic per group of requesting lanes.
    if (kStats) st.requests++;
    const uint8_t tree_size = kMega ? 1 : (c <= pow2_neg(r.depth + 1) ? 1 : 0);
    if (!kMega && a.req_stage) {
      // streaming stores: ~one record per ray, read once by the compaction,
      // and kept from evicting the tree's nodes from L2
      const uint32_t pixel = v.pixel_begin + r.id;
      uint4 *dst = reinterpret_cast<uint4 *>(a.req_stage + pixel);
      const uint64_t lx = loc_x(r), ly = loc_y(r), lz = loc_z(r);
      __stcs(dst, make_uint4((uint32_t)lx, (uint32_t)(lx >> 32), (uint32_t)ly, (uint32_t)(ly >> 32)));
      __stcs(dst + 1, make_uint4((uint32_t)lz, (uint32_t)(lz >> 32), w.cur_addr,
                                 (uint32_t)(uint8_t)r.depth | ((uint32_t)tree_size << 8)));
      __stcs(a.req_flag + pixel, (uint8_t)1);
      return kStepHit;
    }
    cg::coalesced_group g = cg::coalesced_threads();
    const uint32_t slot = claim(g, a.request_count, 1);
    if (slot < a.request_cap && a.requests) {
      svo_child_request *dst = a.requests + slot;
      svo_child_request q;
      q.address = w.cur_addr;
      q.tick = kMega ? v.tick : 0;  // TraceData.Tick is never set by the wavefront's resolveTrace
      q.depth = (uint8_t)r.depth;
      q._pad0 = 0;
      q.location[0] = loc_x(r);
      q.location[1] = loc_y(r);
      q.location[2] = loc_z(r);
      q.tree_size = tree_size;
      for (int k = 0; k < 7; k++) q._pad1[k] = 0;
      *dst = q;
    }
    return kStepHit;
  }
  if (c < pow2_neg(r.depth + 1) && lvl + 1 < a.path_levels) {
    w.path[(lvl + 1) * w.stride] = w.cur_child + octant(r.depth, r.wx, r.wy, r.wz, r.flip);
    r.depth++;
    return kStepOn;
  }
  return kStepHit;
}


// Slot `my` of the batch's ray index space: its view and pixel. Views are
// sorted by ray_begin. A tiled view's slots run over pixel tiles of 32 (tile
// width v.tile, a power of two), row of tiles by row of tiles, so the 32 slots a
// warp takes form one tile; the slots of a tile that fall outside the image are
// padding (returns false).
__device__ __forceinline__ bool ray_slot(const TraceLaunch &a, const ViewParams *s_views, uint32_t my, int &view,
                                         uint32_t &px, uint32_t &py) {
  int lo = 0, hi = a.n_views - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (s_views[mid].ray_begin <= my)
      lo = mid;
    else
      hi = mid - 1;
  }
  const ViewParams &v = s_views[lo];
  view = lo;
  const uint32_t rel = my - v.ray_begin;
  if (v.tile) {
    const uint32_t tw = v.tile, lg = (uint32_t)(__ffs((int)tw) - 1);
    const uint32_t tiles_x = (v.width + tw - 1) >> lg, t = rel >> 5, l = rel & 31u;
    py = (t / tiles_x) * (32u >> lg) + (l >> lg);
    px = (t % tiles_x) * tw + (l & (tw - 1));
    return px < v.width && py < v.height;
  }
  px = rel % v.width;
  py = rel / v.width;
  return true;
}

// setupInitialTrace's direction (wavefront.cl:566-578) of pixel (px, py):
// Facing * (cosU cosV, -sinU cosV, sinV), not normalised, from the view's
// sine/cosine tables.
__device__ __forceinline__ void ray_direction(const ViewParams &v, const float *tables, uint32_t px, uint32_t py,
                                              float &dx, float &dy, float &dz) {
  const float *tb = tables + v.table_off;
  float su = __ldg(tb + px), cu = __ldg(tb + v.width + px);
  float sv = __ldg(tb + 2 * v.width + py), cv = __ldg(tb + 2 * v.width + v.height + py);
  float m0 = __fmul_rn(cu, cv);
  float m1 = __fmul_rn(__fsub_rn(0.0f, su), cv);
  float m2 = sv;
  const float *F = v.facing;
  dx = __fadd_rn(__fadd_rn(__fmul_rn(F[0], m0), __fmul_rn(F[3], m1)), __fmul_rn(F[6], m2));
  dy = __fadd_rn(__fadd_rn(__fmul_rn(F[1], m0), __fmul_rn(F[4], m1)), __fmul_rn(F[7], m2));
  dz = __fadd_rn(__fadd_rn(__fmul_rn(F[2], m0), __fmul_rn(F[5], m1)), __fmul_rn(F[8], m2));
}

// setupInitialTrace (wavefront.cl:563-595) for ray slot `my` of the batch,
// then traceIntoVolume; a ray that misses the cube gets depth 0 (background).
// Returns false (and sets nothing else) for a padding slot. kernel.cl's
// setupInitialTrace (kernel.cl:491-522) also takes the view's DoF (use_dof).
__device__ __forceinline__ bool setup_ray(const TraceLaunch &a, const ViewParams *s_views, uint32_t my, Ray &r,
                                          bool use_dof = false) {
  int view;
  uint32_t px, py;
  if (!ray_slot(a, s_views, my, view, px, py)) return false;
  const ViewParams &v = s_views[view];
  r.view = view;
  r.id = py * v.width + px;
  ray_direction(v, a.tables, px, py, r.dx, r.dy, r.dz);
  r.ix = __frcp_rn(r.dx);
  r.iy = __frcp_rn(r.dy);
  r.iz = __frcp_rn(r.dz);
  r.sx = r.dx >= 0.0f;
  r.sy = r.dy >= 0.0f;
  r.sz = r.dz >= 0.0f;
  r.flip = (r.sx ? 0u : 1u) | (r.sy ? 0u : 2u) | (r.sz ? 0u : 4u);
  r.ox = v.origin[0];
  r.oy = v.origin[1];
  r.oz = v.origin[2];
  r.fov = v.fov_px;
  r.depth = 1;
  r.steps = 0;
  if (!(use_dof ? enter_volume(r, v.dof[0], v.dof[1]) : enter_volume(r)))
    r.depth = 0;
  else if (SVO_TRACE_CELL_CACHE)
    r.cell = cell_index(1, r.wx, r.wy, r.wz, r.flip);
  return true;
}

// The empty-octant part of a step (runBaseTrace / runBlockTrace): move to the
// neighbouring cell (traverseChunk), pop (comparePositions) and rebuild the
// cached path when an ancestor cell changed (getBlockAddress). Returns
// kStepBackground when the ray leaves the cube.
__device__ __forceinline__ int advance(const TraceLaunch &a, const uint4 *blocks, int B, Ray &r, Walk &w) {
  const bool block = r.depth > B;
  uint64_t px = r.wx, py = r.wy, pz = r.wz;
  r.cone = -1.0f;
  if (traverse(r, r.depth)) {
    // traverseChunk's clamp; the megakernel starts cones at a sky primary's exit
    if (r.wx == 0) r.wx = kAll;
    if (r.wy == 0) r.wy = kAll;
    if (r.wz == 0) r.wz = kAll;
    return kStepBackground;
  }
  int nd = pop_depth(r, r.depth, px, py, pz);
  if (block && nd >= B + 2 && (((hi32(px) ^ hi32(r.wx)) | (hi32(py) ^ hi32(r.wy)) | (hi32(pz) ^ hi32(r.wz))) >> (32 - nd)) != 0) {
    uint32_t n = cell_index(B + 2, r.wx, r.wy, r.wz, r.flip);
    w.path[0] = n;
    for (int d = B + 2; d < nd; d++) {
      uint4 n2 = load_node(blocks, a.n_blocks, n);
      n = n2.x + octant(d, r.wx, r.wy, r.wz, r.flip);
      if (!SVO_CHECK(a.error, d - B - 1 < a.path_levels, 5, (uint32_t)(d - B - 1))) return kStepBackground;
      w.path[(d - B - 1) * w.stride] = n;
    }
  }
  r.depth = nd == B + 1 ? B : nd;
  if (SVO_TRACE_CELL_CACHE && r.depth <= B) r.cell = cell_index(r.depth, r.wx, r.wy, r.wz, r.flip);
  return kStepOn;
}

// Warp-batch walks: a ray's steps that keep its location (descents, LOD
// ascents) run in an inner loop before its move (advance), so that the lanes
// of a warp whose octants turned out empty move together. Every ray takes the
// same steps in the same order either way.
#ifndef SVO_TRACE_PROBE_RUNS
#define SVO_TRACE_PROBE_RUNS 0
#endif

// One whole step.
template <bool kStats, bool kSmemBases>
__device__ __forceinline__ int step(const TraceLaunch &a, const ViewParams &v, const uint16_t *s_bases,
                                    const uint4 *blocks, int B, Ray &r, Walk &w, Stats &st) {
  const int f = probe<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
  return f == kStepEmpty ? advance(a, blocks, B, r, w) : f;
}

// Continues a ray past a hit as if the hit octant held no geometry.
__device__ __forceinline__ int step_past(const TraceLaunch &a, const uint4 *blocks, int B, Ray &r, Walk &w) {
  return advance(a, blocks, B, r, w);
}

// Sky colour of evaluateBackground (wavefront.cl:1741-1797) for a primary ray.
__device__ __forceinline__ void sky_colour(const Ray &r, uint32_t &cr, uint32_t &cg_, uint32_t &cb) {
  float dotp = __fadd_rn(__fadd_rn(__fmul_rn(r.dx, 0.0f), __fmul_rn(r.dy, 0.0f)), __fmul_rn(r.dz, -1.0f));
  if (dotp > 0.8f) {
    cr = cg_ = cb = 255;  // luminosity (uchar)(dot*200) >= 160 > 0
  } else {
    cr = 135;
    cg_ = 206;
    cb = 235;
  }
}

}  // namespace
}  // namespace svo
