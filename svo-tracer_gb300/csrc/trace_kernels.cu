// Persistent wavefront trace kernel for sm_103a.
//
// The reference runs the wavefront as one OpenCL launch per traversal step
// (init, runBaseTrace, runBlockTrace, evaluateBackground, resolveRemainders,
// drawTrace: SvoTracer.Kernel/wavefront.cl:1352-1850), compacting ray IDs into
// queues between launches and reading each queue length back to the host
// (SvoTracer.Window/MainWindow.cs:452-481). Here the passes are fused into one
// persistent launch:
//
//  * The ray queue is the batch's ray index space with a device-side head
//    counter. A persistent grid of threads takes rays from it: whenever a
//    thread finishes a ray it claims the next one, the threads of a warp that
//    need rays at the same moment sharing one atomicAdd (coalesced group,
//    `ray_chunk` rays per thread). A thread runs up to `cadence` steps of its
//    ray per pass, so the rays of a warp that finish within the same window are
//    retired and replaced together. No step depends on the warp staying
//    converged, so a lane leaves the loop as soon as the queue is drained.
//    Ray state stays in registers, so the reference's per-step reload of
//    ~74 B of SoA state disappears.
//  * Each step is runBaseTrace or runBlockTrace for one ray. The reference
//    re-walks the block tree from level B+2 at every block step
//    (getBlockAddress, wavefront.cl:296-304); here each lane keeps the node
//    addresses of its current path in shared memory. A step never leaves the
//    ancestor cell that comparePositions returns, so the cached entry is the
//    node the re-walk would reach; the kernel checks that the location bits of
//    those levels are unchanged and re-walks when they are not.
//  * Base chunks (levels 1..B) are staged in shared memory; nodes are read as
//    one 16-byte non-coherent load; comparePositions is a carry-chain count.
//  * Usage ticks are stamped once per block group visited; child requests are
//    pushed with warp-aggregated atomics into a capped queue.
//  * Shading (evaluateBackground, resolveRemainders) and drawTrace's divide are
//    applied when the ray finishes, writing the per-pixel results directly:
//    each pixel has exactly one primary ray, so its integer accumulators are
//    the ray's own contribution.
//
// Arithmetic follows the reference operation by operation with explicit
// round-to-nearest intrinsics (no contraction); ConeDepth comparisons
// (-half_log2(c) against integers) are evaluated exactly as comparisons of
// the cone size c with powers of two.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include <cstdint>
#ifdef SVO_TRACE_DEBUG
#include <cstdio>
#endif

#include "svo_internal.h"

namespace svo {
namespace {

namespace cg = cooperative_groups;

constexpr unsigned kFull = 0xffffffffu;
constexpr uint64_t kAll = ~0ull;

__constant__ uint32_t c_pow_sum[12] = {0,      8,       72,       584,       4680,       37448,
                                       299592, 2396744, 19173960, 153391688, 1227133512, 0};

__device__ __forceinline__ float ulong_to_unit(uint64_t x) { return __fmul_rn(__ull2float_rn(x), 0x1p-64f); }

// floatToUlong (wavefront.cl:200-207); out-of-range products saturate, NaN -> 0.
__device__ __forceinline__ uint64_t unit_to_ulong(float x) {
  if (x >= 0.999999911f) return kAll;
  float v = __fmul_rn(fabsf(x), 0x1p64f);
  if (v != v) return 0;
  if (!(v < 0x1p64f)) return kAll;
  return __float2ull_rz(v);
}

// roundUlong (wavefront.cl:211-221)
__device__ __forceinline__ uint64_t round_ulong(uint64_t v, int d, bool up) {
  uint64_t mask = ~(kAll >> (d + 1));
  if (up) return ((v & mask) + (0x8000000000000000ull >> d)) - v;
  uint64_t out = v - ((v & mask) - 1);
  return out >= v ? v : out;
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// baseLocation (wavefront.cl:405-411) for 1 <= depth <= 10.
__device__ __forceinline__ uint32_t cell_index(int depth, uint64_t x, uint64_t y, uint64_t z) {
  int s = 64 - depth;
  return spread3((uint32_t)(x >> s)) | (spread3((uint32_t)(y >> s)) << 1) | (spread3((uint32_t)(z >> s)) << 2);
}

// chunkPosition (wavefront.cl:428-430)
__device__ __forceinline__ uint32_t octant(int depth, uint64_t x, uint64_t y, uint64_t z) {
  int s = 63 - depth;
  return (uint32_t)(((x >> s) & 1) | (((y >> s) & 1) << 1) | (((z >> s) & 1) << 2));
}

__device__ __forceinline__ float pow2_neg(int k) { return __int_as_float((127 - k) << 23); }

struct Ray {
  uint64_t lx, ly, lz;
  float dx, dy, dz;
  float ix, iy, iz;
  float ox, oy, oz;
  float fov;
  uint32_t id;   // pixel index within its view
  int view;
  int depth;
  int steps;
  bool sx, sy, sz;
};

struct Node {
  uint32_t child;
  uint32_t chunk;
};

__device__ __forceinline__ uint4 load_node(const uint4 *blocks, uint32_t n_blocks, uint32_t addr) {
  if (addr >= n_blocks) return make_uint4(0, 0, 0, 0);
  return __ldg(blocks + addr);
}

// traverseChunk (wavefront.cl:440-497) without the trailing setConeDepth.
__device__ __forceinline__ void traverse(Ray &r, int depth) {
  uint64_t d0 = round_ulong(r.lx, depth, r.sx);
  uint64_t d1 = round_ulong(r.ly, depth, r.sy);
  uint64_t d2 = round_ulong(r.lz, depth, r.sz);
  float a0 = fabsf(__fmul_rn(__ull2float_rn(d0), r.ix));
  float a1 = fabsf(__fmul_rn(__ull2float_rn(d1), r.iy));
  float a2 = fabsf(__fmul_rn(__ull2float_rn(d2), r.iz));
  int ax = (a0 <= a1 && a0 <= a2) ? 0 : ((a1 <= a0 && a1 <= a2) ? 1 : 2);
  float inv = ax == 0 ? r.ix : (ax == 1 ? r.iy : r.iz);
  float u = ulong_to_unit(ax == 0 ? d0 : (ax == 1 ? d1 : d2));
  if (ax != 0) d0 = unit_to_ulong(__fmul_rn(__fmul_rn(r.dx, inv), u));
  if (ax != 1) d1 = unit_to_ulong(__fmul_rn(__fmul_rn(r.dy, inv), u));
  if (ax != 2) d2 = unit_to_ulong(__fmul_rn(__fmul_rn(r.dz, inv), u));
  uint64_t x = r.sx ? r.lx + d0 : r.lx - d0;
  uint64_t y = r.sy ? r.ly + d1 : r.ly - d1;
  uint64_t z = r.sz ? r.lz + d2 : r.lz - d2;
  if (r.sx && x == 0) x = kAll; else if (!r.sx && x == kAll) x = 0;
  if (r.sy && y == 0) y = kAll; else if (!r.sy && y == kAll) y = 0;
  if (r.sz && z == 0) z = kAll; else if (!r.sz && z == kAll) z = 0;
  r.lx = x;
  r.ly = y;
  r.lz = z;
}

// comparePositions (wavefront.cl:413-426): the loop pops one level for every
// consecutive level, counted upwards from `depth`, whose octant bit flipped
// against the travel direction on some axis; it stops at level 1.
__device__ __forceinline__ int pop_depth(const Ray &r, int depth, uint64_t px, uint64_t py, uint64_t pz) {
  uint64_t m = (r.sx ? (px & ~r.lx) : (~px & r.lx)) | (r.sy ? (py & ~r.ly) : (~py & r.ly)) |
               (r.sz ? (pz & ~r.lz) : (~pz & r.lz));
  uint64_t run = ~(m >> (63 - depth));
  int ones = __ffsll((long long)run) - 1;
  return ones < depth ? depth - ones : 1;
}

__device__ __forceinline__ bool leaving(const Ray &r) {
  return (!r.sx && r.lx == 0) || (!r.sy && r.ly == 0) || (!r.sz && r.lz == 0) || (r.sx && r.lx == kAll) ||
         (r.sy && r.ly == kAll) || (r.sz && r.lz == kAll);
}

// coneSize (wavefront.cl:387-391) at the distance setConeDepth uses (:394-399).
__device__ __forceinline__ float cone_at(const Ray &r, float dof0, float dof1) {
  float x = __fsub_rn(r.ox, ulong_to_unit(r.lx));
  float y = __fsub_rn(r.oy, ulong_to_unit(r.ly));
  float z = __fsub_rn(r.oz, ulong_to_unit(r.lz));
  float m = fabsf(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z))));
  float eye = __fmul_rn(r.fov, m);
  float f = fabsf(__fmul_rn(dof0, __fsub_rn(dof1, m)));
  return eye < f ? f : eye;
}

// traceIntoVolume (wavefront.cl:639-1088): enter the unit cube on the face of
// the outside slab with the largest entry distance (ties x, then y); reject
// when the entry point is outside the cube grown by the cone size.
__device__ __forceinline__ bool enter_volume(Ray &r) {
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
    r.lx = unit_to_ulong(o[0]);
    r.ly = unit_to_ulong(o[1]);
    r.lz = unit_to_ulong(o[2]);
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
  r.lx = unit_to_ulong(p[0]);
  r.ly = unit_to_ulong(p[1]);
  r.lz = unit_to_ulong(p[2]);
  // DoF of a fresh TraceData is zero (setupInitialTrace leaves it unset).
  float eye = __fmul_rn(r.fov, m);
  float f = fabsf(__fmul_rn(0.0f, __fsub_rn(0.0f, m)));
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

// Per-thread traversal state besides the ray itself.
struct Walk {
  uint32_t *path;  // path[level * stride]: node address of each level below B+2
  int stride;
  uint32_t cur_addr, cur_child, cur_chunk;  // last node read
  uint32_t last_group;                      // last usage group stamped
  uint32_t v_block, v_base;                 // reference-walk counters (stats launches)
};

enum : int { kStepOn = 0, kStepBackground = 1, kStepHit = 2 };

// One runBaseTrace (wavefront.cl:1400-1463) or runBlockTrace (:1465-1566) step.
// Both read a 2-bit octant pair from a chunk (a base chunk or the current
// node's) and share the empty-octant stepping code, so lanes at base and block
// levels run it together.
template <bool kStats, bool kSmemBases>
__device__ __forceinline__ int step(const TraceLaunch &a, const ViewParams &v, const uint16_t *s_bases,
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
    uint32_t idx = c_pow_sum[r.depth - 1] + cell_index(r.depth, r.lx, r.ly, r.lz);
    chunk = kSmemBases ? s_bases[idx] : __ldg(a.bases + idx);
    if (kStats) w.v_base++;
  } else {
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
  if (((chunk >> (octant(r.depth, r.lx, r.ly, r.lz) * 2)) & 2) == 0) {
    // empty octant: step to the neighbouring cell and pop (traverseChunk, comparePositions)
    uint64_t px = r.lx, py = r.ly, pz = r.lz;
    traverse(r, r.depth);
    if (leaving(r)) return kStepBackground;
    int nd = pop_depth(r, r.depth, px, py, pz);
    if (block && nd >= B + 2 && (((px ^ r.lx) | (py ^ r.ly) | (pz ^ r.lz)) >> (64 - nd)) != 0) {
      // an ancestor cell changed: rebuild the path like getBlockAddress
      uint32_t n = cell_index(B + 2, r.lx, r.ly, r.lz);
      w.path[0] = n;
      for (int d = B + 2; d < nd; d++) {
        uint4 n2 = load_node(blocks, a.n_blocks, n);
        n = n2.x + octant(d, r.lx, r.ly, r.lz);
        w.path[(d - B - 1) * w.stride] = n;
      }
    }
    r.depth = nd == B + 1 ? B : nd;
    return kStepOn;
  }
  if (!block) {
    // geometry below a base cell: descend, jumping from level B to B+2
    if (r.depth < B) {
      r.depth++;
    } else {
      r.depth = B + 2;
      w.path[0] = cell_index(B + 2, r.lx, r.ly, r.lz);
    }
    return kStepOn;
  }
  // geometry below a node: the cone LOD decision (ConeDepth = -half_log2(c))
  float c = cone_at(r, v.dof[0], v.dof[1]);
  if (c > pow2_neg(B + 2)) {
    r.depth = B + 2;
    return kStepHit;
  }
  if (c > pow2_neg(r.depth)) {
    r.depth--;
    if (r.depth == B + 1) r.depth = B;
    return kStepOn;
  }
  if (w.cur_child == SVO_NO_CHILD) {
    // requestChild (wavefront.cl:362-375): one atomic per group of requesting lanes
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t slot = claim(g, a.request_count, 1);
    if (kStats) st.requests++;
    if (slot < a.request_cap && a.requests) {
      svo_child_request q;
      q.address = w.cur_addr;
      q.tick = 0;  // TraceData.Tick is never set by resolveTrace
      q.depth = (uint8_t)r.depth;
      q._pad0 = 0;
      q.location[0] = r.lx;
      q.location[1] = r.ly;
      q.location[2] = r.lz;
      q.tree_size = c <= pow2_neg(r.depth + 1) ? 1 : 0;
      for (int k = 0; k < 7; k++) q._pad1[k] = 0;
      a.requests[slot] = q;
    }
    return kStepHit;
  }
  if (c < pow2_neg(r.depth + 1) && lvl + 1 < a.path_levels) {
    w.path[(lvl + 1) * w.stride] = w.cur_child + octant(r.depth, r.lx, r.ly, r.lz);
    r.depth++;
    return kStepOn;
  }
  return kStepHit;
}

template <bool kStats, bool kSmemBases>
#ifndef SVO_TRACE_MIN_CTAS
#define SVO_TRACE_MIN_CTAS 1
#endif
__global__ void __launch_bounds__(256, SVO_TRACE_MIN_CTAS) trace_kernel(const TraceLaunch a) {
  extern __shared__ __align__(16) uint8_t smem[];
  ViewParams *s_views = reinterpret_cast<ViewParams *>(smem);
  uint16_t *s_bases = reinterpret_cast<uint16_t *>(smem + a.n_views * sizeof(ViewParams));
  size_t bases_bytes = kSmemBases ? ((a.n_bases * 2 + 15) & ~15u) : 0;
  uint32_t *s_path = reinterpret_cast<uint32_t *>(smem + a.n_views * sizeof(ViewParams) + bases_bytes);

  {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(a.views);
    uint32_t *dst = reinterpret_cast<uint32_t *>(s_views);
    for (uint32_t i = threadIdx.x; i < a.n_views * sizeof(ViewParams) / 4; i += blockDim.x) dst[i] = src[i];
    if (kSmemBases)
      for (uint32_t i = threadIdx.x; i < a.n_bases; i += blockDim.x) s_bases[i] = __ldg(a.bases + i);
  }
  __syncthreads();

  const int B = a.base_depth;
  const uint4 *blocks = reinterpret_cast<const uint4 *>(a.blocks);
  const uint32_t chunk = a.ray_chunk;
  const int cadence = a.cadence;

  Stats st = {0, 0, 0, 0, 0, 0, 0};
  Walk w;
  w.path = s_path + threadIdx.x;
  w.stride = blockDim.x;
  w.cur_addr = kFull;
  w.cur_child = 0;
  w.cur_chunk = 0;
  w.last_group = kFull;
  w.v_block = 0;
  w.v_base = 0;
  Ray r;
  r.depth = 0;
  r.steps = 0;
  r.view = 0;
  bool have = false;
  uint32_t ray_global = 0, next_ray = 0, left_in_chunk = 0, chunk_stride = 0;
  // Every pass either starts a ray or advances it by at least one step, so a
  // thread runs at most total_rays * (max_steps + 2) + 64 passes; past that
  // bound it records its state and stops instead of spinning.
  const unsigned long long iter_limit =
      (unsigned long long)a.total_rays * (unsigned long long)(a.max_steps + 2) + 64;
  unsigned long long iters = 0;

  for (;;) {
    if (++iters > iter_limit) {
      if (a.error && atomicCAS(a.error, 0u, (unsigned)SVO_ERR_TIMEOUT) == 0u) {
        a.error[1] = blockIdx.x;
        a.error[2] = threadIdx.x;
        a.error[3] = ray_global;
        a.error[4] = (uint32_t)r.depth;
        a.error[5] = (uint32_t)r.steps;
      }
      break;
    }
    if (!have) {
      // ---- take the next ray from the queue --------------------------------
      uint32_t my;
      if (left_in_chunk == 0) {
        // one atomic per group of idle lanes: each lane gets `chunk` rays,
        // interleaved so that lanes of a group hold neighbouring pixels
        cg::coalesced_group g = cg::coalesced_threads();
        uint32_t first = claim(g, a.ray_counter, chunk);
        chunk_stride = g.size();
        my = first;
        next_ray = first + chunk_stride;
        left_in_chunk = chunk - 1;
      } else {
        my = next_ray;
        next_ray += chunk_stride;
        left_in_chunk--;
      }
      // later rays of this chunk, and every later claim, are larger still
      if (my >= a.total_rays) break;  // queue drained
      ray_global = my;
      int lo = 0, hi = a.n_views - 1;  // views are sorted by ray_begin
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (s_views[mid].ray_begin <= my)
          lo = mid;
        else
          hi = mid - 1;
      }
      const ViewParams &v = s_views[lo];
      r.view = lo;
      r.id = my - v.ray_begin;
      uint32_t px = r.id % v.width, py = r.id / v.width;
      const float *tb = a.tables + v.table_off;
      float su = __ldg(tb + px), cu = __ldg(tb + v.width + px);
      float sv = __ldg(tb + 2 * v.width + py), cv = __ldg(tb + 2 * v.width + v.height + py);
      // setupInitialTrace (wavefront.cl:563-595)
      float m0 = __fmul_rn(cu, cv);
      float m1 = __fmul_rn(__fsub_rn(0.0f, su), cv);
      float m2 = sv;
      const float *F = v.facing;
      r.dx = __fadd_rn(__fadd_rn(__fmul_rn(F[0], m0), __fmul_rn(F[3], m1)), __fmul_rn(F[6], m2));
      r.dy = __fadd_rn(__fadd_rn(__fmul_rn(F[1], m0), __fmul_rn(F[4], m1)), __fmul_rn(F[7], m2));
      r.dz = __fadd_rn(__fadd_rn(__fmul_rn(F[2], m0), __fmul_rn(F[5], m1)), __fmul_rn(F[8], m2));
      r.ix = __frcp_rn(r.dx);
      r.iy = __frcp_rn(r.dy);
      r.iz = __frcp_rn(r.dz);
      r.sx = r.dx >= 0.0f;
      r.sy = r.dy >= 0.0f;
      r.sz = r.dz >= 0.0f;
      r.ox = v.origin[0];
      r.oy = v.origin[1];
      r.oz = v.origin[2];
      r.fov = v.fov_px;
      r.depth = 1;
      r.steps = 0;
      w.v_block = 0;
      w.v_base = 0;
      w.cur_addr = kFull;
      w.last_group = kFull;
      have = true;
      if (!enter_volume(r)) r.depth = 0;  // background at once
    }

    // ---- up to `cadence` traversal steps; retire finished rays together -------
    const ViewParams &v = s_views[r.view];
    int finish = kStepOn;
    for (int k = 0; k < cadence && finish == kStepOn; k++)
      finish = step<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
    if (finish == kStepOn) continue;

    // evaluateBackground / resolveRemainders + drawTrace
    uint32_t hit_index = SVO_MISS, cr, cg_, cb;
    uint8_t hit_depth = 0;
    float t = __int_as_float(0x7f800000);
    if (finish == kStepHit) {
      uint32_t addr = w.path[(r.depth - B - 2) * w.stride];
      uint4 nd = load_node(blocks, a.n_blocks, addr);
      hit_index = addr;
      hit_depth = (uint8_t)r.depth;
      cr = (nd.z >> 16) & 0xffu;
      cg_ = nd.z >> 24;
      cb = nd.w & 0xffu;
      float x = __fsub_rn(ulong_to_unit(r.lx), r.ox);
      float y = __fsub_rn(ulong_to_unit(r.ly), r.oy);
      float z = __fsub_rn(ulong_to_unit(r.lz), r.oz);
      t = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
      if (kStats) {
        w.v_block += (uint32_t)(r.depth - B - 1);
        st.hits++;
      }
    } else {
      float dotp = __fadd_rn(__fadd_rn(__fmul_rn(r.dx, 0.0f), __fmul_rn(r.dy, 0.0f)), __fmul_rn(r.dz, -1.0f));
      if (dotp > 0.8f) {
        cr = cg_ = cb = 255;  // luminosity (uchar)(dot*200) >= 160 > 0
      } else {
        cr = 135;
        cg_ = 206;
        cb = 235;
      }
    }
    const float fw = 65025.0f;  // (float)255 * 255.0f
    float4 px;
    px.x = fminf(__fdiv_rn(__uint2float_rn(cr * 255u), fw), 1.0f);
    px.y = fminf(__fdiv_rn(__uint2float_rn(cg_ * 255u), fw), 1.0f);
    px.z = fminf(__fdiv_rn(__uint2float_rn(cb * 255u), fw), 1.0f);
    px.w = 1.0f;
    if (v.hit_index) v.hit_index[r.id] = hit_index;
    if (v.hit_depth) v.hit_depth[r.id] = hit_depth;
    if (v.t) v.t[r.id] = t;
    if (v.rgba) reinterpret_cast<float4 *>(v.rgba)[r.id] = px;
    if (kStats) {
      st.rays++;
      st.base_steps += w.v_base;
      st.block_reads += w.v_block;
      if (a.ray_v_block) a.ray_v_block[ray_global] = w.v_block;
      if (a.ray_v_base) a.ray_v_base[ray_global] = w.v_base;
    }
    have = false;
  }

  if (kStats && a.stats) {
    unsigned long long vals[7] = {st.rays, st.hits, st.base_steps, st.block_reads, st.block_steps, st.requests,
                                  st.limited};
    cg::coalesced_group g = cg::coalesced_threads();
#pragma unroll
    for (int k = 0; k < 7; k++) {
      unsigned long long x = cg::reduce(g, vals[k], cg::plus<unsigned long long>());
      if (g.thread_rank() == 0 && x) atomicAdd(a.stats + k, x);
    }
  }
}

}  // namespace

size_t trace_smem_bytes(const TraceLaunch &a, bool bases_in_smem) {
  size_t b = (size_t)a.n_views * sizeof(ViewParams);
  if (bases_in_smem) b += ((size_t)a.n_bases * 2 + 15) & ~(size_t)15;
  b += (size_t)a.path_levels * a.block_size * 4;
  return b;
}

static bool bases_fit(const TraceLaunch &a) { return (size_t)a.n_bases * 2 <= 96 * 1024; }

template <bool S, bool M>
static cudaError_t launch_one(const TraceLaunch &a, size_t smem, cudaStream_t stream) {
  auto k = trace_kernel<S, M>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.grid, a.block_size, smem, stream>>>(a);
  return cudaGetLastError();
}

int trace_occupancy(const TraceLaunch &a, bool with_stats) {
  bool m = bases_fit(a);
  size_t smem = trace_smem_bytes(a, m);
  int n = 0;
  const void *k = with_stats ? (m ? (const void *)trace_kernel<true, true> : (const void *)trace_kernel<true, false>)
                             : (m ? (const void *)trace_kernel<false, true> : (const void *)trace_kernel<false, false>);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, a.block_size, smem) != cudaSuccess) return 0;
  return n;
}

svo_status launch_trace(const TraceLaunch &a, bool with_stats, void *stream) {
  bool m = bases_fit(a);
  size_t smem = trace_smem_bytes(a, m);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (with_stats)
    e = m ? launch_one<true, true>(a, smem, s) : launch_one<true, false>(a, smem, s);
  else
    e = m ? launch_one<false, true>(a, smem, s) : launch_one<false, false>(a, smem, s);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("trace kernel launch: ") + cudaGetErrorString(e));
  return SVO_OK;
}

}  // namespace svo
