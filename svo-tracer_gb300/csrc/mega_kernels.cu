// The megakernel path for sm_103a: kernel.cl's `trace` (SvoTracer.Kernel/
// kernel.cl:1531-1558), which runs per pixel a primary cone, spawnRays's fan of
// secondary cones from its end point (:1115-1253) and draw (:1264-1275).
//
// One OpenCL work-item per pixel runs ~20 dependent traces in a row; here the
// pixel's work is split into kernels over the view's 4x8 pixel tiles, so
// that a warp always steps 32 cones that start close together and point the
// same way:
//  1. mega_primary_kernel: the primary cone of every pixel, the persistent
//     warp-batch traversal of trace_kernels.cu with kernel.cl's differences
//     (DoF at the volume entry, ConeDepth 0 until the first move, requests with
//     the frame's Tick and TreeSize 1), ending in a MegaPixel record.
//  2. mega_fan_kernel: spawnRays for each pixel: cone directions and
//     weightings in generation order, stored [tile][cone k][lane], and the
//     cones' common start (traverseChunkNormal, the same for every cone of a
//     pixel).
//  3. mega_scan_kernel / mega_emit_kernel: the band's cones compacted into one
//     list, tile by tile, cone k of the tile's pixels before cone k + 1; then
//     mega_cone_kernel: every cone traced to a surface or the sky, a warp
//     taking 32 consecutive entries of the list.
//  4. mega_resolve_kernel: writeToAccumulator in generation order, then draw.
// The cone slots of a frame are processed in bands of tiles so that their
// memory stays bounded for any cone schedule.
//
// Every float operation is one IEEE round-to-nearest operation in kernel.cl's
// order (no contraction). The trigonometry of the fan is per-launch constants
// and a table over the 65536 int16 normal angles, (float)sin((double)x) on the
// host like the ray-setup tables; normalize of a zero vector is that vector.
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mega_internal.h"
#include "trace_core.cuh"
#include "fan.cuh"

namespace svo {
namespace {

#ifndef SVO_MEGA_MIN_CTAS
#define SVO_MEGA_MIN_CTAS 4
#endif

__device__ __forceinline__ size_t cone_slot(const MegaLaunch &m, uint32_t tile_in_band, uint32_t k, uint32_t lane) {
  return ((size_t)tile_in_band * (uint32_t)m.k_max + k) * 32u + lane;
}

// roundUlong (kernel.cl:240-251) in real coordinates.
__device__ __forceinline__ uint64_t round_ulong(uint64_t v, int depth, bool up) {
  const uint64_t keep = kAll - (kAll >> (depth + 1));
  if (up) return ((v & keep) + ((kAll - (kAll >> 1)) >> depth)) - v;
  const uint64_t out = v - ((v & keep) - 1);
  return out >= v ? v : out;
}

// traverseChunkNormal (kernel.cl:428-489): one level-`depth` cell along the
// normal, the axis of the largest distance chosen.
__device__ __forceinline__ void step_normal(int depth, const float n[3], uint64_t loc[3]) {
  bool s[3];
  float inv[3], a[3];
  uint64_t d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s[k] = n[k] >= 0.0f;
    inv[k] = __frcp_rn(n[k]);
    d[k] = round_ulong(loc[k], depth, s[k]);
    a[k] = fabsf(__fmul_rn(ulong_to_float(d[k]), inv[k]));
  }
  const int ax = (a[0] >= a[1] && a[0] >= a[2]) ? 0 : ((a[1] >= a[0] && a[1] >= a[2]) ? 1 : 2);
  const float u = __fmul_rn(ulong_to_float(d[ax]), 0x1p-64f);
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (k != ax) d[k] = unit_to_ulong(__fmul_rn(__fmul_rn(n[k], inv[ax]), u));
#pragma unroll
  for (int k = 0; k < 3; k++) {
    uint64_t v = s[k] ? loc[k] + d[k] : loc[k] - d[k];
    if (s[k] && v == 0)
      v = kAll;
    else if (!s[k] && v == kAll)
      v = 0;
    loc[k] = v;
  }
}

// resolveBackgroundRayData (kernel.cl:1225-1240). `dotprod > 0.8` compares with
// a double constant; the smallest float above 0.8 is 0.8f.
__device__ __forceinline__ void sky_light(float dx, float dy, float dz, uint32_t &r, uint32_t &g, uint32_t &b,
                                          float &lum) {
  const float dotp = dot3(dx, dy, dz, 0.0f, 0.0f, -1.0f);
  if (dotp >= 0.8f) {
    r = g = b = 255;
    lum = __fmul_rn(dotp, 150.0f);
  } else {
    r = 135;
    g = 206;
    b = 235;
    lum = 10.0f;
  }
}

// Shared-memory prologue of the tracing kernels (view, base chunks, path
// cache, Morton table); zero_dof clears the view's DoF (setupTrace's cones).
template <bool kSmemBases>
__device__ __forceinline__ void stage_shared(const TraceLaunch &a, uint8_t *smem, ViewParams *&s_views,
                                             uint16_t *&s_bases, uint32_t *&s_path, bool zero_dof) {
  s_views = reinterpret_cast<ViewParams *>(smem);
  s_bases = reinterpret_cast<uint16_t *>(smem + a.n_views * sizeof(ViewParams));
  const size_t bases_bytes = kSmemBases ? ((a.n_bases * 2 + 15) & ~15u) : 0;
  s_path = reinterpret_cast<uint32_t *>(smem + a.n_views * sizeof(ViewParams) + bases_bytes);
  const uint32_t *src = reinterpret_cast<const uint32_t *>(a.views);
  uint32_t *dst = reinterpret_cast<uint32_t *>(s_views);
  for (uint32_t i = threadIdx.x; i < a.n_views * sizeof(ViewParams) / 4; i += blockDim.x) dst[i] = src[i];
  if (kSmemBases)
    for (uint32_t i = threadIdx.x; i < a.n_bases; i += blockDim.x) s_bases[i] = __ldg(a.bases + i);
  fill_spread_table();
  __syncthreads();
  if (zero_dof && threadIdx.x == 0) {
    s_views[0].dof[0] = 0.0f;
    s_views[0].dof[1] = 0.0f;
  }
  __syncthreads();
}

__device__ __forceinline__ void reset_walk(Walk &w) {
  w.cur_addr = kFull;
  w.cur_child = 0;
  w.cur_chunk = 0;
  w.last_group = kFull;
  w.v_block = 0;
  w.v_base = 0;
}

// True once a kernel of this call (or an earlier unreported one) recorded an
// error: the kernels after the primary one then return at entry, so none of them
// reads the pixel records of warps that stopped early. Nothing writes the record
// while the fan, scan, emit and resolve kernels run, so every thread of one of
// those launches reads the same value (the scan kernel's __syncthreads stay
// uniform).
__device__ __forceinline__ bool call_stopped(const MegaLaunch &m) {
  return m.t.error && *reinterpret_cast<const volatile uint32_t *>(m.t.error) != 0u;
}

__device__ __forceinline__ void record_timeout(const TraceLaunch &a, uint32_t item, const Ray &r) {
  if (a.error && atomicCAS(a.error, 0u, (unsigned)SVO_ERR_TIMEOUT) == 0u) {
    a.error[1] = blockIdx.x;
    a.error[2] = threadIdx.x;
    a.error[3] = item;
    a.error[4] = (uint32_t)r.depth;
    a.error[5] = (uint32_t)r.steps;
  }
}

// Runs a cone to its end: kStepHit at a surface, kStepBackground in the sky;
// false when its step count reached the pass bound (max_steps + 2, which only a
// fault reaches, or the launch's pass_limit) before it ended. kStats: the
// cone's reference-walk counters (V_block, V_base) and its hit go to st.
template <bool kSmemBases, bool kStats>
__device__ __forceinline__ bool run_cone(const TraceLaunch &a, const ViewParams &v, const uint16_t *s_bases,
                                         const uint4 *blocks, int B, Ray &r, Walk &w, int &finish, Stats &st) {
  const uint32_t limit = a.pass_limit ? a.pass_limit : (uint32_t)a.max_steps + 2u;
  finish = kStepOn;
  while (finish == kStepOn) {
    if ((uint32_t)r.steps >= limit) return false;  // every pass takes a step or ends the cone
    finish = probe<kStats, kSmemBases, true>(a, v, s_bases, blocks, B, r, w, st);
    if (SVO_TRACE_PROBE_RUNS)
      while (finish == kStepOn) {
        if ((uint32_t)r.steps >= limit) return false;
        finish = probe<kStats, kSmemBases, true>(a, v, s_bases, blocks, B, r, w, st);
      }
    if (finish == kStepEmpty) {
      finish = advance(a, blocks, B, r, w);
      r.fresh = false;
    }
  }
  if (kStats) {
    st.rays++;
    st.block_reads += w.v_block;
    st.base_steps += w.v_base;
    if (finish == kStepHit) st.hits++;
  }
  return true;
}

// Adds a thread's counters to the launch's statistics (svo_trace_stats order).
__device__ __forceinline__ void flush_stats(const TraceLaunch &a, const Stats &st) {
  if (!a.stats) return;
  unsigned long long vals[7] = {st.rays, st.hits, st.base_steps, st.block_reads, st.block_steps, st.requests,
                                st.limited};
  cg::coalesced_group g = cg::coalesced_threads();
#pragma unroll
  for (int k = 0; k < 7; k++) {
    unsigned long long x = cg::reduce(g, vals[k], cg::plus<unsigned long long>());
    if (g.thread_rank() == 0 && x) atomicAdd(a.stats + k, x);
  }
}

template <bool kSmemBases, bool kStats>
__global__ void __launch_bounds__(256, SVO_MEGA_MIN_CTAS) mega_primary_kernel(const MegaLaunch m) {
  extern __shared__ __align__(16) uint8_t smem[];
  const TraceLaunch &a = m.t;
  ViewParams *s_views;
  uint16_t *s_bases;
  uint32_t *s_path;
  stage_shared<kSmemBases>(a, smem, s_views, s_bases, s_path, false);
  const int B = a.base_depth;
  const uint4 *blocks = reinterpret_cast<const uint4 *>(a.blocks);
  const ViewParams &v = s_views[0];
  Walk w;
  w.path = s_path + threadIdx.x;
  w.stride = blockDim.x;
  Ray r;
  const uint32_t lane = threadIdx.x & 31u;
  bool timed_out = false;
  unsigned long long surfaces = 0;
  Stats st = {0, 0, 0, 0, 0, 0, 0};
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(a.ray_counter, 32u);
    base = __shfl_sync(kFull, base, 0);
    if (base >= a.total_rays) break;
    const uint32_t my = base + lane;
    if (my < a.total_rays && !timed_out) {
      MegaPixel P;
      P.n_cones = 0;
      P._pad = 0;
      P.node = SVO_MISS;
      if (!setup_ray(a, s_views, my, r, true)) {
        P.kind = kMegaPad;
        P.id = 0;
        P.depth = 0;
      } else {
        reset_walk(w);
        r.fresh = true;
        const bool entered = r.depth != 0;
        int finish;
        if (!run_cone<kSmemBases, kStats>(a, v, s_bases, blocks, B, r, w, finish, st)) {
          record_timeout(a, my, r);
          timed_out = true;
        }
        P.id = r.id;
        P.dir[0] = r.dx;
        P.dir[1] = r.dy;
        P.dir[2] = r.dz;
        P.loc[0] = loc_x(r);
        P.loc[1] = loc_y(r);
        P.loc[2] = loc_z(r);
        uint32_t hit_index = SVO_MISS;
        uint8_t hit_depth = 0;
        float t = __int_as_float(0x7f800000);
        if (!entered) {
          P.kind = kMegaMiss;
          P.depth = 1;
        } else if (finish == kStepHit) {
          // resolveRayData: the block, RayLength = length(Location - Origin)
          P.kind = kMegaSurface;
          P.depth = (uint8_t)r.depth;
          P.node = SVO_CHECK(a.error, r.depth - B - 2 >= 0 && r.depth - B - 2 < a.path_levels, 8,
                             (uint32_t)(r.depth - B - 2))
                       ? w.path[(r.depth - B - 2) * w.stride]
                       : SVO_MISS;
          hit_index = P.node;
          hit_depth = (uint8_t)r.depth;
          const float x = __fsub_rn(ulong_to_unit(P.loc[0]), r.ox);
          const float y = __fsub_rn(ulong_to_unit(P.loc[1]), r.oy);
          const float z = __fsub_rn(ulong_to_unit(P.loc[2]), r.oz);
          t = __fsqrt_rn(dot3(x, y, z, x, y, z));
          surfaces++;
        } else {
          P.kind = kMegaSky;
          P.depth = 1;
        }
        if (v.hit_index) v.hit_index[r.id] = hit_index;
        if (v.hit_depth) v.hit_depth[r.id] = hit_depth;
        if (v.t) v.t[r.id] = t;
      }
      m.pix[my] = P;
    }
    if (__any_sync(kFull, timed_out)) break;
  }
  surfaces = __reduce_add_sync(kFull, (unsigned)surfaces);
  if (lane == 0 && surfaces) atomicAdd(m.totals + 1, surfaces);
  if (kStats) flush_stats(a, st);
}

// spawnRays for one slot of the band; one warp per tile.
__global__ void __launch_bounds__(256) mega_fan_kernel(const MegaLaunch m) {
  if (call_stopped(m)) return;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t tile = gid >> 5, lane = gid & 31u;
  uint32_t count = 0;
  if (tile < m.band_tiles) {
    const size_t slot = ((size_t)m.band_tile0 + tile) * 32u + lane;
    MegaPixel P = m.pix[slot];
    if (P.kind == kMegaSky || P.kind == kMegaSurface) {
      float n[3] = {0.0f, 0.0f, 0.0f};
      if (P.kind == kMegaSurface)
        block_normal(m.normal_sc, load_node(reinterpret_cast<const uint4 *>(m.t.blocks), m.t.n_blocks, P.node), n);
      spawn_fan(n, P.dir[0], P.dir[1], P.dir[2], m.fov_c, m.weighting_c, m.spine, m.n_spines, m.ring,
                [&](float x, float y, float z, float wgt, int s) {
                  const size_t i = cone_slot(m, tile, count, lane);
                  m.cone_dw[i] = make_float4(x, y, z, __fmul_rn(wgt, 1.0f));  // ringWeighting * baseWeighting
                  m.cone_s[i] = (uint16_t)s;
                  count++;
                });
      // setupTrace (kernel.cl:524-544): Origin from the end location, then one
      // cell along the normal
#pragma unroll
      for (int k = 0; k < 3; k++) P.origin[k] = ulong_to_unit(P.loc[k]);
      step_normal(P.depth, n, P.loc);
      P.n_cones = (uint16_t)count;
      MegaPixel *dst = m.pix + slot;
      dst->loc[0] = P.loc[0];
      dst->loc[1] = P.loc[1];
      dst->loc[2] = P.loc[2];
      dst->origin[0] = P.origin[0];
      dst->origin[1] = P.origin[1];
      dst->origin[2] = P.origin[2];
      dst->n_cones = P.n_cones;
    }
  }
  const uint32_t total = __reduce_add_sync(kFull, count);
  if (lane == 0 && tile < m.band_tiles) {
    m.tile_cones[tile] = total;
    if (total) atomicAdd(m.totals, (unsigned long long)total);
  }
}

// Exclusive scan of the band's per-tile cone counts (one CTA), total to queue[1].
__global__ void __launch_bounds__(1024) mega_scan_kernel(const MegaLaunch m) {
  __shared__ uint32_t part[1024];
  if (call_stopped(m)) return;
  const uint32_t n = m.band_tiles;
  const uint32_t per = (n + 1023u) / 1024u, b = threadIdx.x * per, e = min(n, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; i++) s += m.tile_cones[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t off = 1; off < 1024u; off <<= 1) {
    const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - s;
  for (uint32_t i = b; i < e; i++) {
    const uint32_t c = m.tile_cones[i];
    m.tile_cones[i] = run;
    run += c;
  }
  if (threadIdx.x == 1023) {
    m.queue[0] = 0;
    m.queue[1] = min(part[1023], m.max_entries);
  }
}

// The compacted cone list: per tile (one warp), cone k of every pixel that has
// one, k = 0, 1, ... (neighbouring entries start close together and point alike).
__global__ void __launch_bounds__(256) mega_emit_kernel(const MegaLaunch m) {
  if (call_stopped(m)) return;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t tile = gid >> 5, lane = gid & 31u;
  if (tile >= m.band_tiles) return;  // whole warps
  const MegaPixel &P = m.pix[((size_t)m.band_tile0 + tile) * 32u + lane];
  // only fans of this call count (bounded by the slot stride)
  const uint32_t count =
      (P.kind == kMegaSky || P.kind == kMegaSurface) ? min((uint32_t)P.n_cones, (uint32_t)m.k_max) : 0u;
  const uint32_t kmax = __reduce_max_sync(kFull, count);
  uint32_t base = m.tile_cones[tile];
  const uint32_t below = (1u << lane) - 1u;
  for (uint32_t k = 0; k < kmax; k++) {
    const uint32_t b = __ballot_sync(kFull, k < count);
    const uint32_t at = base + __popc(b & below);
    if (k < count && at < m.max_entries) m.entries[at] = (uint32_t)cone_slot(m, tile, k, lane);
    base += __popc(b);
  }
}

// setupTrace (kernel.cl:524-544) of the cone in slot `e` of the band.
__device__ __forceinline__ void start_cone(const MegaLaunch &m, uint32_t e, Ray &r, Walk &w) {
  const uint32_t lane = e & 31u, tk = e >> 5, K = (uint32_t)m.k_max;
  const uint32_t tile = tk / K;
  const MegaPixel *P = m.pix + ((size_t)m.band_tile0 + tile) * 32u + lane;
  const float4 dw = m.cone_dw[e];
  const uint32_t s = m.cone_s[e];
  r.dx = dw.x;
  r.dy = dw.y;
  r.dz = dw.z;
  r.ix = __frcp_rn(r.dx);
  r.iy = __frcp_rn(r.dy);
  r.iz = __frcp_rn(r.dz);
  r.sx = r.dx >= 0.0f;
  r.sy = r.dy >= 0.0f;
  r.sz = r.dz >= 0.0f;
  r.flip = (r.sx ? 0u : 1u) | (r.sy ? 0u : 2u) | (r.sz ? 0u : 4u);
  set_loc(r, P->loc[0], P->loc[1], P->loc[2]);
  r.ox = P->origin[0];
  r.oy = P->origin[1];
  r.oz = P->origin[2];
  r.fov = s ? m.spine[s - 1].fov : m.fov_c;
  r.id = P->id;
  r.depth = 1;
  r.steps = 0;
  if (SVO_TRACE_CELL_CACHE) r.cell = cell_index(1, r.wx, r.wy, r.wz, r.flip);
  reset_walk(w);
}

// SVO_MEGA_WARP_REFILL = T > 0: the cone kernel's warp batches refill their idle
// lanes from the list once at most T lanes hold a cone. Identical images;
// measured on GB300 (1080p megakernel frame, medians), T = 4, 8, 16: 15.51,
// 15.54, 15.40 ms against 14.91 ms.
#ifndef SVO_MEGA_WARP_REFILL
#define SVO_MEGA_WARP_REFILL 0
#endif

// accumulateRay's trace for every cone of the band's compacted list: warps
// claim 32 consecutive entries (kLane false) or lanes refill from the list
// every `cadence` steps (kLane true).
template <bool kSmemBases, bool kLane, bool kStats = false>
__global__ void __launch_bounds__(256, SVO_MEGA_MIN_CTAS) mega_cone_kernel(const MegaLaunch m) {
  extern __shared__ __align__(16) uint8_t smem[];
  // a block that starts after some cone stopped takes no work (the whole block
  // returns together, before the __syncthreads of the staging)
  __shared__ uint32_t s_stop;
  if (threadIdx.x == 0) s_stop = call_stopped(m) ? 1u : 0u;
  __syncthreads();
  if (s_stop) return;
  const TraceLaunch &a = m.t;
  ViewParams *s_views;
  uint16_t *s_bases;
  uint32_t *s_path;
  stage_shared<kSmemBases>(a, smem, s_views, s_bases, s_path, true);
  const int B = a.base_depth;
  const uint4 *blocks = reinterpret_cast<const uint4 *>(a.blocks);
  const ViewParams &v = s_views[0];
  Walk w;
  w.path = s_path + threadIdx.x;
  w.stride = blockDim.x;
  Ray r;
  r.view = 0;
  r.fresh = false;
  const uint32_t n = m.queue[1];
  if (!kLane && SVO_MEGA_WARP_REFILL > 0) {
    // warp batches whose idle lanes take the next list entries once at most
    // SVO_MEGA_WARP_REFILL lanes still hold a cone; all control decisions come
    // from warp votes, so all 32 lanes run every iteration
    const uint32_t lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
    const uint32_t limit = a.pass_limit ? a.pass_limit : (uint32_t)a.max_steps + 2u;
    const unsigned long long iter_limit =
        a.pass_limit ? (unsigned long long)a.pass_limit
                     : (unsigned long long)n * (unsigned long long)(a.max_steps + 2) + 64;
    unsigned long long iters = 0;
    bool have = false, timed_out = false, drained = false;
    uint32_t e = 0, steps = 0;
    Stats cs = {0, 0, 0, 0, 0, 0, 0};
    for (;;) {
      if (++iters > iter_limit) {
        record_timeout(a, e, r);
        break;
      }
      unsigned act = __ballot_sync(kFull, have);
      if (__popc(act) <= SVO_MEGA_WARP_REFILL && !drained) {
        if (__any_sync(kFull, timed_out)) break;
        const unsigned idle = ~act;
        const uint32_t k = (uint32_t)__popc(idle);
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(m.queue, k);
        first = __shfl_sync(kFull, first, 0);
        drained = (uint64_t)first + k >= (uint64_t)n;
        if (!have) {
          const uint32_t i = first + (uint32_t)__popc(idle & below);
          if (i < n) {
            e = m.entries[i];
            start_cone(m, e, r, w);
            have = true;
            steps = 0;
          }
        }
        act = __ballot_sync(kFull, have);
      }
      if (act == 0) {
        if (drained) break;
        continue;
      }
      if (have) {
        if (++steps > limit) {
          record_timeout(a, e, r);
          timed_out = true;
          have = false;
        } else {
          int finish = probe<kStats, kSmemBases, true>(a, v, s_bases, blocks, B, r, w, cs);
          if (finish == kStepEmpty) finish = advance(a, blocks, B, r, w);
          if (finish != kStepOn) {
            if (kStats) {
              cs.rays++;
              cs.block_reads += w.v_block;
              cs.base_steps += w.v_base;
              if (finish == kStepHit) cs.hits++;
            }
            m.cone_sky[e] = finish == kStepBackground ? 1 : 0;
            have = false;
          }
        }
      }
    }
    if (kStats) flush_stats(a, cs);
  } else if (!kLane) {
    const uint32_t lane = threadIdx.x & 31u;
    bool timed_out = false;
    Stats cs = {0, 0, 0, 0, 0, 0, 0};
    for (;;) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(m.queue, 32u);
      base = __shfl_sync(kFull, base, 0);
      if (base >= n) break;
      const uint32_t i = base + lane;
      if (i < n && !timed_out) {
        const uint32_t e = m.entries[i];
        start_cone(m, e, r, w);
        int finish;
        if (!run_cone<kSmemBases, kStats>(a, v, s_bases, blocks, B, r, w, finish, cs)) {
          record_timeout(a, e, r);
          timed_out = true;
        }
        m.cone_sky[e] = finish == kStepBackground ? 1 : 0;
      }
      if (__any_sync(kFull, timed_out)) break;
    }
    if (kStats) flush_stats(a, cs);
  } else {
    // every pass starts a cone or steps one, so a thread runs at most
    // n * (max_steps + 2) + 64 passes; past that it records its state and stops
    const unsigned long long iter_limit =
        a.pass_limit ? (unsigned long long)a.pass_limit
                     : (unsigned long long)n * (unsigned long long)(a.max_steps + 2) + 64;
    unsigned long long iters = 0;
    const int cadence = a.cadence;
    bool have = false;
    uint32_t e = 0;
    Stats st;
    for (;;) {
      if (++iters > iter_limit) {
        record_timeout(a, e, r);
        break;
      }
      if (!have) {
        cg::coalesced_group g = cg::coalesced_threads();
        const uint32_t my = claim(g, m.queue, 1);
        if (my >= n) break;
        e = m.entries[my];
        start_cone(m, e, r, w);
        have = true;
      }
      int finish = kStepOn;
      for (int k = 0; k < cadence && finish == kStepOn; k++) {
        finish = probe<false, kSmemBases, true>(a, v, s_bases, blocks, B, r, w, st);
        if (finish == kStepEmpty) finish = advance(a, blocks, B, r, w);
      }
      if (finish == kStepOn) continue;
      m.cone_sky[e] = finish == kStepBackground ? 1 : 0;
      have = false;
    }
  }
}

// writeToAccumulator over the pixel's cones in generation order, then draw.
__global__ void __launch_bounds__(256) mega_resolve_kernel(const MegaLaunch m) {
  if (call_stopped(m)) return;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t tile = gid >> 5, lane = gid & 31u;
  if (tile >= m.band_tiles) return;
  const MegaPixel P = m.pix[((size_t)m.band_tile0 + tile) * 32u + lane];
  if (P.kind == kMegaPad) return;
  const ViewParams &v = m.t.views[0];
  if (!v.rgba || P.id >= v.width * v.height) return;
  uint32_t cr, cg_, cb;
  if (P.kind == kMegaSurface) {
    const uint4 nd = load_node(reinterpret_cast<const uint4 *>(m.t.blocks), m.t.n_blocks, P.node);
    cr = (nd.z >> 16) & 0xffu;
    cg_ = nd.z >> 24;
    cb = nd.w & 0xffu;
  } else {
    float lum;
    sky_light(P.dir[0], P.dir[1], P.dir[2], cr, cg_, cb, lum);
  }
  float tw = 0.0f, ar = 0.0f, ag = 0.0f, ab = 0.0f;
  const uint32_t n_cones = P.kind == kMegaMiss ? 0u : min((uint32_t)P.n_cones, (uint32_t)m.k_max);
  for (uint32_t k = 0; k < n_cones; k++) {
    const size_t i = cone_slot(m, tile, k, lane);
    const float4 dw = m.cone_dw[i];
    tw = __fadd_rn(tw, dw.w);
    if (!m.cone_sky[i]) continue;  // a surface has Luminosity 0
    uint32_t r, g, b;
    float lum;
    sky_light(dw.x, dw.y, dw.z, r, g, b, lum);
    ar = __fadd_rn(ar, __fmul_rn(__fmul_rn(__fdiv_rn(__uint2float_rn(r), 255.0f), dw.w), lum));
    ag = __fadd_rn(ag, __fmul_rn(__fmul_rn(__fdiv_rn(__uint2float_rn(g), 255.0f), dw.w), lum));
    ab = __fadd_rn(ab, __fmul_rn(__fmul_rn(__fdiv_rn(__uint2float_rn(b), 255.0f), dw.w), lum));
  }
  float4 px;
  if (tw > 0.01f) {
    px.x = fminf(__fdiv_rn(__fadd_rn(__uint2float_rn(cr), __fdiv_rn(ar, tw)), 255.0f), 1.0f);
    px.y = fminf(__fdiv_rn(__fadd_rn(__uint2float_rn(cg_), __fdiv_rn(ag, tw)), 255.0f), 1.0f);
    px.z = fminf(__fdiv_rn(__fadd_rn(__uint2float_rn(cb), __fdiv_rn(ab, tw)), 255.0f), 1.0f);
  } else {
    px.x = __fdiv_rn(__uint2float_rn(cr), 255.0f);
    px.y = __fdiv_rn(__uint2float_rn(cg_), 255.0f);
    px.z = __fdiv_rn(__uint2float_rn(cb), 255.0f);
  }
  px.w = 1.0f;
  reinterpret_cast<float4 *>(v.rgba)[P.id] = px;
}

bool bases_in_smem(const TraceLaunch &a) { return (size_t)a.n_bases * 2 <= 96 * 1024; }

template <class K>
cudaError_t launch_traversal(K kernel, const MegaLaunch &m, int grid, cudaStream_t s) {
  const size_t smem = trace_smem_bytes(m.t, bases_in_smem(m.t));
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kernel<<<grid, m.t.block_size, smem, s>>>(m);
  return cudaGetLastError();
}

}  // namespace

int mega_occupancy(const MegaLaunch &m) {
  const bool sb = bases_in_smem(m.t);
  const size_t smem = trace_smem_bytes(m.t, sb);
  const void *k = sb ? (const void *)mega_cone_kernel<true, false> : (const void *)mega_cone_kernel<false, false>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, m.t.block_size, smem) != cudaSuccess) return 0;
  return n;
}

svo_status launch_mega_primary(const MegaLaunch &m, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // statistics (m.t.stats) are counted by the shared-memory-bases warp-batch variants
  cudaError_t e = !bases_in_smem(m.t) ? launch_traversal(mega_primary_kernel<false, false>, m, m.t.grid, s)
                  : m.t.stats         ? launch_traversal(mega_primary_kernel<true, true>, m, m.t.grid, s)
                                      : launch_traversal(mega_primary_kernel<true, false>, m, m.t.grid, s);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("megakernel primary launch: ") + cudaGetErrorString(e));
  return SVO_OK;
}

svo_status launch_mega_band(const MegaLaunch &m, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint32_t blocks = (m.band_tiles * 32u + 255u) / 256u;
  mega_fan_kernel<<<blocks, 256, 0, s>>>(m);
  mega_scan_kernel<<<1, 1024, 0, s>>>(m);
  mega_emit_kernel<<<blocks, 256, 0, s>>>(m);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    const bool sb = bases_in_smem(m.t), lane = m.cone_schedule == SVO_SCHEDULE_LANE;
    e = sb ? (lane ? launch_traversal(mega_cone_kernel<true, true>, m, m.grid_cones, s)
                   : (m.t.stats ? launch_traversal(mega_cone_kernel<true, false, true>, m, m.grid_cones, s)
                                : launch_traversal(mega_cone_kernel<true, false>, m, m.grid_cones, s)))
           : (lane ? launch_traversal(mega_cone_kernel<false, true>, m, m.grid_cones, s)
                   : launch_traversal(mega_cone_kernel<false, false>, m, m.grid_cones, s));
  }
  if (e == cudaSuccess) {
    mega_resolve_kernel<<<blocks, 256, 0, s>>>(m);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("megakernel band launch: ") + cudaGetErrorString(e));
  return SVO_OK;
}

}  // namespace svo
