// Differentiable colour fitting over a fixed-geometry octree (no reference
// counterpart; an added pattern beside the drop-in trace).
//
// Forward model: a primary ray is traversed exactly as the trace kernel does
// (same ray setup, same steps, same cone LOD stop). At every LOD hit the hit
// node's parameters p = (r, g, b, a) are composited front to back,
//   C += T * a * rgb,   T *= (1 - a),
// and the ray continues as if that octant held no geometry, until it leaves
// the cube (C += T * sky colour), reaches `max_hits` hits or the step limit.
// No transmittance cut-off is applied, so the hit sequence depends on the
// geometry only and the loss is a smooth function of the parameters.
//
// Loss: L = sum over pixels and channels of (C - target)^2 / pixels.
//
// Backward: the traversal is recomputed rather than storing per-ray hit lists.
// A walk over the hits replays the prefix sums S_i of the contributions up to
// and including hit i, so the colour contributed behind hit i is
// R_i = C - S_i and
//   dL/drgb_i = T_i a_i dL/dC,
//   dL/da_i   = dL/dC . (T_i rgb_i - R_i / (1 - a_i)).
// C is the forward's saved colour or, without it, a first walk that recomputes
// it with the forward's own code.
//
// Precision without FP64 arithmetic (slow on this part): every contribution
// T_i a_i rgb_i and every T_{i+1} = T_i (1 - a_i) is one rounded FP32 product,
// computed identically by the forward and both backward walks, and the sums C
// and S_i are compensated (Knuth's TwoSum: a float pair hi + lo carries the
// exact rounding error of each addition). S_i then equals the forward's running
// sum after i hits bit for bit, and C - S_i keeps ~1e-7 relative precision
// however small the colour behind hit i is. The loss is summed in FP64.
//
// Gradient accumulation: warp-aggregated atomics. The lanes of a warp that
// hit the same node in the same step find each other with match.any; the
// lowest of them sums the group's gradients through shared memory and issues
// one 16-byte atomic add (a lane alone adds directly).
//
// Scheduling: a persistent grid whose warps claim 32 consecutive ray slots at
// a time from a device counter (one 8x4 pixel tile: the views are staged
// tiled, outputs stay indexed by pixel); lane i takes slot base + i, and the warp regroups
// with a warp vote (a regrouping point) between the walks of a ray and before the next claim, so
// lanes do not drift apart over rays and phases (measured 2-3x faster than a
// free per-thread grid-stride loop).
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"
// The base cell kept in a register across descents (the trace kernel's default)
// costs these kernels registers: measured on GB300 (16 x 512^2 sphere views),
// forward 1.93 -> 1.92 ms, saved-colour backward 2.22 -> 2.12 ms, recomputing
// backward 6.99 -> 6.19 ms without it (the backward's spill 280 -> 160 bytes).
#ifndef SVO_TRACE_CELL_CACHE
#define SVO_TRACE_CELL_CACHE 0
#endif
#include "trace_core.cuh"

// Resident CTAs of 256 threads per SM the kernels are compiled for (4 and 4
// measured fastest on the 16-view 512x512 sphere workload; the backward then
// spills a few registers to L1).
#ifndef SVO_DIFF_BWD_MIN_CTAS
#define SVO_DIFF_BWD_MIN_CTAS 4
#endif
#ifndef SVO_DIFF_FWD_MIN_CTAS
#define SVO_DIFF_FWD_MIN_CTAS 4
#endif

namespace svo {
namespace {

struct DiffLaunch {
  TraceLaunch t;           // traversal state (usage and requests disabled)
  const float4 *params;    // per node
  float4 *grads;           // per node (backward)
  float *rgb;              // forward output: 3 floats per ray, or null
  float *saved;            // forward colour (hi, lo) pairs: written by the forward, read by a saved backward
  const float *target;     // backward: 3 floats per ray
  double *loss;            // backward: accumulated loss
  double inv_pixels;       // 1 / total rays
  int32_t max_hits;
  int32_t use_saved;       // backward: read C from `saved` instead of recomputing it
};

// Knuth's TwoSum (round-to-nearest, no contraction): hi + b = s + e exactly;
// s replaces hi and the error e is added to lo.
__device__ __forceinline__ void acc2(float &hi, float &lo, float b) {
  float s = __fadd_rn(hi, b);
  float bb = __fsub_rn(s, hi);
  float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  hi = s;
  lo = __fadd_rn(lo, e);
}

// Front-to-back compositing state of one ray.
struct Composite {
  float hi[3], lo[3], T;
  __device__ __forceinline__ void init() {
    for (int k = 0; k < 3; k++) hi[k] = lo[k] = 0.0f;
    T = 1.0f;
  }
  __device__ __forceinline__ void hit(float4 p) {
    float ta = __fmul_rn(T, p.w);
    acc2(hi[0], lo[0], __fmul_rn(ta, p.x));
    acc2(hi[1], lo[1], __fmul_rn(ta, p.y));
    acc2(hi[2], lo[2], __fmul_rn(ta, p.z));
    T = __fmul_rn(T, __fsub_rn(1.0f, p.w));
  }
  __device__ __forceinline__ void sky(float3 c) {
    acc2(hi[0], lo[0], __fmul_rn(T, c.x));
    acc2(hi[1], lo[1], __fmul_rn(T, c.y));
    acc2(hi[2], lo[2], __fmul_rn(T, c.z));
  }
};

__device__ __forceinline__ float3 sky_rgb(const Ray &r) {
  uint32_t cr, cg_, cb;
  sky_colour(r, cr, cg_, cb);
  const float fw = 65025.0f;
  return make_float3(__fdiv_rn(__uint2float_rn(cr * 255u), fw), __fdiv_rn(__uint2float_rn(cg_ * 255u), fw),
                     __fdiv_rn(__uint2float_rn(cb * 255u), fw));
}

// Visits the hits of one ray in order: visit(node, is_background) with
// is_background = true once for the sky contribution (node unused). Each pass
// of the loop probes (and counts, in r.steps) a step, and a probe past
// max_steps ends the ray in the sky, so a walk takes at most max_steps + 1
// passes. A walk that has taken its bound of steps (max_steps + 2, or the
// launch's pass_limit) without finishing records the timeout in the error
// record and returns false.
// kStats: the walk's reference-walk counters (V_block, V_base, hits) are
// added to st, as the trace kernel's statistics count them.
// kSmemBases: the base chunks are read from shared memory (staged by the
// kernel) rather than from global memory.
template <bool kStats, bool kSmemBases, class Visit>
__device__ __forceinline__ bool walk_hits(const DiffLaunch &d, const ViewParams *s_views, const uint16_t *s_bases,
                                          uint32_t ray, Walk &w, Stats &st, Visit &&visit) {
  const TraceLaunch &a = d.t;
  const int B = a.base_depth;
  const uint4 *blocks = reinterpret_cast<const uint4 *>(a.blocks);
  Ray r;
  setup_ray(a, s_views, ray, r);
  w.cur_addr = 0xffffffffu;
  w.last_group = 0xffffffffu;
  w.v_block = 0;
  w.v_base = 0;
  auto counted = [&](bool ok) {
    if (kStats) {
      st.rays++;
      st.block_reads += w.v_block;
      st.base_steps += w.v_base;
    }
    return ok;
  };
  const ViewParams &v = s_views[r.view];
  int hits = 0;
  // every pass probes one step (r.steps counts them) or ends the walk
  const uint32_t limit = a.pass_limit ? a.pass_limit : (uint32_t)a.max_steps + 2u;
  for (;;) {
    if ((uint32_t)r.steps >= limit) {
      if (a.error && atomicCAS(a.error, 0u, (unsigned)SVO_ERR_TIMEOUT) == 0u) {
        a.error[1] = blockIdx.x;
        a.error[2] = threadIdx.x;
        a.error[3] = ray;
        a.error[4] = (uint32_t)r.depth;
        a.error[5] = (uint32_t)r.steps;
      }
      return counted(false);
    }
    int f = step<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
    if (f == kStepOn) continue;
    if (f == kStepBackground) {
      visit(0u, true, r);
      return counted(true);
    }
    if (!SVO_CHECK(a.error, r.depth - B - 2 >= 0 && r.depth - B - 2 < a.path_levels, 9, (uint32_t)(r.depth - B - 2)))
      return counted(false);
    visit(w.path[(r.depth - B - 2) * w.stride], false, r);
    if (kStats) st.hits++;
    if (++hits >= d.max_hits) return counted(true);
    if (step_past(a, blocks, B, r, w) == kStepBackground) {
      visit(0u, true, r);
      return counted(true);
    }
  }
}

template <bool kBackward, bool kStats, bool kSmemBases>
__global__ void __launch_bounds__(256, kBackward ? SVO_DIFF_BWD_MIN_CTAS : SVO_DIFF_FWD_MIN_CTAS) diff_kernel(const DiffLaunch d) {
  extern __shared__ __align__(16) uint8_t smem[];
  const TraceLaunch &a = d.t;
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
    fill_spread_table();
  }
  __syncthreads();
  __shared__ float4 s_agg[256];  // gradient slots of the warp aggregation, one per thread
  Walk w;
  w.path = s_path + threadIdx.x;
  w.stride = blockDim.x;
  double loss_part = 0.0;
  Stats st = {0, 0, 0, 0, 0, 0, 0};
  // Warp-uniform loop over rays (lane i of a warp takes ray base + i) with a
  // warp vote (__any_sync, which also regroups the lanes) after each phase,
  // which every lane of the warp reaches on every iteration: the lanes regroup
  // before each walk instead of drifting apart over rays and phases, and the
  // whole warp leaves the loop when one of its walks ran past its pass bound.
  const uint32_t lane = threadIdx.x & 31u;
  for (;;) {
    // the warp claims the next 32 rays (persistent grid, dynamic balance)
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(a.ray_counter, 32u);
    base = __shfl_sync(kFull, base, 0);
    if (base >= a.total_rays) break;
    const uint32_t ray = base + lane;
    int view = 0;
    uint32_t px = 0, py = 0;
    const bool live = ray < a.total_rays && ray_slot(a, s_views, ray, view, px, py);  // not a padding slot
    const uint32_t pixel = live ? s_views[view].pixel_begin + py * s_views[view].width + px : 0;
    Composite full;
    full.init();
    bool stopped = false;  // a walk ran past its pass bound: the warp leaves the loop
    if (live && (!kBackward || !d.use_saved)) {
      stopped = !walk_hits<kStats, kSmemBases>(d, s_views, s_bases, ray, w, st, [&](uint32_t node, bool bg, const Ray &r) {
        if (bg)
          full.sky(sky_rgb(r));
        else
          full.hit(__ldg(d.params + node));
      });
    }
    if (__any_sync(kFull, stopped)) break;
    if (!kBackward) {
      if (live && d.rgb)
        for (int k = 0; k < 3; k++) d.rgb[3ull * pixel + k] = __fadd_rn(full.hi[k], full.lo[k]);
      if (live && d.saved)
        for (int k = 0; k < 3; k++) {
          d.saved[6ull * pixel + 2 * k] = full.hi[k];
          d.saved[6ull * pixel + 2 * k + 1] = full.lo[k];
        }
      continue;
    }
    float G[3] = {0.0f, 0.0f, 0.0f};
    if (live) {
      if (d.use_saved)
        for (int k = 0; k < 3; k++) {
          full.hi[k] = __ldg(d.saved + 6ull * pixel + 2 * k);
          full.lo[k] = __ldg(d.saved + 6ull * pixel + 2 * k + 1);
        }
      const float *tg = d.target + 3ull * pixel;
      for (int k = 0; k < 3; k++) {
        double e = ((double)full.hi[k] - (double)__ldg(tg + k)) + (double)full.lo[k];
        loss_part += e * e * d.inv_pixels;
        G[k] = (float)(2.0 * e * d.inv_pixels);  // dL/dC
      }
      // the gradient walk: replay the prefix sums, one contribution at a time
      Composite pre;
      pre.init();
      stopped = !walk_hits<false, kSmemBases>(d, s_views, s_bases, ray, w, st, [&](uint32_t node, bool bg, const Ray &) {
        if (bg) return;
        float4 p = __ldg(d.params + node);
        float T = pre.T, ta = __fmul_rn(T, p.w);
        pre.hit(p);
        // 1 / (1 - a); a = 1 ends the transmittance and nothing lies behind the hit
        float om = __fsub_rn(1.0f, p.w);
        float inv_om = om > 0.0f ? __frcp_rn(om) : 0.0f;
        const float pc[3] = {p.x, p.y, p.z};
        float4 g;
        float *gv = &g.x;
        float dot = 0.0f;
        for (int k = 0; k < 3; k++) {
          float behind = __fadd_rn(__fsub_rn(full.hi[k], pre.hi[k]), __fsub_rn(full.lo[k], pre.lo[k]));
          dot = __fadd_rn(dot, __fmul_rn(G[k], __fsub_rn(__fmul_rn(T, pc[k]), __fmul_rn(behind, inv_om))));
          gv[k] = __fmul_rn(ta, G[k]);
        }
        g.w = dot;
        {
          // lanes of the warp that hit the same node now add through one
          // 16-byte atomic: the lowest such lane sums the others' slots
          const unsigned active = __activemask();
          const unsigned peers = __match_any_sync(active, node);
          const unsigned grouped = __ballot_sync(active, peers != (1u << lane));
          if (peers == (1u << lane)) {
            atomicAdd(d.grads + node, g);
          } else {
            s_agg[threadIdx.x] = g;
            __syncwarp(grouped);
            if (lane == (unsigned)(__ffs(peers) - 1)) {
              float4 sum = g;
              for (unsigned m = peers & (peers - 1); m; m &= m - 1) {
                float4 o = s_agg[(threadIdx.x & ~31u) + (__ffs(m) - 1)];
                sum.x = __fadd_rn(sum.x, o.x);
                sum.y = __fadd_rn(sum.y, o.y);
                sum.z = __fadd_rn(sum.z, o.z);
                sum.w = __fadd_rn(sum.w, o.w);
              }
              atomicAdd(d.grads + node, sum);
            }
            __syncwarp(grouped);
          }
        }
      });
    }
    if (__any_sync(kFull, stopped)) break;
  }
  if (kBackward) {
    cooperative_groups::coalesced_group g = cooperative_groups::coalesced_threads();
    double v = cooperative_groups::reduce(g, loss_part, cooperative_groups::plus<double>());
    if (g.thread_rank() == 0) atomicAdd(d.loss, v);
  }
  if (kStats && a.stats) {
    unsigned long long vals[7] = {st.rays, st.hits, st.base_steps, st.block_reads, st.block_steps, 0, st.limited};
    cooperative_groups::coalesced_group g = cooperative_groups::coalesced_threads();
#pragma unroll
    for (int k = 0; k < 7; k++) {
      unsigned long long x = cooperative_groups::reduce(g, vals[k], cooperative_groups::plus<unsigned long long>());
      if (g.thread_rank() == 0 && x) atomicAdd(a.stats + k, x);
    }
  }
}

template <bool kBackward>
svo_status run_diff(Context &c, const svo_trace_input *views, int32_t n, const float *target_dev, float *rgb_dev,
                    bool use_saved, double *loss_host) {
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_diff: no octree uploaded");
  if (!c.has_params) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_diff: no parameters set");
  if (n <= 0 || n > 512 || !views) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_diff: bad view list");
  std::vector<svo_trace_output> outs(n);
  std::memset(outs.data(), 0, sizeof(svo_trace_output) * n);
  for (auto &o : outs) o.on_device = 1;
  SVO_CUDA(cudaEventSynchronize(c.staged), "svo_diff: staging");
  uint32_t total = 0, pixels = 0;
  size_t table_floats = 0;
  svo_status st = stage_views(c, views, n, outs.data(), true, kDiffTileW, total, pixels, table_floats);
  if (st) return st;
  if (kBackward && use_saved &&
      !(c.saved_valid && c.saved_params_gen == c.params_gen && c.saved_max_hits == c.cfg.max_hits &&
        c.saved_views.size() == (size_t)n && std::memcmp(c.saved_views.data(), views, sizeof(svo_trace_input) * n) == 0))
    return fail(SVO_ERR_INVALID_ARGUMENT,
                "svo_diff_backward: no saved forward colour for these views, parameters and max_hits");
  if (c.views.reserve(n) || c.tables.reserve(table_floats) || c.diff_loss.reserve(1) ||
      (!kBackward && c.diff_saved.reserve(6ull * pixels)))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_diff: allocation failed");
  DiffLaunch d{};
  st = prepare_launch(c, n, total, d.t, false);
  if (st) return st;
  d.t.usage = nullptr;
  d.t.requests = nullptr;
  d.t.request_cap = 0;
  d.params = reinterpret_cast<const float4 *>(c.params.p);
  d.grads = reinterpret_cast<float4 *>(c.grads.p);
  d.rgb = rgb_dev;
  d.target = target_dev;
  d.saved = c.diff_saved.p;
  d.use_saved = use_saved ? 1 : 0;
  d.loss = c.diff_loss.p;
  d.inv_pixels = 1.0 / (double)pixels;
  d.max_hits = c.cfg.max_hits;
  d.t.block_size = 256;
  // base chunks of up to 96 KB (base depth 5 and less) are staged in shared
  // memory, larger ones read from global memory, as the trace kernels do
  const bool smem_bases = c.n_bases * 2 <= 96 * 1024;
  size_t smem = (size_t)n * sizeof(ViewParams) + (smem_bases ? ((c.n_bases * 2 + 15) & ~(size_t)15) : 0) +
                (size_t)d.t.path_levels * 256 * 4;
  // collect_stats: the forward counts its walk (V_block, V_base, hits) into the
  // context's trace statistics (svo_last_trace_stats)
  const bool stats = !kBackward && c.cfg.collect_stats > 0;
  d.t.stats = stats ? c.stats.p : nullptr;
  auto kernel = smem_bases ? diff_kernel<kBackward, false, true> : diff_kernel<kBackward, false, false>;
  if constexpr (!kBackward)
    if (stats) kernel = smem_bases ? diff_kernel<false, true, true> : diff_kernel<false, true, false>;
  SVO_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "svo_diff: smem");
  int occ = 0;
  SVO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, smem), "svo_diff: occupancy");
  if (occ <= 0) return fail(SVO_ERR_NO_DEVICE, "svo_diff: kernel cannot be resident");
  int grid = (int)std::min<long>((long)occ * c.sm_count, ((long)total + 255) / 256);
  SVO_CUDA(cudaMemcpyAsync(c.views.p, c.h_views.p, sizeof(ViewParams) * n, cudaMemcpyHostToDevice, c.stream),
           "svo_diff: views");
  SVO_CUDA(cudaMemcpyAsync(c.tables.p, c.h_tables.p, sizeof(float) * table_floats, cudaMemcpyHostToDevice, c.stream),
           "svo_diff: tables");
  SVO_CUDA(cudaEventRecord(c.staged, c.stream), "svo_diff: staging event");
  SVO_CUDA(cudaMemsetAsync(c.counters.p, 0, kErrorOffset * sizeof(uint32_t), c.stream), "svo_diff: counters");
  if (stats) SVO_CUDA(cudaMemsetAsync(c.stats.p, 0, 8 * sizeof(unsigned long long), c.stream), "svo_diff: stats");
  if (kBackward) {
    SVO_CUDA(cudaMemsetAsync(c.grads.p, 0, c.grads.n * sizeof(float), c.stream), "svo_diff: grads");
    SVO_CUDA(cudaMemsetAsync(c.diff_loss.p, 0, sizeof(double), c.stream), "svo_diff: loss");
  }
  kernel<<<std::max(1, grid), 256, smem, c.stream>>>(d);
  SVO_CUDA(cudaGetLastError(), "svo_diff: launch");
  if (kBackward && loss_host) {
    SVO_CUDA(cudaMemcpyAsync(loss_host, c.diff_loss.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream),
             "svo_diff: loss");
    svo_status es = report_kernel_error(c, "svo_diff_backward");  // synchronises
    if (es) return es;
  }
  if (!kBackward) {
    c.last_stats_valid = stats;
    c.saved_views.assign(views, views + n);
    c.saved_params_gen = c.params_gen;
    c.saved_max_hits = c.cfg.max_hits;
    c.saved_valid = true;
  }
  c.last_rays = pixels;
  return SVO_OK;
}

uint64_t view_rays(const svo_trace_input *views, int32_t n) {
  uint64_t t = 0;
  for (int i = 0; i < n; i++) t += (uint64_t)views[i].screen_size[0] * views[i].screen_size[1];
  return t;
}

}  // namespace
}  // namespace svo

using svo::Context;
using svo::fail;

#define DCTX(ptr, fn)                                                                        \
  if (!(ptr)) return fail(SVO_ERR_INVALID_ARGUMENT, std::string(fn) + ": null context"); \
  Context &c = *static_cast<Context *>(ptr);                                               \
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, std::string(fn) + ": no octree uploaded");  \
  SVO_CUDA(cudaSetDevice(c.device), "cudaSetDevice")

extern "C" {

SVO_API svo_status svo_diff_set_params(void *ctx, const float *rgba, size_t n_nodes, int32_t on_device) {
  DCTX(ctx, "svo_diff_set_params");
  if (!rgba || n_nodes > c.budget) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_diff_set_params: bad parameter array");
  if (c.params.reserve(4 * c.budget) || c.grads.reserve(4 * c.budget))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_diff_set_params: allocation failed");
  SVO_CUDA(cudaMemsetAsync(c.params.p, 0, 4 * c.budget * sizeof(float), c.stream), "svo_diff_set_params");
  SVO_CUDA(cudaMemcpyAsync(c.params.p, rgba, 4 * n_nodes * sizeof(float),
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c.stream),
           "svo_diff_set_params");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_diff_set_params: synchronize");
  c.has_params = true;
  c.params_gen++;
  return SVO_OK;
}

SVO_API svo_status svo_diff_get_grads(void *ctx, float *grad, size_t n_nodes, int32_t on_device) {
  DCTX(ctx, "svo_diff_get_grads");
  if (!c.has_params || !grad || n_nodes > c.budget)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_diff_get_grads: bad gradient array");
  SVO_CUDA(cudaMemcpyAsync(grad, c.grads.p, 4 * n_nodes * sizeof(float),
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c.stream),
           "svo_diff_get_grads");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_diff_get_grads: synchronize");
  return SVO_OK;
}

SVO_API svo_status svo_diff_forward(void *ctx, const svo_trace_input *views, int32_t n, float *rgb, int32_t on_device) {
  DCTX(ctx, "svo_diff_forward");
  if (!rgb) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_diff_forward: null output");
  uint64_t rays = svo::view_rays(views, n);
  float *dst = rgb;
  // a pinned host output is written by the kernel itself; other host memory
  // through a device buffer and a copy
  float *pinned = on_device ? nullptr : static_cast<float *>(svo::pinned_device_ptr(rgb));
  if (pinned) {
    dst = pinned;
  } else if (!on_device) {
    if (c.diff_rgb.reserve(3 * rays)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_diff_forward: allocation failed");
    dst = c.diff_rgb.p;
  }
  svo_status st = svo::run_diff<false>(c, views, n, nullptr, dst, false, nullptr);
  if (st) return st;
  if (!on_device && !pinned)
    SVO_CUDA(cudaMemcpyAsync(rgb, dst, 3 * rays * sizeof(float), cudaMemcpyDeviceToHost, c.stream),
             "svo_diff_forward: read");
  if (!on_device) return svo::report_kernel_error(c, "svo_diff_forward");  // synchronises
  return SVO_OK;
}

SVO_API svo_status svo_diff_backward(void *ctx, const svo_trace_input *views, int32_t n, const float *target,
                                     int32_t use_saved, int32_t on_device, double *loss) {
  DCTX(ctx, "svo_diff_backward");
  if (!target || !views || n <= 0) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_diff_backward: null target or views");
  uint64_t rays = svo::view_rays(views, n);
  const float *src = target;
  // a pinned host target is read by the kernel itself; other host memory is copied
  const float *pinned = on_device ? nullptr : static_cast<const float *>(svo::pinned_device_ptr(target));
  if (pinned) {
    src = pinned;
  } else if (!on_device) {
    if (c.diff_target.reserve(3 * rays)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_diff_backward: allocation failed");
    SVO_CUDA(cudaMemcpyAsync(c.diff_target.p, target, 3 * rays * sizeof(float), cudaMemcpyHostToDevice, c.stream),
             "svo_diff_backward: target");
    src = c.diff_target.p;
  }
  svo_status st = svo::run_diff<true>(c, views, n, src, nullptr, use_saved != 0, loss);
  if (st) return st;
  // the caller may reuse a host target once the call returns
  if (pinned && !loss) return svo::report_kernel_error(c, "svo_diff_backward");  // synchronises
  return SVO_OK;
}

}  // extern "C"
