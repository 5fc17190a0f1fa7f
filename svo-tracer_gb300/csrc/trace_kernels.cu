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
//    counter, and a persistent grid takes rays from it. Warp batches (the
//    default): a warp claims 32 consecutive slots, one pixel tile of a tiled
//    view, traces them to the end and claims again; the coherence of a tile
//    is worth more than keeping every lane busy. Lane refills: whenever a
//    thread finishes a ray it claims the next one, the threads of a warp that
//    need rays at the same moment sharing one atomicAdd (coalesced group,
//    `ray_chunk` rays per thread), and rays are retired and replaced every
//    `cadence` steps. No step depends on the warp staying converged. Ray
//    state stays in registers, so the reference's per-step reload of ~74 B of
//    SoA state disappears.
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

#include "trace_core.cuh"

namespace svo {
namespace {

#ifndef SVO_TRACE_MIN_CTAS
#define SVO_TRACE_MIN_CTAS 4  // 55 registers, no spills (5: 48 registers, no spill, 1.56 vs 1.45 ms on the 1080p frame at 53)
#endif
// SVO_TRACE_WARP_REFILL = T > 0: warp batches whose idle lanes take the next
// ray slots (tile order, one atomic per warp) once at most T lanes of the warp
// still hold a ray, instead of waiting for the whole batch. 0: plain batches.
// Identical results; measured on GB300 (1080p frame / 64 views, medians), T = 4,
// 8, 16: 1.72, 1.83, 1.93 ms and 9.48, 9.77, 10.28 ms against 1.52 and 8.50 ms. The
// refilled lanes start far from the stragglers they join, so the steps of the
// warp diverge more than the idle lanes cost.
#ifndef SVO_TRACE_WARP_REFILL
#define SVO_TRACE_WARP_REFILL 0
#endif
// Dynamic shared memory before the wavefront schedule's area: the view table,
// the base chunks (when staged) and the path cache, rounded to 16 bytes.
__host__ __device__ inline size_t trace_smem_bytes_base(const TraceLaunch &a, bool bases_in_smem) {
  size_t b = (size_t)a.n_views * sizeof(ViewParams);
  if (bases_in_smem) b += ((size_t)a.n_bases * 2 + 15) & ~(size_t)15;
  b += (size_t)a.path_levels * a.block_size * 4;
  return (b + 15) & ~(size_t)15;
}
// The wavefront schedule's per-thread slots: location (24 B), direction and
// inverse direction (24 B), depth/result/flip (4 B), two queue entries (4 B).
constexpr size_t kWavefrontSlotBytes = 56;

// kSched: 0 lane refills, 1 warp batches, 2 the CTA wavefront (moves compacted).
template <bool kStats, bool kSmemBases, int kSched>
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
    fill_spread_table();
  }
  __syncthreads();

  const int B = a.base_depth;
  const uint4 *blocks = reinterpret_cast<const uint4 *>(a.blocks);

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
  uint32_t ray_global = 0;
  // Every pass either starts a ray or advances it by at least one step, so a
  // thread runs at most total_rays * (max_steps + 2) + 64 passes; past that
  // bound it records its state and stops instead of spinning.
  // (a.pass_limit, when set, replaces that bound: a test of the timeout path)
  const unsigned long long iter_limit =
      a.pass_limit ? (unsigned long long)a.pass_limit
                   : (unsigned long long)a.total_rays * (unsigned long long)(a.max_steps + 2) + 64;
  unsigned long long iters = 0;
  auto record_timeout = [&]() {
    if (a.error && atomicCAS(a.error, 0u, (unsigned)SVO_ERR_TIMEOUT) == 0u) {
      a.error[1] = blockIdx.x;
      a.error[2] = threadIdx.x;
      a.error[3] = ray_global;
      a.error[4] = (uint32_t)r.depth;
      a.error[5] = (uint32_t)r.steps;
    }
  };
  // false for the padding slots of tiled views
  auto start_ray = [&](uint32_t my) -> bool {
    ray_global = my;
    if (!setup_ray(a, s_views, my, r)) return false;
    w.v_block = 0;
    w.v_base = 0;
    w.cur_addr = kFull;
    w.last_group = kFull;
    return true;
  };
  // evaluateBackground / resolveRemainders + drawTrace for a finished ray
  auto finish_ray = [&](const ViewParams &v, int finish) {
    uint32_t hit_index = SVO_MISS, cr, cg_, cb;
    uint8_t hit_depth = 0;
    float t = __int_as_float(0x7f800000);
    if (finish == kStepHit &&
        SVO_CHECK(a.error, r.depth - B - 2 >= 0 && r.depth - B - 2 < a.path_levels, 6, (uint32_t)(r.depth - B - 2))) {
      uint32_t addr = w.path[(r.depth - B - 2) * w.stride];
      uint4 nd = load_node(blocks, a.n_blocks, addr);
      hit_index = addr;
      hit_depth = (uint8_t)r.depth;
      cr = (nd.z >> 16) & 0xffu;
      cg_ = nd.z >> 24;
      cb = nd.w & 0xffu;
      float x = __fsub_rn(ulong_to_unit(loc_x(r)), r.ox);
      float y = __fsub_rn(ulong_to_unit(loc_y(r)), r.oy);
      float z = __fsub_rn(ulong_to_unit(loc_z(r)), r.oz);
      t = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
      if (kStats) {
        w.v_block += (uint32_t)(r.depth - B - 1);
        st.hits++;
      }
    } else {
      sky_colour(r, cr, cg_, cb);
    }
    const float fw = 65025.0f;  // (float)255 * 255.0f
    float4 px;
    px.x = fminf(__fdiv_rn(__uint2float_rn(cr * 255u), fw), 1.0f);
    px.y = fminf(__fdiv_rn(__uint2float_rn(cg_ * 255u), fw), 1.0f);
    px.z = fminf(__fdiv_rn(__uint2float_rn(cb * 255u), fw), 1.0f);
    px.w = 1.0f;
    if (!SVO_CHECK(a.error, r.id < v.width * v.height, 7, r.id)) return;
    if (v.hit_index) v.hit_index[r.id] = hit_index;
    if (v.hit_depth) v.hit_depth[r.id] = hit_depth;
    if (v.t) v.t[r.id] = t;
    if (v.rgba) reinterpret_cast<float4 *>(v.rgba)[r.id] = px;
    if (kStats) {
      st.rays++;
      st.base_steps += w.v_base;
      st.block_reads += w.v_block;
      const uint32_t pixel = v.pixel_begin + r.id;  // per-ray counters by pixel of the batch
      if (a.ray_v_block) a.ray_v_block[pixel] = w.v_block;
      if (a.ray_v_base) a.ray_v_base[pixel] = w.v_base;
    }
  };

  if (kSched == 1 && SVO_TRACE_WARP_REFILL > 0) {
    // ---- warp batches with refills: every control decision below is taken
    // from warp votes, so all 32 lanes run every iteration of the loop
    const uint32_t lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
    const uint32_t ray_limit = a.pass_limit ? a.pass_limit : (uint32_t)a.max_steps + 2u;
    bool have = false, timed_out = false, drained = false;
    uint32_t ray_iters = 0;
    for (;;) {
      if (++iters > iter_limit) {  // the same count in every lane
        record_timeout();
        break;
      }
      unsigned act = __ballot_sync(kFull, have);
      if (__popc(act) <= SVO_TRACE_WARP_REFILL && !drained) {
        if (__any_sync(kFull, timed_out)) break;
        const unsigned idle = ~act;
        const uint32_t n = (uint32_t)__popc(idle);
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(a.ray_counter, n);
        first = __shfl_sync(kFull, first, 0);
        drained = (uint64_t)first + n >= (uint64_t)a.total_rays;
        if (!have) {
          const uint32_t my = first + (uint32_t)__popc(idle & below);
          if (my < a.total_rays && start_ray(my)) {
            have = true;
            ray_iters = 0;
          }
        }
        act = __ballot_sync(kFull, have);
      }
      if (act == 0) {
        if (drained) break;
        continue;
      }
      if (have) {
        if (++ray_iters > ray_limit) {
          record_timeout();
          timed_out = true;
          have = false;
        } else {
          const ViewParams &v = s_views[r.view];
          const int f = probe<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
          const int finish = f == kStepEmpty ? advance(a, blocks, B, r, w) : f;
          if (finish != kStepOn) {
            finish_ray(v, finish);
            have = false;
          }
        }
      }
    }
  } else if (kSched == 1) {
    // ---- warp batches: 32 consecutive ray slots (one pixel tile of a tiled
    // view) per warp, regrouped between batches
    const uint32_t lane = threadIdx.x & 31u;
    bool timed_out = false;
    for (;;) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(a.ray_counter, 32u);
      base = __shfl_sync(kFull, base, 0);
      if (base >= a.total_rays) break;
      const uint32_t my = base + lane;
      if (my < a.total_rays && !timed_out && start_ray(my)) {
        const ViewParams &v = s_views[r.view];
        int finish = kStepOn;
        // a probe ends a ray once it has taken max_steps steps, so a ray whose
        // step count reaches max_steps + 2 is a fault: record it and stop the warp
        const uint32_t ray_limit = a.pass_limit ? a.pass_limit : (uint32_t)a.max_steps + 2u;
        while (finish == kStepOn) {
          // every pass takes a step (counted in r.steps) or ends the ray
          if ((uint32_t)r.steps >= ray_limit) {
            record_timeout();
            timed_out = true;
            break;
          }
          int f = probe<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
          if (SVO_TRACE_PROBE_RUNS) {
            // steps that keep the location (descents, LOD ascents) run back to
            // back, so the move below runs with every lane whose octant is empty
            while (f == kStepOn && (uint32_t)r.steps < ray_limit) f = probe<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
            if (f == kStepOn) {
              record_timeout();
              timed_out = true;
              break;
            }
          }
          finish = f == kStepEmpty ? advance(a, blocks, B, r, w) : f;
        }
        if (!timed_out) finish_ray(v, finish);
      }
      // every lane of the warp arrives here on every iteration
      if (__any_sync(kFull, timed_out)) break;
    }
  } else if (kSched == 2) {
    // ---- the CTA wavefront: every pass, each thread probes its own ray; the
    // rays whose octant is empty are compacted into a shared-memory queue
    // (warp-aggregated appends, the reference's `increment` per work-group) and
    // moved by the CTA's first threads, full warps of moves, through the
    // movers' state in shared memory; the owners then read the moved state
    // back. A thread without a ray claims the next one each pass. Two CTA
    // barriers per pass, reached by every thread; the loop ends by a CTA vote.
    // Measured on GB300 against warp batches (1080p frame / 64 views): 3.25 vs
    // 1.52 ms and 21.2 vs 8.6 ms; the barriers of every step cost more than the
    // compacted moves save (running a ray's descents within its pass: 3.83 ms).
    const uint32_t T = blockDim.x, slot = threadIdx.x;
    uint8_t *wf = smem + trace_smem_bytes_base(a, kSmemBases);
    uint64_t *s_w = reinterpret_cast<uint64_t *>(wf);             // [3][T] travel-space location
    float *s_f = reinterpret_cast<float *>(s_w + 3 * T);          // [6][T] direction, inverse direction
    uint32_t *s_st = reinterpret_cast<uint32_t *>(s_f + 6 * T);   // [T] depth | result << 8 | flip << 16
    uint16_t *s_q = reinterpret_cast<uint16_t *>(s_st + T);       // [2][T] move queues (alternate passes)
    __shared__ uint32_t s_nmove[2];
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
      s_nmove[0] = s_nmove[1] = 0;
      s_stop = 0;
    }
    __syncthreads();
    bool have = false, drained = false;
    int parity = 0;
    for (;;) {
      int f = kStepOn;
      if (++iters > iter_limit) {
        record_timeout();
        s_stop = 1;
      } else {
        if (!have && !drained) {
          cg::coalesced_group g = cg::coalesced_threads();
          const uint32_t my = claim(g, a.ray_counter, 1);
          if (my >= a.total_rays) {
            drained = true;
          } else if (start_ray(my)) {  // padding slots of tiled views claim again next pass
            have = true;
            s_f[0 * T + slot] = r.dx;
            s_f[1 * T + slot] = r.dy;
            s_f[2 * T + slot] = r.dz;
            s_f[3 * T + slot] = r.ix;
            s_f[4 * T + slot] = r.iy;
            s_f[5 * T + slot] = r.iz;
          }
        }
        if (have) {
          const ViewParams &v = s_views[r.view];
          f = probe<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
          if (f == kStepEmpty) {
            s_w[0 * T + slot] = r.wx;
            s_w[1 * T + slot] = r.wy;
            s_w[2 * T + slot] = r.wz;
            s_st[slot] = (uint32_t)r.depth | (r.flip << 16);
            cg::coalesced_group g = cg::coalesced_threads();
            s_q[parity * T + claim(g, &s_nmove[parity], 1)] = (uint16_t)slot;
          } else if (f != kStepOn) {
            finish_ray(v, f);
            have = false;
          }
        }
      }
      __syncthreads();
      // the moves (traverseChunk, comparePositions, path rebuild), one per thread
      const uint32_t n_move = s_nmove[parity];
      if (threadIdx.x < n_move) {
        const uint32_t o = s_q[parity * T + threadIdx.x];
        Ray m;
        m.wx = s_w[0 * T + o];
        m.wy = s_w[1 * T + o];
        m.wz = s_w[2 * T + o];
        m.dx = s_f[0 * T + o];
        m.dy = s_f[1 * T + o];
        m.dz = s_f[2 * T + o];
        m.ix = s_f[3 * T + o];
        m.iy = s_f[4 * T + o];
        m.iz = s_f[5 * T + o];
        const uint32_t sw = s_st[o];
        m.depth = (int)(sw & 0xffu);
        m.flip = sw >> 16;
        m.sx = (m.flip & 1u) == 0;
        m.sy = (m.flip & 2u) == 0;
        m.sz = (m.flip & 4u) == 0;
        Walk wm;
        wm.path = s_path + o;
        wm.stride = (int)T;
        const int res = advance(a, blocks, B, m, wm);
        s_w[0 * T + o] = m.wx;
        s_w[1 * T + o] = m.wy;
        s_w[2 * T + o] = m.wz;
        s_st[o] = (uint32_t)m.depth | ((uint32_t)res << 8);
      }
      if (threadIdx.x == 0) s_nmove[parity ^ 1] = 0;  // the next pass appends after the barrier below
      const int busy = __syncthreads_or(have || !drained);
      if (!busy || s_stop) break;
      if (have && f == kStepEmpty) {  // the moved state back to its owner
        r.wx = s_w[0 * T + slot];
        r.wy = s_w[1 * T + slot];
        r.wz = s_w[2 * T + slot];
        const uint32_t sw = s_st[slot];
        r.depth = (int)(sw & 0xffu);
        r.cone = -1.0f;
        if (SVO_TRACE_CELL_CACHE && r.depth >= 1 && r.depth <= B) r.cell = cell_index(r.depth, r.wx, r.wy, r.wz, r.flip);
        if ((int)(sw >> 8) == kStepBackground) {
          finish_ray(s_views[r.view], kStepBackground);
          have = false;
        }
      }
      parity ^= 1;
    }
  } else {
    // ---- lanes: each thread claims rays on its own ------------------------------
    const uint32_t chunk = a.ray_chunk;
    const int cadence = a.cadence;
    bool have = false;
    uint32_t next_ray = 0, left_in_chunk = 0, chunk_stride = 0;
    for (;;) {
      if (++iters > iter_limit) {
        record_timeout();
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
        if (!start_ray(my)) continue;   // padding slot of a tiled view
        have = true;
      }

      // ---- up to `cadence` traversal steps; retire finished rays together -----
      const ViewParams &v = s_views[r.view];
      int finish = kStepOn;
      for (int k = 0; k < cadence && finish == kStepOn; k++)
        finish = step<kStats, kSmemBases>(a, v, s_bases, blocks, B, r, w, st);
      if (finish == kStepOn) continue;
      finish_ray(v, finish);
      have = false;
    }
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

// ---- the child-request queue of the pixel-order rule ---------------------------
// A chunk of kRequestChunk pixel flags is one CTA of 256 threads, 16 flags (one
// 16-byte load) per thread; flags are 0 or 1 bytes, so a word's population
// count is the number of its flagged pixels.
constexpr int kReqThreads = 256;
static_assert(kRequestChunk == kReqThreads * 16, "one 16-byte load of flags per thread");

__device__ __forceinline__ uint32_t flag_count(uint4 f) { return __popc(f.x) + __popc(f.y) + __popc(f.z) + __popc(f.w); }

// Exclusive prefix of `x` over the CTA (256 threads) and the CTA's total.
__device__ __forceinline__ uint32_t cta_exclusive(uint32_t x, uint32_t &total) {
  __shared__ uint32_t s_warp[kReqThreads / 32];
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  uint32_t inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, inc, o);
    if (lane >= (uint32_t)o) inc += y;
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  uint32_t before = 0;
  total = 0;
#pragma unroll
  for (int k = 0; k < kReqThreads / 32; k++) {
    const uint32_t c = s_warp[k];
    if ((uint32_t)k < wid) before += c;
    total += c;
  }
  return before + inc - x;
}

__global__ void __launch_bounds__(kReqThreads) k_req_count(const uint8_t *flags, uint32_t *chunk_counts) {
  const uint4 f = reinterpret_cast<const uint4 *>(flags)[(size_t)blockIdx.x * kReqThreads + threadIdx.x];
  uint32_t total;
  cta_exclusive(flag_count(f), total);
  if (threadIdx.x == 0) chunk_counts[blockIdx.x] = total;
}

// One CTA of 1024 threads: chunk counts -> exclusive chunk offsets (in place);
// *raised = the total.
__global__ void __launch_bounds__(1024) k_req_scan(uint32_t *chunk, uint32_t n, uint32_t *raised) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (n + 1023u) / 1024u, b = threadIdx.x * per, e = min(n, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; i++) s += chunk[i];
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
    const uint32_t c = chunk[i];
    chunk[i] = run;
    run += c;
  }
  if (threadIdx.x == 1023) *raised = part[1023];
}

// Each flagged pixel's staged record goes to queue slot (its rank in pixel
// order) while that rank is below the cap.
__global__ void __launch_bounds__(kReqThreads) k_req_scatter(const uint8_t *flags, const uint32_t *chunk_offsets,
                                                             const StagedRequest *stage, svo_child_request *queue,
                                                             uint32_t cap) {
  const uint32_t first = chunk_offsets[blockIdx.x];
  if (first >= cap) return;  // the whole CTA: its ranks all lie past the cap
  const size_t word = (size_t)blockIdx.x * kReqThreads + threadIdx.x;
  const uint4 f = reinterpret_cast<const uint4 *>(flags)[word];
  uint32_t total;
  uint32_t rank = first + cta_exclusive(flag_count(f), total);
  const uint32_t w4[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
  for (int k = 0; k < 16; k++) {
    if ((w4[k >> 2] >> (8 * (k & 3))) & 0xffu) {
      if (rank < cap) {
        const StagedRequest sr = stage[word * 16 + k];
        svo_child_request q;
        q.address = sr.address;
        q.tick = 0;  // TraceData.Tick is never set by the wavefront's resolveTrace
        q.depth = sr.depth;
        q._pad0 = 0;
        q.location[0] = sr.location[0];
        q.location[1] = sr.location[1];
        q.location[2] = sr.location[2];
        q.tree_size = sr.tree_size;
        for (int j = 0; j < 7; j++) q._pad1[j] = 0;
        queue[rank] = q;
      }
      rank++;
    }
  }
}

}  // namespace

svo_status launch_request_compaction(const TraceLaunch &a, uint32_t total_pixels, uint32_t *chunk_offsets,
                                     void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint32_t chunks = (total_pixels + kRequestChunk - 1) / kRequestChunk;
  if (!chunks) return SVO_OK;
  k_req_count<<<chunks, kReqThreads, 0, s>>>(a.req_flag, chunk_offsets);
  k_req_scan<<<1, 1024, 0, s>>>(chunk_offsets, chunks, a.request_count);
  if (a.requests && a.request_cap)
    k_req_scatter<<<chunks, kReqThreads, 0, s>>>(a.req_flag, chunk_offsets, a.req_stage, a.requests, a.request_cap);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("request compaction launch: ") + cudaGetErrorString(e));
  return SVO_OK;
}

size_t trace_smem_bytes(const TraceLaunch &a, bool bases_in_smem) {
  size_t b = trace_smem_bytes_base(a, bases_in_smem);
  if (a.schedule == SVO_SCHEDULE_WAVEFRONT) b += kWavefrontSlotBytes * (size_t)a.block_size;
  return b;
}

static bool bases_fit(const TraceLaunch &a) { return (size_t)a.n_bases * 2 <= 96 * 1024; }

template <bool S, bool M, int W>
static cudaError_t launch_one(const TraceLaunch &a, size_t smem, cudaStream_t stream) {
  auto k = trace_kernel<S, M, W>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (!a.l2_bytes) {
    k<<<a.grid, a.block_size, smem, stream>>>(a);
    return cudaGetLastError();
  }
  // the launch's node reads in [l2_base, l2_base + l2_bytes) persist in L2
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
  attr[0].val.accessPolicyWindow.base_ptr = const_cast<void *>(a.l2_base);
  attr[0].val.accessPolicyWindow.num_bytes = a.l2_bytes;
  attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
  attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
  attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)a.grid);
  cfg.blockDim = dim3((unsigned)a.block_size);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, a);
}

template <int W>
static const void *kernel_for(bool stats, bool m) {
  return stats ? (m ? (const void *)trace_kernel<true, true, W> : (const void *)trace_kernel<true, false, W>)
               : (m ? (const void *)trace_kernel<false, true, W> : (const void *)trace_kernel<false, false, W>);
}

int trace_occupancy(const TraceLaunch &a, bool with_stats) {
  bool m = bases_fit(a);
  size_t smem = trace_smem_bytes(a, m);
  int n = 0;
  const void *k = a.schedule == SVO_SCHEDULE_WARP        ? kernel_for<1>(with_stats, m)
                  : a.schedule == SVO_SCHEDULE_WAVEFRONT ? kernel_for<2>(with_stats, m)
                                                         : kernel_for<0>(with_stats, m);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, a.block_size, smem) != cudaSuccess) return 0;
  return n;
}

template <int W>
static cudaError_t launch_sched(const TraceLaunch &a, bool with_stats, bool m, size_t smem, cudaStream_t s) {
  if (with_stats) return m ? launch_one<true, true, W>(a, smem, s) : launch_one<true, false, W>(a, smem, s);
  return m ? launch_one<false, true, W>(a, smem, s) : launch_one<false, false, W>(a, smem, s);
}

svo_status launch_trace(const TraceLaunch &a, bool with_stats, void *stream) {
  bool m = bases_fit(a);
  size_t smem = trace_smem_bytes(a, m);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = a.schedule == SVO_SCHEDULE_WARP        ? launch_sched<1>(a, with_stats, m, smem, s)
                  : a.schedule == SVO_SCHEDULE_WAVEFRONT ? launch_sched<2>(a, with_stats, m, smem, s)
                                                         : launch_sched<0>(a, with_stats, m, smem, s);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("trace kernel launch: ") + cudaGetErrorString(e));
  return SVO_OK;
}

}  // namespace svo
