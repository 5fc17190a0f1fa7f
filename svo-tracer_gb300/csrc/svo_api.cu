// C ABI of libsvo: context, octree residency and the trace entry points.
//
// This layer replaces the reference's OpenCL host wrapper
// (SvoTracer.Kernel/ComputeManager.cs, ComputeManagerFactory.cs) and the frame
// driver MainWindow.RunWavefront (SvoTracer.Window/MainWindow.cs:356-622):
// buffers are owned by a context, the kernels read the same OpenCL struct
// layouts, and every failure comes back as a status code with a message (the
// reference throws "{method}: {code}", ComputeManager.cs:283-287).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "context.h"

namespace svo {

static thread_local std::string g_last_error;

svo_status fail(svo_status status, const std::string &message) {
  g_last_error = message;
  return status;
}

static svo_trace_config default_config() {
  svo_trace_config c{};
  // 192 threads: with the trace kernel's 55 registers, 6 CTAs (36 warps) fit an
  // SM against 4 of 256 threads (32 warps). Measured on GB300, 256 / 128 / 192 /
  // 224 threads: 1080p frame 1.373 / 1.350 / 1.340 / 1.351 ms, megakernel frame
  // 13.85 / 13.44 / 13.41 / 13.52 ms, the frame with the secondary-cone stage
  // 1.526 / 1.505 / 1.500 / 1.515 ms, identical outputs.
  c.block_size = 192;
  c.ctas_per_sm = 0;  // occupancy-derived
  c.ray_chunk = 1;
  c.cadence = 16;
  c.max_steps = 1 << 16;
  c.collect_stats = 0;
  c.max_hits = 16;
  c.schedule = SVO_SCHEDULE_WARP;  // 13% faster than lane refills on the 1080p terrain frame
  c.l2_window = -1;
  c.pass_limit = 0;
  c.request_order = SVO_REQUESTS_ARRIVAL;
  c.gi_stage = -1;
  return c;
}

static uint32_t pow_sum(int depth) {
  uint32_t s = 0, p = 1;
  for (int i = 1; i <= depth; i++) {
    p *= 8;
    s += p;
  }
  return s;
}

// Deepest node level reachable from the dense level B+2 through child links
// (host scan, bounded by SVO_MAX_TREE_DEPTH + 1).
static int scan_tree_depth(const svo_block *blocks, size_t n_blocks, int B) {
  size_t dense = (size_t)1 << (3 * (B + 2));
  int threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<int> best(threads, B + 2);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) {
    pool.emplace_back([&, t]() {
      std::vector<std::pair<uint32_t, int>> stack;
      for (size_t a = t; a < std::min(dense, n_blocks); a += threads) {
        stack.clear();
        stack.push_back({(uint32_t)a, B + 2});
        while (!stack.empty()) {
          auto [addr, d] = stack.back();
          stack.pop_back();
          if (d > best[t]) best[t] = d;
          if (d >= SVO_MAX_TREE_DEPTH + 1) continue;
          uint32_t c = blocks[addr].child;
          // every child group, as the reachability of the tree updates walks
          // them (a tree may hang groups below octants without geometry)
          if (c == SVO_NO_CHILD || (size_t)c + 8 > n_blocks) continue;
          for (uint32_t k = 0; k < 8; k++) stack.push_back({c + k, d + 1});
        }
      }
    });
  }
  for (auto &th : pool) th.join();
  return *std::max_element(best.begin(), best.end());
}

// Builds the view table and trig tables for `n` views in pinned staging.
svo_status stage_views(Context &c, const svo_trace_input *in, int32_t n, const svo_trace_output *out,
                       bool outputs_on_device, uint32_t tile_w, uint32_t &total_rays, uint32_t &total_pixels,
                       size_t &table_floats, uint32_t *hit_fallback) {
  const uint32_t tile_h = tile_w ? 32 / tile_w : 0;
  total_rays = 0;
  total_pixels = 0;
  table_floats = 0;
  for (int i = 0; i < n; i++) {
    uint64_t w = in[i].screen_size[0], h = in[i].screen_size[1];
    if (w == 0 || h == 0 || w > 65536 || h > 65536)
      return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace: screen_size must be 1..65536 per axis");
    if (in[i].base_depth != 0 && in[i].base_depth != c.base_depth)
      return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace: input base_depth differs from the resident tree's");
    uint64_t slots = tile_w ? ((w + tile_w - 1) / tile_w) * ((h + tile_h - 1) / tile_h) * 32 : w * h;
    if ((uint64_t)total_rays + slots > 0xF0000000ull)
      return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace: too many rays in one call");
    total_rays += (uint32_t)slots;
    total_pixels += (uint32_t)(w * h);
    table_floats += 2 * (w + h);
  }
  if (c.h_views.reserve(n) != cudaSuccess || c.h_tables.reserve(table_floats) != cudaSuccess)
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: pinned staging allocation failed");
  uint32_t ray = 0;
  size_t toff = 0;
  size_t out_off = 0;
  for (int i = 0; i < n; i++) {
    const svo_trace_input &t = in[i];
    ViewParams &v = c.h_views.p[i];
    std::memset(&v, 0, sizeof(v));
    for (int k = 0; k < 3; k++) v.origin[k] = t.origin[k];
    for (int k = 0; k < 9; k++) v.facing[k] = t.facing[k];
    uint32_t W = t.screen_size[0], H = t.screen_size[1];
    v.fov_px = t.fov[0] / (float)W;  // native_divide(FoV[0], ScreenSize.x)
    v.dof[0] = t.dof[0];
    v.dof[1] = t.dof[1];
    v.width = W;
    v.height = H;
    v.ray_begin = ray;
    v.pixel_begin = (uint32_t)out_off;
    v.tile = (uint16_t)tile_w;
    v.table_off = (uint32_t)toff;
    v.tick = t.tick;
    if (outputs_on_device) {
      v.hit_index = out[i].hit_index;
      v.hit_depth = out[i].hit_depth;
      v.t = out[i].t;
      v.rgba = out[i].rgba;
    } else {
      v.hit_index = out[i].hit_index ? c.o_index.p + out_off : nullptr;
      v.hit_depth = out[i].hit_depth ? c.o_depth.p + out_off : nullptr;
      v.t = out[i].t ? c.o_t.p + out_off : nullptr;
      v.rgba = out[i].rgba ? c.o_rgba.p + 4 * out_off : nullptr;
    }
    if (!v.hit_index && hit_fallback) v.hit_index = hit_fallback + out_off;
    // Ray-setup angles (wavefront.cl:566-572); sin/cos are (float)sin((double)a).
    // Views of the same field of view and size share their tables.
    float *tb = c.h_tables.p + toff;
    uint32_t f0, f1;
    std::memcpy(&f0, &t.fov[0], 4);
    std::memcpy(&f1, &t.fov[1], 4);
    const std::array<uint32_t, 4> key{f0, f1, W, H};
    auto it = c.table_cache.find(key);
    if (it == c.table_cache.end()) {
      if (c.table_cache.size() >= 256) c.table_cache.clear();
      std::vector<float> tab(2 * ((size_t)W + H));
      float fw = (float)W, fh = (float)H;
      for (uint32_t x = 0; x < W; x++) {
        float u = t.fov[0] * ((fw / 2.0f - (float)x) / fw);
        tab[x] = (float)std::sin((double)u);
        tab[W + x] = (float)std::cos((double)u);
      }
      for (uint32_t y = 0; y < H; y++) {
        float vv = t.fov[1] * ((fh / 2.0f - (float)y) / fh);
        tab[2 * W + y] = (float)std::sin((double)vv);
        tab[2 * W + H + y] = (float)std::cos((double)vv);
      }
      it = c.table_cache.emplace(key, std::move(tab)).first;
    }
    std::memcpy(tb, it->second.data(), it->second.size() * sizeof(float));
    toff += 2 * ((size_t)W + H);
    out_off += (size_t)W * H;
    ray += tile_w ? ((W + tile_w - 1) / tile_w) * ((H + tile_h - 1) / tile_h) * 32 : W * H;
  }
  return SVO_OK;
}

// The L2 persisting window of a trace launch: the dense level-(B+2) nodes at the
// head of the node array, which every ray entering a block reads first. The
// context's persisting set-aside is raised to the window's size the first time
// (within the device's limits) and given back when the window is switched off
// or the context is destroyed.
static void plan_l2_window(Context &c, TraceLaunch &a) {
  if (c.cfg.l2_window <= 0 || !c.blocks.p || !c.n_blocks) return;
  int max_persist = 0, max_window = 0;
  if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, c.device) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, c.device) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  const size_t dense = std::min(c.n_blocks, (size_t)1 << (3 * (c.base_depth + 2))) * sizeof(svo_block);
  const size_t bytes = std::min(dense, (size_t)std::min(max_persist, max_window));
  if (!bytes) return;
  if (!c.l2_limit_set) {
    size_t prev = 0;
    if (cudaDeviceGetLimit(&prev, cudaLimitPersistingL2CacheSize) != cudaSuccess ||
        (prev < bytes && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, bytes) != cudaSuccess)) {
      cudaGetLastError();
      return;
    }
    c.l2_limit_prev = prev;
    c.l2_limit_set = true;
  }
  a.l2_base = c.blocks.p;
  a.l2_bytes = bytes;
}

svo_status prepare_launch(Context &c, int32_t n_views, uint32_t total_rays, TraceLaunch &a, bool stats) {
  a = TraceLaunch{};
  a.bases = c.bases.p;
  a.blocks = c.blocks.p;
  a.usage = c.usage.p;
  a.requests = c.requests.p;
  a.request_cap = c.request_cap;
  a.ray_counter = c.counters.p;
  a.error = c.counters.p + kErrorOffset;
  a.request_count = c.counters.p + 1;
  a.stats = stats ? c.stats.p : nullptr;
  a.ray_v_block = (stats && c.cfg.collect_stats >= 2) ? c.ray_v_block.p : nullptr;
  a.ray_v_base = (stats && c.cfg.collect_stats >= 2) ? c.ray_v_base.p : nullptr;
  a.views = c.views.p;
  a.tables = c.tables.p;
  a.n_bases = (uint32_t)c.n_bases;
  a.n_blocks = (uint32_t)c.budget;
  a.n_groups = (uint32_t)c.n_groups;
  a.total_rays = total_rays;
  a.n_views = n_views;
  a.base_depth = c.base_depth;
  a.max_steps = c.cfg.max_steps;
  a.ray_chunk = (uint32_t)std::max(1, c.cfg.ray_chunk);
  a.cadence = std::max(1, c.cfg.cadence);
  a.block_size = c.cfg.block_size;
  a.schedule = c.cfg.schedule;
  a.path_levels = std::max(1, c.tree_depth - (int)c.base_depth - 1);
  a.pass_limit = (uint32_t)c.cfg.pass_limit;
  plan_l2_window(c, a);
  int occ = c.cfg.ctas_per_sm > 0 ? c.cfg.ctas_per_sm : trace_occupancy(a, stats);
  if (occ <= 0) return fail(SVO_ERR_NO_DEVICE, "svo_trace: the trace kernel cannot be resident (no sm_103a image?)");
  long want = (long)occ * c.sm_count;
  long need = ((long)total_rays + 31) / 32 * 32 / a.block_size + 1;
  a.grid = (int)std::max(1L, std::min(want, need));
  return SVO_OK;
}

// The view table lives in shared memory (120 B per view).
constexpr int kMaxViews = 512;

svo_status report_kernel_error(Context &c, const char *fn) {
  // through pinned memory: one asynchronous copy behind the stream's work, one wait
  uint32_t *e = c.h_counters.p;
  SVO_CUDA(cudaMemcpyAsync(e, c.counters.p + kErrorOffset, kErrorWords * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           c.stream),
           std::string(fn) + ": error record");
  SVO_CUDA(cudaStreamSynchronize(c.stream), std::string(fn) + ": synchronize");
  if (!e[0]) return SVO_OK;
  // reported once: the next launches start with a clear record
  SVO_CUDA(cudaMemsetAsync(c.counters.p + kErrorOffset, 0, kErrorWords * sizeof(uint32_t), c.stream),
           std::string(fn) + ": error record");
  SVO_CUDA(cudaStreamSynchronize(c.stream), std::string(fn) + ": synchronize");
  if (e[0] == SVO_ERR_TIMEOUT)
    return fail(SVO_ERR_TIMEOUT, std::string(fn) + ": thread " + std::to_string(e[2]) + " of block " +
                                     std::to_string(e[1]) + " exceeded its pass bound on ray " + std::to_string(e[3]) +
                                     " (depth " + std::to_string(e[4]) + ", steps " + std::to_string(e[5]) + ")");
  if (e[0] == SVO_ERR_INTERNAL)
    return fail(SVO_ERR_INTERNAL, std::string(fn) + ": index check " + std::to_string(e[3]) + " failed (index " +
                                      std::to_string(e[4]) + ") in thread " + std::to_string(e[2]) + " of block " +
                                      std::to_string(e[1]));
  return fail((svo_status)e[0], std::string(fn) + ": kernel reported error " + std::to_string(e[0]));
}

static svo_status check_kernel_error(Context &c) { return report_kernel_error(c, "svo_trace"); }

static svo_status run_trace(Context &c, const svo_trace_input *in, int32_t n, const svo_trace_output *out,
                            bool use_graph) {
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_trace: no octree uploaded");
  if (n <= 0 || !in || !out) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace: bad view list");
  if (n > kMaxViews) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_batch: at most 512 views per call");
  SVO_CUDA(cudaSetDevice(c.device), "cudaSetDevice");
  const bool host_outputs = out[0].on_device == 0;
  for (int i = 1; i < n; i++)
    if ((out[i].on_device == 0) != host_outputs)
      return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace: outputs of one call must all be host or all device");
  size_t pixels = 0;
  uint32_t cap = 0;
  for (int i = 0; i < n; i++) {
    pixels += (size_t)in[i].screen_size[0] * in[i].screen_size[1];
    cap = std::max(cap, in[i].max_child_request_id);
  }
  // Host outputs in pinned memory are written by the kernel itself (the GPU
  // addresses pinned memory directly), so their transfer overlaps the trace.
  // The outputs in kStagedHostOutputs are the exception: a warp's stores of
  // them are too small to cross to host memory efficiently (one byte of hit
  // depth per pixel), so they go to a device buffer and one copy per view
  // after the trace. Any other host output goes through device buffers and
  // copies afterwards.
  std::vector<svo_trace_output> mapped;
  const svo_trace_output *caller_out = out;
  bool staged_copies = false;
  if (host_outputs) {
    bool all_pinned = true;
    mapped.assign(out, out + n);
    for (int i = 0; i < n && all_pinned; i++) {
      void **ptrs[4] = {reinterpret_cast<void **>(&mapped[i].hit_index), reinterpret_cast<void **>(&mapped[i].hit_depth),
                        reinterpret_cast<void **>(&mapped[i].t), reinterpret_cast<void **>(&mapped[i].rgba)};
      for (int k = 0; k < 4 && all_pinned; k++) {
        void **pp = ptrs[k];
        if (!*pp) continue;
        if (kStagedHostOutputs & (1u << k)) {
          staged_copies = true;  // checked below; the pointer is replaced once the buffers exist
          if (!pinned_device_ptr(*pp)) all_pinned = false;
          continue;
        }
        void *d = pinned_device_ptr(*pp);
        if (!d) {
          all_pinned = false;
          break;
        }
        *pp = d;
      }
      mapped[i].on_device = 1;
    }
    if (all_pinned) {
      if (staged_copies) {
        if (((kStagedHostOutputs & 1u) && c.o_index.reserve(pixels)) || ((kStagedHostOutputs & 2u) && c.o_depth.reserve(pixels)) ||
            ((kStagedHostOutputs & 4u) && c.o_t.reserve(pixels)) || ((kStagedHostOutputs & 8u) && c.o_rgba.reserve(4 * pixels)))
          return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: output buffer allocation failed");
        size_t off = 0;
        for (int i = 0; i < n; i++) {
          if ((kStagedHostOutputs & 1u) && mapped[i].hit_index) mapped[i].hit_index = c.o_index.p + off;
          if ((kStagedHostOutputs & 2u) && mapped[i].hit_depth) mapped[i].hit_depth = c.o_depth.p + off;
          if ((kStagedHostOutputs & 4u) && mapped[i].t) mapped[i].t = c.o_t.p + off;
          if ((kStagedHostOutputs & 8u) && mapped[i].rgba) mapped[i].rgba = c.o_rgba.p + 4 * off;
          off += (size_t)in[i].screen_size[0] * in[i].screen_size[1];
        }
      }
      out = mapped.data();
    } else {
      staged_copies = false;
    }
  }
  const bool on_device = out[0].on_device != 0;  // device buffers, or pinned host memory the kernel writes
  if (!on_device) {
    if (c.o_index.reserve(pixels) || c.o_depth.reserve(pixels) || c.o_t.reserve(pixels) ||
        c.o_rgba.reserve(4 * pixels))
      return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: output buffer allocation failed");
  }
  if (c.requests.reserve(cap) != cudaSuccess) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: request queue allocation");
  c.request_cap = cap;
  // the wavefront's secondary-cone stage: one cone schedule for the call, and
  // every view's hit indices (in a library buffer where the caller wants none)
  const bool gi = c.cfg.gi_stage == 1;
  bool gi_valid = false;
  if (gi) {
    for (int i = 1; i < n; i++)
      if (in[i].fov_multiplier != in[0].fov_multiplier || in[i].fov_constant != in[0].fov_constant ||
          in[i].weighting_multiplier != in[0].weighting_multiplier ||
          in[i].weighting_constant != in[0].weighting_constant ||
          in[i].ambient_light_level != in[0].ambient_light_level)
        return fail(SVO_ERR_INVALID_ARGUMENT,
                    "svo_trace: with gi_stage the views of a call must share their cone parameters and AmbientLightLevel");
    // evaluateMaterial returns at once for these (wavefront.cl:1575-1576)
    gi_valid = !(in[0].fov_constant <= 0 || in[0].fov_multiplier >= 1 || in[0].fov_multiplier <= -1);
    svo_status sst = SVO_OK;
    if (gi_valid && ensure_cone_schedule(c, in[0], sst) <= 0)
      return sst ? sst
                 : fail(SVO_ERR_INVALID_ARGUMENT,
                        "svo_trace: the cone schedule exceeds SVO_MEGA_MAX_CONES cones per pixel (its loops would not end)");
    sst = ensure_normal_table(c);
    if (sst) return sst;
    if (c.gi_hit.reserve(pixels)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: hit index buffer allocation failed");
  }
  uint32_t total_rays, total_pixels;
  size_t table_floats;
  // the previous call's uploads must have read the pinned staging before it is rewritten
  SVO_CUDA(cudaEventSynchronize(c.staged), "svo_trace: staging");
  // warp batches take pixel tiles: wider ones when the kernel writes host memory
  const uint32_t tile_w =
      c.cfg.schedule == SVO_SCHEDULE_LANE ? 0 : (host_outputs && on_device ? kTraceHostTileW : kTraceTileW);
  svo_status st = stage_views(c, in, n, out, on_device, tile_w, total_rays, total_pixels, table_floats,
                              gi ? c.gi_hit.p : nullptr);
  if (st) return st;
  bool stats = c.cfg.collect_stats > 0;
  if (c.views.reserve(n) || c.tables.reserve(table_floats))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: view table allocation failed");
  if (stats && c.cfg.collect_stats >= 2 && (c.ray_v_block.reserve(total_pixels) || c.ray_v_base.reserve(total_pixels)))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: per-ray counter allocation failed");
  TraceLaunch a;
  st = prepare_launch(c, n, total_rays, a, stats);
  if (st) return st;
  GiLaunch g{};
  if (gi) {
    g.views = c.views.p;
    g.tables = c.tables.p;
    g.blocks = reinterpret_cast<const uint4 *>(c.blocks.p);
    g.usage = c.usage.p;
    g.normal_sc = c.mega_normal_sc.p;
    g.spine = c.mega_spine.p;
    g.ring = c.mega_ring.p;
    g.n_blocks = (uint32_t)c.budget;
    g.n_groups = (uint32_t)c.n_groups;
    g.total_pixels = total_pixels;
    g.n_views = n;
    g.n_spines = gi_valid ? c.mega_n_spines : 0;
    g.fov_c = in[0].fov_constant;
    g.weighting_c = in[0].weighting_constant;
    g.ambient = in[0].ambient_light_level;
    g.valid = gi_valid ? 1 : 0;
  }
  // pixel-order child requests: staged per pixel, the queue built after the trace
  const bool pixel_order = c.cfg.request_order == SVO_REQUESTS_PIXEL;
  const size_t flag_bytes = ((size_t)total_pixels + kRequestChunk - 1) / kRequestChunk * kRequestChunk;
  if (pixel_order) {
    if (c.req_stage.reserve(total_pixels) || c.req_flag.reserve(flag_bytes) ||
        c.req_chunks.reserve(flag_bytes / kRequestChunk))
      return fail(SVO_ERR_OUT_OF_MEMORY, "svo_trace: pixel-order request staging allocation failed");
    a.req_stage = c.req_stage.p;
    a.req_flag = c.req_flag.p;
  }

  auto enqueue = [&](bool capturing) -> svo_status {
    SVO_CUDA(cudaMemcpyAsync(c.views.p, c.h_views.p, sizeof(ViewParams) * n, cudaMemcpyHostToDevice, c.stream),
             "svo_trace: view upload");
    SVO_CUDA(cudaMemcpyAsync(c.tables.p, c.h_tables.p, sizeof(float) * table_floats, cudaMemcpyHostToDevice, c.stream),
             "svo_trace: table upload");
    SVO_CUDA(cudaEventRecordWithFlags(c.staged, c.stream, capturing ? cudaEventRecordExternal : cudaEventRecordDefault),
             "svo_trace: staging event");
    SVO_CUDA(cudaMemsetAsync(c.counters.p, 0, kErrorOffset * sizeof(uint32_t), c.stream), "svo_trace: counter reset");
    if (stats) SVO_CUDA(cudaMemsetAsync(c.stats.p, 0, 8 * sizeof(unsigned long long), c.stream), "svo_trace: stats reset");
    if (pixel_order) SVO_CUDA(cudaMemsetAsync(a.req_flag, 0, flag_bytes, c.stream), "svo_trace: request flags");
    svo_status lst = launch_trace(a, stats, c.stream);
    if (!lst && pixel_order) lst = launch_request_compaction(a, total_pixels, c.req_chunks.p, c.stream);
    if (!lst && gi) lst = launch_gi(g, c.stream);
    return lst;
  };

  if (use_graph && !stats) {
    std::vector<uint32_t> key;
    key.push_back((uint32_t)n);
    key.push_back(on_device ? 1u : 0u);
    key.push_back(tile_w);  // the launch's ray count depends on it
    for (int i = 0; i < n; i++) {
      key.push_back(in[i].screen_size[0]);
      key.push_back(in[i].screen_size[1]);
    }
    key.push_back((uint32_t)(uintptr_t)c.h_views.p);
    key.push_back((uint32_t)(uintptr_t)c.h_tables.p);
    key.push_back((uint32_t)(uintptr_t)c.views.p);
    key.push_back((uint32_t)(uintptr_t)c.tables.p);
    key.push_back((uint32_t)a.grid);
    key.push_back(pixel_order ? 1u : 0u);
    key.push_back((uint32_t)(uintptr_t)c.req_stage.p);
    key.push_back((uint32_t)(uintptr_t)c.requests.p);
    key.push_back(c.request_cap);
    key.push_back(gi ? 1u + (uint32_t)g.valid : 0u);
    if (gi) {
      uint32_t bits[3];
      std::memcpy(&bits[0], &g.fov_c, 4);
      std::memcpy(&bits[1], &g.weighting_c, 4);
      bits[2] = g.ambient;
      key.insert(key.end(), bits, bits + 3);
      key.push_back((uint32_t)g.n_spines);
      key.push_back((uint32_t)(uintptr_t)g.spine);
      key.push_back((uint32_t)(uintptr_t)g.ring);
      key.push_back((uint32_t)(uintptr_t)g.normal_sc);
      key.push_back((uint32_t)(uintptr_t)c.gi_hit.p);
    }
    if (!c.graph_exec || key != c.graph_key) {
      if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
      c.graph_exec = nullptr;
      cudaStream_t cap_stream = c.stream;
      SVO_CUDA(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal), "svo_trace_batch_graph: capture");
      svo_status est = enqueue(true);
      cudaGraph_t g = nullptr;
      cudaError_t ce = cudaStreamEndCapture(cap_stream, &g);
      if (est) {
        if (g) cudaGraphDestroy(g);
        return est;
      }
      if (ce != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("svo_trace_batch_graph: end capture: ") + cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&c.graph_exec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        c.graph_exec = nullptr;
        return fail(SVO_ERR_CUDA, std::string("svo_trace_batch_graph: instantiate: ") + cudaGetErrorString(ce));
      }
      c.graph_key = key;
    }
    SVO_CUDA(cudaGraphLaunch(c.graph_exec, c.stream), "svo_trace_batch_graph: launch");
  } else {
    st = enqueue(false);
    if (st) return st;
  }
  c.last_rays = total_pixels;
  c.last_stats_valid = stats;

  if (!on_device) {
    size_t off = 0;
    for (int i = 0; i < n; i++) {
      size_t np = (size_t)in[i].screen_size[0] * in[i].screen_size[1];
      if (out[i].hit_index)
        SVO_CUDA(cudaMemcpyAsync(out[i].hit_index, c.o_index.p + off, np * 4, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read hit_index");
      if (out[i].hit_depth)
        SVO_CUDA(cudaMemcpyAsync(out[i].hit_depth, c.o_depth.p + off, np, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read hit_depth");
      if (out[i].t)
        SVO_CUDA(cudaMemcpyAsync(out[i].t, c.o_t.p + off, np * 4, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read t");
      if (out[i].rgba)
        SVO_CUDA(cudaMemcpyAsync(out[i].rgba, c.o_rgba.p + 4 * off, np * 16, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read rgba");
      off += np;
    }
    return check_kernel_error(c);  // synchronises after the copies
  }
  if (staged_copies) {
    // the staged outputs of pinned host buffers: from the device buffers to the
    // caller's host memory
    size_t off = 0;
    for (int i = 0; i < n; i++) {
      const size_t np = (size_t)in[i].screen_size[0] * in[i].screen_size[1];
      const svo_trace_output &h = caller_out[i];
      if ((kStagedHostOutputs & 1u) && h.hit_index)
        SVO_CUDA(cudaMemcpyAsync(h.hit_index, c.o_index.p + off, np * 4, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read hit_index");
      if ((kStagedHostOutputs & 2u) && h.hit_depth)
        SVO_CUDA(cudaMemcpyAsync(h.hit_depth, c.o_depth.p + off, np, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read hit_depth");
      if ((kStagedHostOutputs & 4u) && h.t)
        SVO_CUDA(cudaMemcpyAsync(h.t, c.o_t.p + off, np * 4, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read t");
      if ((kStagedHostOutputs & 8u) && h.rgba)
        SVO_CUDA(cudaMemcpyAsync(h.rgba, c.o_rgba.p + 4 * off, np * 16, cudaMemcpyDeviceToHost, c.stream), "svo_trace: read rgba");
      off += np;
    }
  }
  if (host_outputs) return check_kernel_error(c);  // the kernel wrote pinned host memory: wait for it
  return SVO_OK;
}

}  // namespace svo

using svo::Context;
using svo::fail;

#define CTX_OR_FAIL(ptr, fn)                                                        \
  if (!(ptr)) return fail(SVO_ERR_INVALID_ARGUMENT, std::string(fn) + ": null context"); \
  Context &c = *static_cast<Context *>(ptr)

#define GUARD_BEGIN try {
#define GUARD_END(fn)                                                                  \
  }                                                                                    \
  catch (const std::bad_alloc &) {                                                     \
    return fail(SVO_ERR_OUT_OF_MEMORY, std::string(fn) + ": out of host memory");      \
  }                                                                                    \
  catch (const std::exception &e) {                                                    \
    return fail(SVO_ERR_INTERNAL, std::string(fn) + ": " + e.what());                  \
  }

extern "C" {

SVO_API const char *svo_last_error_string(void) { return svo::g_last_error.c_str(); }

SVO_API const char *svo_version(void) { return "svo-gb300 0.1 (sm_103a)"; }

SVO_API svo_status svo_create(int32_t device, void **ctx) {
  if (!ctx) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_create: null output");
  *ctx = nullptr;
  GUARD_BEGIN
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(SVO_ERR_NO_DEVICE, "svo_create: no CUDA device");
  if (device < 0 || device >= n) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_create: device index out of range");
  SVO_CUDA(cudaSetDevice(device), "svo_create: cudaSetDevice");
  std::unique_ptr<Context> c(new Context);
  c->device = device;
  SVO_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device), "svo_create: SM count");
  SVO_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking), "svo_create: stream");
  SVO_CUDA(cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming), "svo_create: event");
  c->stream = c->own_stream;
  c->cfg = svo::default_config();
  SVO_CUDA(c->counters.reserve(svo::kCounterWords), "svo_create: counters");
  SVO_CUDA(cudaMemset(c->counters.p, 0, svo::kCounterWords * sizeof(uint32_t)), "svo_create: counters");
  SVO_CUDA(c->stats.reserve(8), "svo_create: stats");
  SVO_CUDA(c->h_counters.reserve(svo::kErrorWords), "svo_create: pinned counters");
  *ctx = c.release();
  return SVO_OK;
  GUARD_END("svo_create")
}

SVO_API svo_status svo_destroy(void *ctx) {
  if (!ctx) return SVO_OK;
  delete static_cast<Context *>(ctx);
  return SVO_OK;
}

SVO_API svo_status svo_set_stream(void *ctx, void *stream) {
  CTX_OR_FAIL(ctx, "svo_set_stream");
  c.stream = stream ? static_cast<cudaStream_t>(stream) : c.own_stream;
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  c.graph_exec = nullptr;
  return SVO_OK;
}

SVO_API svo_status svo_synchronize(void *ctx) {
  CTX_OR_FAIL(ctx, "svo_synchronize");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_synchronize");
  return svo::report_kernel_error(c, "svo_synchronize");
}

SVO_API svo_status svo_set_trace_config(void *ctx, const svo_trace_config *cfg) {
  CTX_OR_FAIL(ctx, "svo_set_trace_config");
  if (!cfg) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_set_trace_config: null config");
  svo_trace_config d = svo::default_config(), n = *cfg;
  if (n.block_size == 0) n.block_size = d.block_size;
  if (n.ray_chunk == 0) n.ray_chunk = d.ray_chunk;
  if (n.cadence == 0) n.cadence = d.cadence;
  if (n.max_steps == 0) n.max_steps = d.max_steps;
  if (n.max_hits == 0) n.max_hits = d.max_hits;
  if (n.schedule == 0) n.schedule = d.schedule;
  if (n.l2_window == 0) n.l2_window = d.l2_window;
  if (n.request_order == 0) n.request_order = d.request_order;
  if (n.gi_stage == 0) n.gi_stage = -1;
  if (n.gi_stage != 1 && n.gi_stage != -1)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_set_trace_config: gi_stage must be 1 (on) or -1 / 0 (off)");
  if (n.request_order != SVO_REQUESTS_ARRIVAL && n.request_order != SVO_REQUESTS_PIXEL)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_set_trace_config: request_order must be SVO_REQUESTS_ARRIVAL or _PIXEL");
  if (n.pass_limit < 0) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_set_trace_config: pass_limit must be >= 0");
  if (n.block_size % 32 || n.block_size < 32 || n.block_size > 256)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_set_trace_config: block_size must be a multiple of 32 in 32..256");
  if (n.ray_chunk < 1 || n.ray_chunk > 64 || n.cadence < 1 || n.cadence > 1024 || n.max_steps < 1 || n.ctas_per_sm < 0 ||
      n.collect_stats < 0 || n.collect_stats > 2 || n.max_hits < 1 || n.max_hits > 1024 || n.mega_band_tiles < 0 ||
      (n.schedule != SVO_SCHEDULE_LANE && n.schedule != SVO_SCHEDULE_WARP && n.schedule != SVO_SCHEDULE_WAVEFRONT) ||
      (n.l2_window != 1 && n.l2_window != -1))
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_set_trace_config: value out of range");
  if (n.l2_window < 0) c.release_l2_set_aside();
  c.cfg = n;
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  c.graph_exec = nullptr;
  return SVO_OK;
}

SVO_API svo_status svo_get_trace_config(void *ctx, svo_trace_config *cfg) {
  CTX_OR_FAIL(ctx, "svo_get_trace_config");
  if (!cfg) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_get_trace_config: null config");
  *cfg = c.cfg;
  return SVO_OK;
}

SVO_API svo_status svo_upload_octree(void *ctx, uint8_t base_depth, const uint16_t *bases, size_t n_bases,
                                     const svo_block *blocks, size_t n_blocks, uint32_t block_budget) {
  CTX_OR_FAIL(ctx, "svo_upload_octree");
  GUARD_BEGIN
  if (base_depth < 1 || base_depth > 8) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_upload_octree: base_depth must be 1..8");
  if (!bases || n_bases != svo::pow_sum(base_depth))
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_upload_octree: need powSum(base_depth) base chunks");
  if (!blocks && n_blocks) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_upload_octree: null blocks");
  if (n_blocks > 0xFFFFFFF8ull) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_upload_octree: too many blocks");
  size_t dense = (size_t)1 << (3 * (base_depth + 2));
  size_t budget = std::max<size_t>({(size_t)block_budget, n_blocks, dense});
  budget = (budget + 7) & ~(size_t)7;
  if (budget > 0xFFFFFFF8ull) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_upload_octree: block budget too large");
  int depth = svo::scan_tree_depth(blocks, n_blocks, base_depth);
  if (depth > SVO_MAX_TREE_DEPTH) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_upload_octree: tree deeper than SVO_MAX_TREE_DEPTH");
  SVO_CUDA(cudaSetDevice(c.device), "cudaSetDevice");
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  c.graph_exec = nullptr;
  c.has_tree = false;
  c.has_params = false;  // per-node parameters belong to the previous tree
  if (c.bases.reserve(n_bases) || c.blocks.reserve(budget) || c.usage.reserve(budget / 8))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_upload_octree: device allocation failed");
  SVO_CUDA(cudaMemcpyAsync(c.bases.p, bases, n_bases * 2, cudaMemcpyHostToDevice, c.stream), "svo_upload_octree: bases");
  if (n_blocks)
    SVO_CUDA(cudaMemcpyAsync(c.blocks.p, blocks, n_blocks * sizeof(svo_block), cudaMemcpyHostToDevice, c.stream),
             "svo_upload_octree: blocks");
  if (budget > n_blocks)
    SVO_CUDA(cudaMemsetAsync(c.blocks.p + n_blocks, 0, (budget - n_blocks) * sizeof(svo_block), c.stream),
             "svo_upload_octree: block padding");
  SVO_CUDA(cudaMemsetAsync(c.usage.p, 0, budget / 8 * sizeof(svo_usage), c.stream), "svo_upload_octree: usage");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_upload_octree: synchronize");
  c.base_depth = base_depth;
  c.n_bases = n_bases;
  c.n_blocks = n_blocks;
  c.budget = budget;
  c.n_groups = budget / 8;
  c.tree_depth = std::max(depth, base_depth + 2);
  c.free_valid = false;
  c.free_used = c.n_free = c.n_pruned = c.n_freed = c.n_claimed = 0;
  c.has_tree = true;
  return SVO_OK;
  GUARD_END("svo_upload_octree")
}

SVO_API svo_status svo_init_usage(void *ctx) {
  CTX_OR_FAIL(ctx, "svo_init_usage");
  GUARD_BEGIN
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_init_usage: no octree uploaded");
  // MainWindow.cs:129-141: entries [0, 8^B) become inviolate when the level-B
  // base chunk of the same index has air+geometry in one of its low 4 octants.
  std::vector<uint16_t> hb(c.n_bases);
  SVO_CUDA(cudaMemcpy(hb.data(), c.bases.p, c.n_bases * 2, cudaMemcpyDeviceToHost), "svo_init_usage: read bases");
  uint32_t start = svo::pow_sum(c.base_depth - 1), range = svo::pow_sum(c.base_depth);
  std::vector<svo_usage> u(std::min<size_t>(range - start, c.n_groups));
  std::memset(u.data(), 0, u.size() * sizeof(svo_usage));
  for (size_t i = 0; i < u.size(); i++)
    for (uint32_t j = 3; j <= 255; j <<= 2)
      if ((hb[start + i] & j) == j) {
        u[i].tick = 65535;
        u[i].parent = 0xFFFFFFFFu;
        break;
      }
  SVO_CUDA(cudaMemsetAsync(c.usage.p, 0, c.n_groups * sizeof(svo_usage), c.stream), "svo_init_usage: clear");
  SVO_CUDA(cudaMemcpyAsync(c.usage.p, u.data(), u.size() * sizeof(svo_usage), cudaMemcpyHostToDevice, c.stream),
           "svo_init_usage: write");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_init_usage: synchronize");
  return SVO_OK;
  GUARD_END("svo_init_usage")
}

SVO_API svo_status svo_read_usage(void *ctx, svo_usage *out, size_t n_groups) {
  CTX_OR_FAIL(ctx, "svo_read_usage");
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_read_usage: no octree uploaded");
  if (!out || n_groups > c.n_groups) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_read_usage: bad output");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_usage: synchronize");
  SVO_CUDA(cudaMemcpy(out, c.usage.p, n_groups * sizeof(svo_usage), cudaMemcpyDeviceToHost), "svo_read_usage");
  return SVO_OK;
}

SVO_API svo_status svo_write_usage(void *ctx, const svo_usage *in, size_t n_groups) {
  CTX_OR_FAIL(ctx, "svo_write_usage");
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_write_usage: no octree uploaded");
  if (!in || n_groups > c.n_groups) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_write_usage: bad input");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_write_usage: synchronize");
  SVO_CUDA(cudaMemcpy(c.usage.p, in, n_groups * sizeof(svo_usage), cudaMemcpyHostToDevice), "svo_write_usage");
  return SVO_OK;
}

SVO_API svo_status svo_read_blocks(void *ctx, svo_block *out, size_t first, size_t n) {
  CTX_OR_FAIL(ctx, "svo_read_blocks");
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_read_blocks: no octree uploaded");
  if (!out || first > c.budget || n > c.budget - first) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_read_blocks: range");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_blocks: synchronize");
  SVO_CUDA(cudaMemcpy(out, c.blocks.p + first, n * sizeof(svo_block), cudaMemcpyDeviceToHost), "svo_read_blocks");
  return SVO_OK;
}

SVO_API svo_status svo_read_bases(void *ctx, uint16_t *out, size_t n) {
  CTX_OR_FAIL(ctx, "svo_read_bases");
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_read_bases: no octree uploaded");
  if (!out || n > c.n_bases) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_read_bases: range");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_bases: synchronize");
  SVO_CUDA(cudaMemcpy(out, c.bases.p, n * 2, cudaMemcpyDeviceToHost), "svo_read_bases");
  return SVO_OK;
}

SVO_API svo_status svo_tree_size(void *ctx, uint8_t *base_depth, size_t *n_bases, size_t *n_blocks,
                                 size_t *block_budget) {
  CTX_OR_FAIL(ctx, "svo_tree_size");
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_tree_size: no octree uploaded");
  if (base_depth) *base_depth = c.base_depth;
  if (n_bases) *n_bases = c.n_bases;
  if (n_blocks) *n_blocks = c.n_blocks;
  if (block_budget) *block_budget = c.budget;
  return SVO_OK;
}

SVO_API svo_status svo_trace(void *ctx, const svo_trace_input *input, const svo_trace_output *out) {
  CTX_OR_FAIL(ctx, "svo_trace");
  GUARD_BEGIN
  return svo::run_trace(c, input, 1, out, false);
  GUARD_END("svo_trace")
}

SVO_API svo_status svo_trace_batch(void *ctx, const svo_trace_input *inputs, int32_t n_views,
                                   const svo_trace_output *out) {
  CTX_OR_FAIL(ctx, "svo_trace_batch");
  GUARD_BEGIN
  return svo::run_trace(c, inputs, n_views, out, false);
  GUARD_END("svo_trace_batch")
}

SVO_API svo_status svo_trace_batch_graph(void *ctx, const svo_trace_input *inputs, int32_t n_views,
                                         const svo_trace_output *out) {
  CTX_OR_FAIL(ctx, "svo_trace_batch_graph");
  GUARD_BEGIN
  return svo::run_trace(c, inputs, n_views, out, true);
  GUARD_END("svo_trace_batch_graph")
}

SVO_API svo_status svo_autotune(void *ctx, const svo_trace_input *inputs, int32_t n_views,
                                const svo_trace_output *out, int32_t repeats, svo_trace_config *best,
                                float *best_ms) {
  CTX_OR_FAIL(ctx, "svo_autotune");
  GUARD_BEGIN
  if (n_views <= 0 || !inputs || !out) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_autotune: bad view list");
  for (int i = 0; i < n_views; i++)
    if (!out[i].on_device) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_autotune: outputs must be device pointers");
  if (repeats <= 0) repeats = 3;
  SVO_CUDA(cudaSetDevice(c.device), "cudaSetDevice");
  svo_trace_config base = c.cfg, chosen = c.cfg;
  base.collect_stats = 0;
  float chosen_ms = 1e30f;
  cudaEvent_t e0, e1;
  SVO_CUDA(cudaEventCreate(&e0), "svo_autotune: event");
  SVO_CUDA(cudaEventCreate(&e1), "svo_autotune: event");
  svo_status st = SVO_OK;
  // Scheduling, block size, rays claimed per queue fetch and steps between
  // retire points (the last two for lane scheduling only); results do not
  // depend on any of them, only the time does.
  const int sizes[] = {64, 128, 192, 256};
  const int chunks[] = {1, 2, 4, 8};
  const int cadences[] = {4, 8, 16, 32};
  std::vector<svo_trace_config> cands;
  for (int bs : sizes) {
    svo_trace_config cfg = base;
    cfg.block_size = bs;
    cfg.schedule = SVO_SCHEDULE_WARP;
    cands.push_back(cfg);
    cfg.schedule = SVO_SCHEDULE_WAVEFRONT;
    cands.push_back(cfg);
    for (int ch : chunks)
      for (int cd : cadences) {
        cfg.schedule = SVO_SCHEDULE_LANE;
        cfg.ray_chunk = ch;
        cfg.cadence = cd;
        cands.push_back(cfg);
      }
  }
  for (const svo_trace_config &cfg : cands) {
        if (st) break;
        c.cfg = cfg;
        st = svo::run_trace(c, inputs, n_views, out, false);  // warm-up
        if (st) break;
        float best_rep = 1e30f;
        for (int r = 0; r < repeats && !st; r++) {
          cudaEventRecord(e0, c.stream);
          st = svo::run_trace(c, inputs, n_views, out, false);
          cudaEventRecord(e1, c.stream);
          if (cudaEventSynchronize(e1) != cudaSuccess) st = fail(SVO_ERR_CUDA, "svo_autotune: event sync");
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          best_rep = std::min(best_rep, ms);
        }
        if (!st && best_rep < chosen_ms) {
          chosen_ms = best_rep;
          chosen = cfg;
        }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  chosen.collect_stats = 0;
  c.cfg = st ? base : chosen;
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  c.graph_exec = nullptr;
  if (st) return st;
  if (best) *best = chosen;
  if (best_ms) *best_ms = chosen_ms;
  return SVO_OK;
  GUARD_END("svo_autotune")
}

SVO_API svo_status svo_last_trace_stats(void *ctx, svo_trace_stats *stats) {
  CTX_OR_FAIL(ctx, "svo_last_trace_stats");
  if (!stats) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_last_trace_stats: null output");
  std::memset(stats, 0, sizeof(*stats));
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_last_trace_stats: synchronize");
  uint32_t counters[2];
  SVO_CUDA(cudaMemcpy(counters, c.counters.p, sizeof(counters), cudaMemcpyDeviceToHost), "svo_last_trace_stats: counters");
  stats->rays = c.last_rays;
  stats->child_requests = counters[1];
  if (c.last_stats_valid) {
    unsigned long long v[7];
    SVO_CUDA(cudaMemcpy(v, c.stats.p, sizeof(v), cudaMemcpyDeviceToHost), "svo_last_trace_stats: stats");
    stats->hits = v[1];
    stats->base_steps = v[2];
    stats->block_node_reads = v[3];
    stats->block_steps = v[4];
    stats->step_limited = v[6];
  }
  return SVO_OK;
}

SVO_API svo_status svo_read_ray_counts(void *ctx, uint32_t *v_block, uint32_t *v_base, size_t n) {
  CTX_OR_FAIL(ctx, "svo_read_ray_counts");
  if (!c.last_stats_valid || c.cfg.collect_stats < 2 || n > c.last_rays)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_read_ray_counts: last trace had no per-ray counts");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_ray_counts: synchronize");
  if (v_block) SVO_CUDA(cudaMemcpy(v_block, c.ray_v_block.p, n * 4, cudaMemcpyDeviceToHost), "svo_read_ray_counts");
  if (v_base) SVO_CUDA(cudaMemcpy(v_base, c.ray_v_base.p, n * 4, cudaMemcpyDeviceToHost), "svo_read_ray_counts");
  return SVO_OK;
}

SVO_API svo_status svo_read_child_requests(void *ctx, svo_child_request *out, uint32_t cap, uint32_t *n) {
  CTX_OR_FAIL(ctx, "svo_read_child_requests");
  if (!n) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_read_child_requests: null count");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_child_requests: synchronize");
  uint32_t raised = 0;
  SVO_CUDA(cudaMemcpy(&raised, c.counters.p + 1, 4, cudaMemcpyDeviceToHost), "svo_read_child_requests: count");
  *n = raised;
  uint32_t stored = std::min(raised, c.request_cap);
  uint32_t copy = std::min(stored, cap);
  if (copy && out)
    SVO_CUDA(cudaMemcpy(out, c.requests.p, (size_t)copy * sizeof(svo_child_request), cudaMemcpyDeviceToHost),
             "svo_read_child_requests: records");
  return SVO_OK;
}

}  // extern "C"
