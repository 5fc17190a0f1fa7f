// C ABI of the megakernel path: svo_mega_trace (kernel.cl's `trace` over a
// view) and svo_last_mega_stats. The kernels are in mega_kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

namespace svo {
namespace {

constexpr float kPiF = 3.14159274101257324219f;   // M_PI_F
constexpr float kPi2F = 1.57079637050628662109f;  // M_PI_2_F
// Cone slots of one band (16 + 2 + 1 bytes each).
constexpr uint64_t kBandSlots = 1ull << 26;

}  // namespace

// spawnRays's spine and ring loops (kernel.cl:1115-1253) evaluated once per
// input: they depend only on FovMultiplier/Constant and
// WeightingMultiplier/Constant. native_sin/cos are (float)sin((double)x).
// Returns the cones of a fan that takes no `break` (the slot stride), or 0 when
// that exceeds SVO_MEGA_MAX_CONES.
static int32_t build_schedule(const svo_trace_input &in, std::vector<MegaSpine> &spines, std::vector<MegaRing> &rings) {
  spines.clear();
  rings.clear();
  const float FM = in.fov_multiplier, FC = in.fov_constant;
  float fov = FC, oldfov = fov, spine = 0.0f;
  int64_t cones = 1;  // the reflection cone
  while (spine < kPiF) {
    fov = (FM * (spine + fov) + FC) / (1 - FM);
    spine = (1 + FM) * (spine + oldfov) / (1 - FM);
    oldfov = fov;
    MegaSpine sp{};
    sp.fov = fov;
    sp.weighting = spine * in.weighting_multiplier + in.weighting_constant;
    sp.c = (float)std::cos((double)(-spine));
    sp.s = (float)std::sin((double)(-spine));
    sp.k = 1.0f - sp.c;
    sp.ring_begin = (uint32_t)rings.size();
    cones += 1;
    for (int j = 1; (float)j * fov < kPi2F; j++) {
      cones += 2;
      if (cones > SVO_MEGA_MAX_CONES) return 0;
      const float angle = (float)(j * 2) * fov;
      MegaRing rg{};
      rg.c = (float)std::cos((double)(-angle));
      rg.s = (float)std::sin((double)(-angle));
      rg.k = 1.0f - rg.c;
      rings.push_back(rg);
    }
    sp.n_rings = (uint32_t)rings.size() - sp.ring_begin;
    spines.push_back(sp);
    if (cones > SVO_MEGA_MAX_CONES) return 0;
  }
  return (int32_t)cones;
}

int32_t ensure_cone_schedule(Context &c, const svo_trace_input &in, svo_status &st) {
  st = SVO_OK;
  uint32_t key[4];
  std::memcpy(&key[0], &in.fov_multiplier, 4);
  std::memcpy(&key[1], &in.fov_constant, 4);
  std::memcpy(&key[2], &in.weighting_multiplier, 4);
  std::memcpy(&key[3], &in.weighting_constant, 4);
  const std::array<uint32_t, 4> k4{key[0], key[1], key[2], key[3]};
  if (c.mega_sched_valid && c.mega_sched_key == k4) return c.mega_k_max;
  std::vector<MegaSpine> spines;
  std::vector<MegaRing> rings;
  const int32_t k_max = build_schedule(in, spines, rings);
  if (k_max <= 0) return 0;
  if (c.mega_spine.reserve(std::max<size_t>(1, spines.size())) || c.mega_ring.reserve(std::max<size_t>(1, rings.size()))) {
    st = fail(SVO_ERR_OUT_OF_MEMORY, "cone schedule allocation");
    return 0;
  }
  // a running kernel may still read the old schedule
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (e == cudaSuccess && !spines.empty())
    e = cudaMemcpy(c.mega_spine.p, spines.data(), sizeof(MegaSpine) * spines.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !rings.empty())
    e = cudaMemcpy(c.mega_ring.p, rings.data(), sizeof(MegaRing) * rings.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    st = fail(SVO_ERR_CUDA, std::string("cone schedule upload: ") + cudaGetErrorString(e));
    return 0;
  }
  c.mega_sched_key = k4;
  c.mega_sched_valid = true;
  c.mega_n_spines = (int32_t)spines.size();
  c.mega_k_max = k_max;
  return k_max;
}

svo_status ensure_normal_table(Context &c) {
  if (c.mega_normal_sc.n == 65536) return SVO_OK;
  // normalVector (kernel.cl:264-275): angle = a * M_PI_F / 32767.0f
  std::vector<float2> tab(65536);
  for (int a = -32768; a <= 32767; a++) {
    const float x = (float)a * kPiF / 32767.0f;
    tab[a + 32768] = make_float2((float)std::sin((double)x), (float)std::cos((double)x));
  }
  if (c.mega_normal_sc.reserve(65536)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_mega_trace: normal table allocation");
  SVO_CUDA(cudaMemcpy(c.mega_normal_sc.p, tab.data(), sizeof(float2) * 65536, cudaMemcpyHostToDevice),
           "svo_mega_trace: normal table");
  return SVO_OK;
}

namespace {

svo_status read_error(Context &c, const char *fn) { return report_kernel_error(c, fn); }

svo_status run_mega(Context &c, const svo_trace_input *in, const svo_trace_output *out_in) {
  const char *fn = "svo_mega_trace";
  if (!in || !out_in) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_mega_trace: null argument");
  c.last_mega = svo_mega_stats{};
  // kernel.cl:1533-1534: the kernel returns without drawing
  if (in->fov_constant <= 0 || in->fov_multiplier >= 1 || in->fov_multiplier <= -1) return SVO_OK;
  if (c.cfg.block_size % 32 || c.cfg.block_size > 256)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_mega_trace: block size must be a multiple of 32 up to 256");

  // the cone schedule, uploaded when the input's cone parameters change
  svo_status st = SVO_OK;
  if (ensure_cone_schedule(c, *in, st) <= 0)
    return st ? st
              : fail(SVO_ERR_INVALID_ARGUMENT,
                     "svo_mega_trace: the cone schedule exceeds SVO_MEGA_MAX_CONES cones per pixel (its loops would not end)");
  st = ensure_normal_table(c);
  if (st) return st;

  // outputs: device pointers, pinned host memory the kernels write directly
  // (but for the outputs in kStagedHostOutputs, which go to library buffers and
  // one copy each, as in svo_trace), or library buffers copied back to pageable
  // host memory
  svo_trace_output out = *out_in;
  const svo_trace_output caller = *out_in;
  const bool host_outputs = out.on_device == 0;
  bool direct = !host_outputs;
  uint32_t staged = 0;  // outputs of pinned buffers staged in library buffers
  if (host_outputs) {
    svo_trace_output mapped = out;
    bool all_pinned = true;
    void **ptrs[4] = {reinterpret_cast<void **>(&mapped.hit_index), reinterpret_cast<void **>(&mapped.hit_depth),
                      reinterpret_cast<void **>(&mapped.t), reinterpret_cast<void **>(&mapped.rgba)};
    for (int k = 0; k < 4; k++) {
      void **pp = ptrs[k];
      if (!*pp) continue;
      void *d = pinned_device_ptr(*pp);
      if (!d) {
        all_pinned = false;
        break;
      }
      if (kStagedHostOutputs & (1u << k))
        staged |= 1u << k;
      else
        *pp = d;
    }
    if (all_pinned) {
      mapped.on_device = 1;
      out = mapped;
      direct = true;
    } else {
      staged = 0;
    }
  }
  const size_t pixels = (size_t)in->screen_size[0] * in->screen_size[1];
  if (staged) {
    if (((staged & 1u) && c.o_index.reserve(pixels)) || ((staged & 2u) && c.o_depth.reserve(pixels)) ||
        ((staged & 4u) && c.o_t.reserve(pixels)) || ((staged & 8u) && c.o_rgba.reserve(4 * pixels)))
      return fail(SVO_ERR_OUT_OF_MEMORY, "svo_mega_trace: output buffer allocation failed");
    if (staged & 1u) out.hit_index = c.o_index.p;
    if (staged & 2u) out.hit_depth = c.o_depth.p;
    if (staged & 4u) out.t = c.o_t.p;
    if (staged & 8u) out.rgba = c.o_rgba.p;
  }
  if (!direct && (c.o_index.reserve(pixels) || c.o_depth.reserve(pixels) || c.o_t.reserve(pixels) ||
                  c.o_rgba.reserve(4 * pixels)))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_mega_trace: output buffer allocation failed");
  if (c.requests.reserve(in->max_child_request_id) != cudaSuccess)
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_mega_trace: request queue allocation");
  c.request_cap = in->max_child_request_id;

  SVO_CUDA(cudaEventSynchronize(c.staged), "svo_mega_trace: staging");
  uint32_t total_rays = 0, total_pixels = 0;
  size_t table_floats = 0;
  st = stage_views(c, in, 1, &out, direct, kTraceTileW, total_rays, total_pixels, table_floats);
  if (st) return st;
  const uint32_t n_tiles = total_rays / 32;
  const int32_t K = c.mega_k_max;
  const uint64_t band_pref = c.cfg.mega_band_tiles > 0 ? (uint64_t)c.cfg.mega_band_tiles : kBandSlots / (32ull * (uint64_t)K);
  const uint32_t band_tiles = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(n_tiles, band_pref));
  const size_t band_slots = (size_t)band_tiles * K * 32;
  if (c.views.reserve(1) || c.tables.reserve(table_floats) || c.mega_pix.reserve(total_rays) ||
      c.mega_cone_dw.reserve(band_slots) || c.mega_cone_s.reserve(band_slots) || c.mega_cone_sky.reserve(band_slots) ||
      c.mega_tile_cones.reserve(band_tiles) || c.mega_entries.reserve(band_slots) || c.mega_queue.reserve(2) ||
      c.mega_totals.reserve(2) || c.h_mega_totals.reserve(2))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_mega_trace: allocation failed");

  MegaLaunch m{};
  // collect_stats: the primary and cone kernels count their reference-walk reads
  // (svo_last_trace_stats; rays = primary + secondary cones)
  const bool stats = c.cfg.collect_stats > 0;
  st = prepare_launch(c, 1, total_rays, m.t, stats);
  if (st) return st;
  m.t.schedule = c.cfg.schedule == SVO_SCHEDULE_LANE ? SVO_SCHEDULE_LANE : SVO_SCHEDULE_WARP;  // the cone kernel's two
  m.pix = c.mega_pix.p;
  m.cone_dw = c.mega_cone_dw.p;
  m.cone_s = c.mega_cone_s.p;
  m.cone_sky = c.mega_cone_sky.p;
  m.tile_cones = c.mega_tile_cones.p;
  m.entries = c.mega_entries.p;
  m.queue = c.mega_queue.p;
  m.max_entries = (uint32_t)band_slots;
  m.cone_schedule = c.cfg.schedule;
  m.normal_sc = c.mega_normal_sc.p;
  m.spine = c.mega_spine.p;
  m.ring = c.mega_ring.p;
  m.totals = c.mega_totals.p;
  m.n_spines = c.mega_n_spines;
  m.k_max = K;
  m.fov_c = in->fov_constant;
  m.weighting_c = in->weighting_constant;
  const int occ = c.cfg.ctas_per_sm > 0 ? c.cfg.ctas_per_sm : mega_occupancy(m);
  if (occ <= 0) return fail(SVO_ERR_NO_DEVICE, "svo_mega_trace: the megakernel cannot be resident");
  const long persistent = (long)occ * c.sm_count;
  m.t.grid = (int)std::max(1L, std::min(persistent, ((long)total_rays + m.t.block_size - 1) / m.t.block_size));

  SVO_CUDA(cudaMemcpyAsync(c.views.p, c.h_views.p, sizeof(ViewParams), cudaMemcpyHostToDevice, c.stream), fn);
  SVO_CUDA(cudaMemcpyAsync(c.tables.p, c.h_tables.p, sizeof(float) * table_floats, cudaMemcpyHostToDevice, c.stream),
           fn);
  SVO_CUDA(cudaEventRecord(c.staged, c.stream), fn);
  SVO_CUDA(cudaMemsetAsync(c.counters.p, 0, kErrorOffset * sizeof(uint32_t), c.stream), fn);
  SVO_CUDA(cudaMemsetAsync(c.mega_totals.p, 0, 2 * sizeof(unsigned long long), c.stream), fn);
  if (stats) SVO_CUDA(cudaMemsetAsync(c.stats.p, 0, 8 * sizeof(unsigned long long), c.stream), fn);
  st = launch_mega_primary(m, c.stream);
  if (st) return st;
  uint64_t slots = 0;
  for (uint32_t t0 = 0; t0 < n_tiles; t0 += band_tiles) {
    m.band_tile0 = t0;
    m.band_tiles = std::min(band_tiles, n_tiles - t0);
    const uint64_t band_cone_slots = (uint64_t)m.band_tiles * (uint32_t)K * 32;
    m.grid_cones = (int)std::max(1L, std::min(persistent, (long)((band_cone_slots + m.t.block_size - 1) / m.t.block_size)));
    slots += band_cone_slots;
    st = launch_mega_band(m, c.stream);
    if (st) return st;
  }
  SVO_CUDA(cudaMemcpyAsync(c.h_mega_totals.p, c.mega_totals.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           c.stream),
           fn);
  if (staged & 1u) SVO_CUDA(cudaMemcpyAsync(caller.hit_index, c.o_index.p, pixels * 4, cudaMemcpyDeviceToHost, c.stream), fn);
  if (staged & 2u) SVO_CUDA(cudaMemcpyAsync(caller.hit_depth, c.o_depth.p, pixels, cudaMemcpyDeviceToHost, c.stream), fn);
  if (staged & 4u) SVO_CUDA(cudaMemcpyAsync(caller.t, c.o_t.p, pixels * 4, cudaMemcpyDeviceToHost, c.stream), fn);
  if (staged & 8u) SVO_CUDA(cudaMemcpyAsync(caller.rgba, c.o_rgba.p, pixels * 16, cudaMemcpyDeviceToHost, c.stream), fn);
  if (!direct) {
    if (out.hit_index)
      SVO_CUDA(cudaMemcpyAsync(out.hit_index, c.o_index.p, pixels * 4, cudaMemcpyDeviceToHost, c.stream), fn);
    if (out.hit_depth)
      SVO_CUDA(cudaMemcpyAsync(out.hit_depth, c.o_depth.p, pixels, cudaMemcpyDeviceToHost, c.stream), fn);
    if (out.t) SVO_CUDA(cudaMemcpyAsync(out.t, c.o_t.p, pixels * 4, cudaMemcpyDeviceToHost, c.stream), fn);
    if (out.rgba) SVO_CUDA(cudaMemcpyAsync(out.rgba, c.o_rgba.p, pixels * 16, cudaMemcpyDeviceToHost, c.stream), fn);
  }
  st = read_error(c, fn);  // one synchronisation: outputs, totals and the error record
  if (st) return st;
  c.last_rays = total_pixels;
  c.last_stats_valid = stats;
  c.last_mega.pixels = total_pixels;
  c.last_mega.cones = c.h_mega_totals.p[0];
  c.last_mega.surfaces = c.h_mega_totals.p[1];
  c.last_mega.cone_slots = slots;
  return SVO_OK;
}

}  // namespace
}  // namespace svo

using svo::Context;
using svo::fail;

extern "C" {

SVO_API svo_status svo_mega_trace(void *ctx, const svo_trace_input *input, const svo_trace_output *out) {
  if (!ctx) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_mega_trace: null context");
  Context &c = *static_cast<Context *>(ctx);
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_mega_trace: no octree uploaded");
  SVO_CUDA(cudaSetDevice(c.device), "cudaSetDevice");
  try {
    return svo::run_mega(c, input, out);
  } catch (const std::bad_alloc &) {
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_mega_trace: out of host memory");
  } catch (const std::exception &e) {
    return fail(SVO_ERR_INTERNAL, std::string("svo_mega_trace: ") + e.what());
  }
}

SVO_API svo_status svo_last_mega_stats(void *ctx, svo_mega_stats *stats) {
  if (!ctx) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_last_mega_stats: null context");
  if (!stats) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_last_mega_stats: null output");
  *stats = static_cast<Context *>(ctx)->last_mega;
  return SVO_OK;
}

}  // extern "C"
