// Context of libsvo (one GPU, one stream) and device-buffer helpers, shared by
// the translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <string>
#include <vector>

#include "mega_internal.h"
#include "svo_internal.h"

namespace svo {

#define SVO_CUDA(call, what)                                                                  \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(SVO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T));
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

template <class T>
struct PinBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMallocHost(&p, std::max<size_t>(want, 1) * sizeof(T));
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

struct Context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // resident tree
  bool has_tree = false;
  uint8_t base_depth = 0;
  size_t n_bases = 0, n_blocks = 0, budget = 0, n_groups = 0;
  int tree_depth = 0;
  DevBuf<uint16_t> bases;
  DevBuf<svo_block> blocks;
  DevBuf<svo_usage> usage;
  // trace scratch
  // kCounterWords: [0] ray queue head, [1] child requests raised, then the
  // kernel error record at kErrorOffset. Launches reset the words before the
  // record; the record keeps a stopped kernel's report until a synchronising
  // call returns it (report_kernel_error), which clears it.
  DevBuf<uint32_t> counters;
  DevBuf<unsigned long long> stats;
  DevBuf<svo_child_request> requests;
  // pixel-order requests: the staged record and flag per pixel, chunk offsets
  DevBuf<StagedRequest> req_stage;
  DevBuf<uint8_t> req_flag;
  DevBuf<uint32_t> req_chunks;
  // the material stage (gi_stage): hit indices of views whose caller asked for none
  DevBuf<uint32_t> gi_hit;
  DevBuf<ViewParams> views;
  DevBuf<float> tables;
  DevBuf<uint32_t> ray_v_block, ray_v_base;
  PinBuf<ViewParams> h_views;
  PinBuf<float> h_tables;
  PinBuf<uint32_t> h_counters;
  // library-owned outputs for host-memory results
  DevBuf<uint32_t> o_index;
  DevBuf<uint8_t> o_depth;
  DevBuf<float> o_t;
  DevBuf<float> o_rgba;
  uint32_t request_cap = 0;
  uint64_t last_rays = 0;
  bool last_stats_valid = false;
  svo_trace_config cfg{};
  // recorded after the view/table uploads: the pinned staging may be rewritten once it fired
  cudaEvent_t staged = nullptr;
  // tree updates: reachability marks, stale/freed flags, free list
  DevBuf<uint32_t> reach, parent_min, frontier_a, frontier_b, scan_tmp;
  DevBuf<uint8_t> flags;
  DevBuf<uint32_t> free_list, pruned_list, freed_list, claimed_list;
  DevBuf<svo_block> payload;
  DevBuf<svo_grafting> graft_records;
  DevBuf<uint32_t> graft_jobs, graft_targets;
  DevBuf<svo_pruning> prune_records;
  DevBuf<uint64_t> locations;
  // ray-setup tables (sin/cos per column and row) by (fov bits, width, height)
  std::map<std::array<uint32_t, 4>, std::vector<float>> table_cache;

  // graft payloads generated on the device: the terrain's column pyramids (all
  // levels concatenated) of the scene `terrain_id`, a per-node request marker
  // (kept zero between calls), compaction counts, jobs and counters
  DevBuf<uint16_t> terrain_lo, terrain_hi;
  uint64_t terrain_id = 0;
  DevBuf<uint32_t> gen_marker, gen_bits, gen_counts, gen_addr, gen_groups, gen_scalars;
  DevBuf<uint8_t> gen_jobs;

  // differentiable colour fitting: per-node RGBA parameters and gradients
  DevBuf<float> params, grads, diff_rgb, diff_target;
  DevBuf<float> diff_saved;  // forward colour as (hi, lo) float pairs, 6 per ray
  DevBuf<double> diff_loss;
  bool has_params = false;
  uint64_t params_gen = 0;   // bumped by every parameter upload
  // what diff_saved holds: the views, parameter generation and max_hits of the last forward
  std::vector<svo_trace_input> saved_views;
  uint64_t saved_params_gen = 0;
  int32_t saved_max_hits = 0;
  bool saved_valid = false;
  // megakernel: per-slot pixel records, one band's cone slots, normalVector's
  // table of the int16 angles, the cone schedule of the last input (by the bits
  // of FovMultiplier, FovConstant, WeightingMultiplier, WeightingConstant)
  DevBuf<MegaPixel> mega_pix;
  DevBuf<float4> mega_cone_dw;
  DevBuf<uint16_t> mega_cone_s;
  DevBuf<uint32_t> mega_tile_cones, mega_entries, mega_queue;
  DevBuf<uint8_t> mega_cone_sky;
  DevBuf<float2> mega_normal_sc;
  DevBuf<MegaSpine> mega_spine;
  DevBuf<MegaRing> mega_ring;
  DevBuf<unsigned long long> mega_totals;
  PinBuf<unsigned long long> h_mega_totals;
  std::array<uint32_t, 4> mega_sched_key{};
  bool mega_sched_valid = false;
  int32_t mega_n_spines = 0, mega_k_max = 0;
  svo_mega_stats last_mega{};
  uint64_t n_free = 0, free_used = 0, n_pruned = 0, n_freed = 0, n_claimed = 0;
  bool free_valid = false;
  // L2 set-aside for persisting accesses taken by this context (restored on release)
  bool l2_limit_set = false;
  size_t l2_limit_prev = 0;
  void release_l2_set_aside() {
    if (!l2_limit_set) return;
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, l2_limit_prev);
    cudaGetLastError();
    l2_limit_set = false;
  }
  // graph cache for svo_trace_batch_graph
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<uint32_t> graph_key;
  // the GC's launch sequence as a graph (svo_gc), its key, the tick/threshold
  // word it copies in and the counts it copies out (pinned)
  cudaGraphExec_t gc_exec = nullptr;
  std::vector<uint64_t> gc_key;
  DevBuf<uint32_t> gc_params;
  PinBuf<uint32_t> h_gc_params, h_gc_out;

  ~Context() {
    if (device >= 0) cudaSetDevice(device);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (gc_exec) cudaGraphExecDestroy(gc_exec);
    gc_params.release();
    h_gc_params.release();
    h_gc_out.release();
    release_l2_set_aside();
    if (staged) cudaEventDestroy(staged);
    bases.release();
    blocks.release();
    usage.release();
    gi_hit.release();
    req_stage.release();
    req_flag.release();
    req_chunks.release();
    counters.release();
    stats.release();
    requests.release();
    views.release();
    tables.release();
    ray_v_block.release();
    ray_v_base.release();
    h_views.release();
    h_tables.release();
    h_counters.release();
    o_index.release();
    o_depth.release();
    o_t.release();
    o_rgba.release();
    reach.release();
    parent_min.release();
    frontier_a.release();
    frontier_b.release();
    scan_tmp.release();
    flags.release();
    free_list.release();
    pruned_list.release();
    freed_list.release();
    claimed_list.release();
    payload.release();
    graft_records.release();
    graft_jobs.release();
    graft_targets.release();
    prune_records.release();
    locations.release();
    params.release();
    grads.release();
    diff_rgb.release();
    diff_target.release();
    terrain_lo.release();
    terrain_hi.release();
    gen_marker.release();
    gen_bits.release();
    gen_groups.release();
    gen_counts.release();
    gen_addr.release();
    gen_scalars.release();
    gen_jobs.release();
    diff_saved.release();
    diff_loss.release();
    mega_pix.release();
    mega_cone_dw.release();
    mega_cone_s.release();
    mega_tile_cones.release();
    mega_entries.release();
    mega_queue.release();
    mega_cone_sky.release();
    mega_normal_sc.release();
    mega_spine.release();
    mega_ring.release();
    mega_totals.release();
    h_mega_totals.release();
    if (own_stream) cudaStreamDestroy(own_stream);
  }
};


// The device address of pinned (page-locked, registered) host memory, which
// kernels can read and write directly; nullptr for any other pointer.
inline void *pinned_device_ptr(const void *p) {
  cudaPointerAttributes at{};
  if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer is not an error here
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Views, ray-setup tables and outputs of a batch into pinned staging. With a
// tile width, each view's ray slots cover whole tile_w x (32 / tile_w) pixel
// tiles (total_rays then exceeds total_pixels by the padding slots); 0 = rows.
svo_status stage_views(Context &c, const svo_trace_input *in, int32_t n, const svo_trace_output *out,
                       bool outputs_on_device, uint32_t tile_w, uint32_t &total_rays, uint32_t &total_pixels,
                       size_t &table_floats, uint32_t *hit_fallback = nullptr);
svo_status prepare_launch(Context &c, int32_t n_views, uint32_t total_rays, TraceLaunch &a, bool stats);
// Synchronises the context's stream and returns the error a kernel recorded
// since the last report (SVO_ERR_TIMEOUT with the stopped thread's ray, depth
// and steps), clearing the record; SVO_OK when none did.
svo_status report_kernel_error(Context &c, const char *fn);
// Reserves the tree updates' scratch for the context's budget (tree_ops.cu).
svo_status ensure_tree_buffers(Context &c);

}  // namespace svo
