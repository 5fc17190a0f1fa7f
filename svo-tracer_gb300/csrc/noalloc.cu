// svo_trace_noalloc: a trace entry point that allocates no memory.
//
// Some callers cannot allocate device memory themselves: an engine whose
// renderer owns every GPU allocation through its own pool, a host loop running
// in a real-time thread where cudaMalloc's implicit synchronisation and
// unbounded latency are not allowed, or code that runs while a CUDA graph is
// being captured elsewhere. They can still trace into buffers they already own.
// This entry point traces one view of a tree the caller keeps in device memory
// into output buffers the caller owns; the little scratch memory the trace
// kernel needs (ray queue head, child-request counter, error record, the view
// record and the ray-setup sine/cosine tables) lives in a file-scope device
// array of fixed size, so the call performs no cudaMalloc/cudaFree and creates
// no context-owned buffer. It runs the library's default schedule (warp
// batches over 4x8 pixel tiles), so its results are those of svo_trace.
//
// Limits and sharing rules:
//  * the static scratch holds 132 KiB; it allows views with
//    width + height <= 16384 (larger views are rejected with
//    SVO_ERR_INVALID_ARGUMENT);
//  * every process that loads libsvo keeps those 132 KiB on every GPU it uses
//    until it exits;
//  * every call uses the same scratch, which keeps the previous call's
//    contents; the call clears the counters it needs at the start. Two calls
//    whose work overlapped on the GPU would race on it, so a process-wide lock
//    is held from the staging of a call until its trace has completed: calls
//    from different host threads run one after another, and a call blocks
//    while another thread's call is tracing. What the lock cannot order is the
//    caller's own work on the outputs, the usage array or the request array
//    (on other streams): that must not run while a call traces;
//  * the call switches to `device` for its work and restores the calling
//    thread's current device before it returns;
//  * the first call on a device looks up the scratch's device address on that
//    device (cudaGetSymbolAddress) and caches it; make that first call before
//    any stream capture on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "svo_internal.h"

namespace svo {
namespace {

constexpr size_t kScratchBytes = 132 * 1024;
constexpr uint32_t kMaxWidthPlusHeight = 16384;
constexpr size_t kCountersOff = 0;  // 16 words: queue head, request count, 2 spare, error record
constexpr size_t kViewOff = 256;    // one ViewParams
constexpr size_t kTablesOff = 512;  // 2 * (W + H) floats
constexpr int kMaxDevices = 64;
static_assert(kTablesOff + 2 * sizeof(float) * kMaxWidthPlusHeight <= kScratchBytes, "scratch layout");
static_assert(kViewOff + sizeof(ViewParams) <= kTablesOff, "scratch layout");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host-side staging for the view record and the tables (static: no allocation).
ViewParams g_host_view;
float g_host_tables[2 * kMaxWidthPlusHeight];
std::mutex g_lock;
unsigned char *g_scratch_ptr[kMaxDevices];

// Restores the calling thread's current device when a call returns.
struct DeviceRestore {
  int prev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      prev = -1;
      cudaGetLastError();
    }
  }
  ~DeviceRestore() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

svo_status scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: device index");
  if (!g_scratch_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess)
      return fail(SVO_ERR_CUDA, std::string("svo_trace_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_scratch_ptr[device];
  return SVO_OK;
}

}  // namespace
}  // namespace svo

using svo::fail;

extern "C" SVO_API svo_status svo_trace_noalloc(int32_t device, void *stream, uint8_t base_depth,
                                                const uint16_t *bases, size_t n_bases, const svo_block *blocks,
                                                size_t n_blocks, svo_usage *usage, size_t n_groups,
                                                int32_t max_node_depth, const svo_trace_input *input,
                                                const svo_trace_output *out, svo_child_request *requests,
                                                uint32_t request_cap, uint32_t *requests_raised) {
  using namespace svo;
  if (!input || !out || !bases || !blocks) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: null argument");
  if (!out->on_device)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: outputs must be device pointers (on_device = 1)");
  if (base_depth < 1 || base_depth > 8) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: base_depth 1..8");
  uint32_t W = input->screen_size[0], H = input->screen_size[1];
  if (W == 0 || H == 0 || (uint64_t)W + H > kMaxWidthPlusHeight)
    return fail(SVO_ERR_INVALID_ARGUMENT,
                "svo_trace_noalloc: width + height must be 2..16384 (the static scratch holds the ray tables)");
  if ((uint64_t)W * H > 0xF0000000ull) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: too many rays");
  if (input->base_depth != 0 && input->base_depth != base_depth)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: input base_depth differs from the tree's");
  uint32_t pow_sum = 0, p8 = 1;
  for (int i = 1; i <= base_depth; i++) pow_sum += (p8 *= 8);
  if (n_bases != pow_sum) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: need powSum(base_depth) bases");
  if (n_blocks > 0xFFFFFFF8ull) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: too many blocks");
  int depth = max_node_depth > 0 ? max_node_depth : SVO_MAX_TREE_DEPTH;
  if (depth < base_depth + 2 || depth > SVO_MAX_TREE_DEPTH)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_trace_noalloc: max_node_depth must be base_depth+2..SVO_MAX_TREE_DEPTH");

  std::lock_guard<std::mutex> guard(g_lock);
  DeviceRestore restore;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(SVO_ERR_NO_DEVICE, std::string("svo_trace_noalloc: ") + cudaGetErrorString(e));
  unsigned char *scratch = nullptr;
  svo_status st = scratch_address(device, &scratch);
  if (st) return st;
  int sm_count = 0;
  e = cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("svo_trace_noalloc: ") + cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // view record and ray-setup tables (wavefront.cl:563-595), as svo_trace builds them
  ViewParams &v = g_host_view;
  std::memset(&v, 0, sizeof(v));
  for (int k = 0; k < 3; k++) v.origin[k] = input->origin[k];
  for (int k = 0; k < 9; k++) v.facing[k] = input->facing[k];
  v.fov_px = input->fov[0] / (float)W;
  v.dof[0] = input->dof[0];
  v.dof[1] = input->dof[1];
  v.width = W;
  v.height = H;
  v.ray_begin = 0;
  v.pixel_begin = 0;
  v.table_off = 0;
  v.tick = input->tick;
  v.tile = (uint16_t)kTraceTileW;  // warp batches over kTraceTileW x (32 / kTraceTileW) pixel tiles
  v.hit_index = out->hit_index;
  v.hit_depth = out->hit_depth;
  v.t = out->t;
  v.rgba = out->rgba;
  float fw = (float)W, fh = (float)H;
  for (uint32_t x = 0; x < W; x++) {
    float u = input->fov[0] * ((fw / 2.0f - (float)x) / fw);
    g_host_tables[x] = (float)std::sin((double)u);
    g_host_tables[W + x] = (float)std::cos((double)u);
  }
  for (uint32_t y = 0; y < H; y++) {
    float a = input->fov[1] * ((fh / 2.0f - (float)y) / fh);
    g_host_tables[2 * W + y] = (float)std::sin((double)a);
    g_host_tables[2 * W + H + y] = (float)std::cos((double)a);
  }
  // Pageable sources: each copy has consumed the host data when it returns.
  e = cudaMemsetAsync(scratch + kCountersOff, 0, 16 * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(scratch + kViewOff, &v, sizeof(v), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kTablesOff, g_host_tables, sizeof(float) * 2 * ((size_t)W + H),
                        cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("svo_trace_noalloc: staging: ") + cudaGetErrorString(e));

  uint32_t *counters = reinterpret_cast<uint32_t *>(scratch + kCountersOff);
  TraceLaunch a{};
  a.bases = bases;
  a.blocks = blocks;
  a.usage = usage;
  a.requests = requests;
  a.request_cap = requests ? request_cap : 0;
  a.ray_counter = counters;
  a.request_count = counters + 1;
  a.error = counters + 4;
  a.stats = nullptr;
  a.views = reinterpret_cast<const ViewParams *>(scratch + kViewOff);
  a.tables = reinterpret_cast<const float *>(scratch + kTablesOff);
  a.n_bases = (uint32_t)n_bases;
  a.n_blocks = (uint32_t)n_blocks;
  a.n_groups = usage ? (uint32_t)n_groups : 0;
  // ray slots: whole 32-pixel tiles (the padding slots of edge tiles are skipped)
  const uint32_t tile_h = 32u / kTraceTileW;
  a.total_rays = ((W + kTraceTileW - 1) / kTraceTileW) * ((H + tile_h - 1) / tile_h) * 32u;
  a.n_views = 1;
  a.base_depth = base_depth;
  a.max_steps = 1 << 16;
  a.ray_chunk = 1;
  a.cadence = 16;
  a.block_size = 192;  // svo_trace's default block size
  a.schedule = SVO_SCHEDULE_WARP;
  a.path_levels = depth - base_depth - 1;
  int occ = trace_occupancy(a, false);
  if (occ <= 0) return fail(SVO_ERR_NO_DEVICE, "svo_trace_noalloc: the trace kernel cannot be resident");
  // the persistent grid of svo_trace: every resident CTA, or one per 32-slot tile when fewer
  long need = ((long)a.total_rays + 31) / 32 * 32 / a.block_size + 1;
  a.grid = (int)std::max(1L, std::min<long>((long)occ * sm_count, need));
  st = launch_trace(a, false, stream);
  if (st) return st;

  // read back the error record and the request count (host stack, no allocation)
  uint32_t words[10];
  e = cudaMemcpyAsync(words, counters, sizeof(words), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("svo_trace_noalloc: ") + cudaGetErrorString(e));
  if (requests_raised) *requests_raised = words[1];
  if (words[4] == SVO_ERR_TIMEOUT)
    return fail(SVO_ERR_TIMEOUT, "svo_trace_noalloc: a thread exceeded its iteration bound on ray " +
                                     std::to_string(words[7]));
  if (words[4]) return fail((svo_status)words[4], "svo_trace_noalloc: kernel reported an error");
  return SVO_OK;
}
