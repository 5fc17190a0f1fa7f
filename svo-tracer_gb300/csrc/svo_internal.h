// Internal declarations shared by the libsvo translation units.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/svo.h"

namespace svo {

// Records the message returned by svo_last_error_string and returns `status`.
svo_status fail(svo_status status, const std::string &message);

struct TreeHost;

// Pixel tile of a warp batch: tile_w x (32 / tile_w) pixels, tile_w a power of
// two; results do not depend on it. Measured on GB300: 4x8 tiles for the trace
// and the megakernel (1080p frame 1.80 -> 1.78 ms, megakernel 18.39 -> 17.73 ms
// against 8x4), but 8x4 for a trace whose kernel writes pinned host outputs
// directly (its stores leave the GPU in row segments of the tile width: e2e 1041
// Mrays/s with 4x8 against 1100 with 8x4), and 8x4 for the colour-fitting kernels
// (2.21 / 2.43 ms against 2.24 / 2.46 ms with 4x8).
#ifndef SVO_TRACE_TILE_W
#define SVO_TRACE_TILE_W 4
#endif
#ifndef SVO_TRACE_HOST_TILE_W
#define SVO_TRACE_HOST_TILE_W 8
#endif
#ifndef SVO_DIFF_TILE_W
#define SVO_DIFF_TILE_W 8
#endif
// The outputs of pinned host buffers that a trace stages in device memory and
// copies after the kernel instead of writing them from the kernel (bit 0 hit
// index, 1 hit depth, 2 t, 3 RGBA).
#ifndef SVO_STAGED_HOST_OUTPUTS
#define SVO_STAGED_HOST_OUTPUTS 2
#endif
constexpr uint32_t kTraceTileW = SVO_TRACE_TILE_W, kTraceHostTileW = SVO_TRACE_HOST_TILE_W,
                   kDiffTileW = SVO_DIFF_TILE_W, kStagedHostOutputs = SVO_STAGED_HOST_OUTPUTS;
static_assert((kTraceTileW & (kTraceTileW - 1)) == 0 && kTraceTileW <= 32, "tile width: a power of two up to 32");
static_assert((kDiffTileW & (kDiffTileW - 1)) == 0 && kDiffTileW <= 32, "tile width: a power of two up to 32");
static_assert((kTraceHostTileW & (kTraceHostTileW - 1)) == 0 && kTraceHostTileW <= 32, "tile width");

// The device counter words of a trace launch: [0] ray queue head, [1] child
// requests raised, [2..3] spare, [4 .. 4 + kErrorWords) the kernel error record
// ([0] status, then block, thread, ray, depth and steps of the first thread that
// stopped), the rest spare.
constexpr int kCounterWords = 12;
constexpr int kErrorOffset = 4;
constexpr int kErrorWords = 6;
static_assert(kErrorOffset + kErrorWords <= kCounterWords, "the counter area holds the error record");

// Per-view constants of one trace, as the kernel reads them.

struct ViewParams {
  float origin[3];
  float facing[9];
  float fov_px;       // FoV[0] / ScreenSize.x (the pixel cone factor)
  float dof[2];
  uint32_t width;
  uint32_t height;
  uint32_t ray_begin;  // first ray of this view in the batch's ray index space
  uint32_t table_off;  // sinU, cosU at [off, off+W); sinV, cosV at [off+2W, off+2W+2H)
  uint16_t tick;
  uint16_t tile;         // tile width: rays are claimed in tile x (32 / tile) pixel tiles (slots padded to whole tiles); 0: rows
  uint32_t pixel_begin;  // first pixel of this view in the batch's concatenated pixel space
  uint32_t *hit_index;
  uint8_t *hit_depth;
  float *t;
  float *rgba;
};
static_assert(sizeof(ViewParams) % 8 == 0, "ViewParams alignment");

// A child request staged by its pixel (the pixel-order rule): one aligned
// 32-byte sector, written with a streaming store; the queue's 40-byte
// svo_child_request is rebuilt from it (Tick 0, as the wavefront's requests).
struct alignas(32) StagedRequest {
  uint64_t location[3];
  uint32_t address;
  uint8_t depth;
  uint8_t tree_size;
  uint16_t _pad;
};
static_assert(sizeof(StagedRequest) == 32, "one sector per staged request");

struct TraceLaunch {
  const uint16_t *bases;
  const void *blocks;  // svo_block[n_blocks]
  svo_usage *usage;
  svo_child_request *requests;
  uint32_t *request_count;
  uint32_t *ray_counter;
  uint32_t *error;            // kErrorWords: [0] status, [1..5] block, thread, ray, depth, steps of a stopped thread
  unsigned long long *stats;  // 7 counters in svo_trace_stats order, or null
  uint32_t *ray_v_block;      // per-ray V_block (stats launches only), or null
  uint32_t *ray_v_base;
  const ViewParams *views;    // device array
  const float *tables;        // device trig tables
  uint32_t n_bases;
  uint32_t n_blocks;
  uint32_t n_groups;
  uint32_t request_cap;
  uint32_t total_rays;
  int32_t n_views;
  int32_t base_depth;
  int32_t max_steps;
  uint32_t ray_chunk;
  int32_t cadence;
  int32_t block_size;
  int32_t schedule;  // SVO_SCHEDULE_LANE / SVO_SCHEDULE_WARP
  int32_t grid;
  int32_t path_levels;
  // per-ray pass bound of the device loops; 0: max_steps + 2 (a step ends a ray
  // after max_steps steps, so only a fault can reach it). Lower values make the
  // kernels stop with SVO_ERR_TIMEOUT, which tests that path.
  uint32_t pass_limit;
  // SVO_REQUESTS_PIXEL: a ray's child request goes to req_stage[pixel] with
  // req_flag[pixel] = 1 (pixel in the batch's pixel space; the flags are
  // cleared before the launch), and launch_request_compaction builds the queue
  // afterwards. Null: requests are queued in arrival order.
  struct StagedRequest *req_stage;
  uint8_t *req_flag;
  // L2 persisting access-policy window of the launch (host side only; 0 bytes: none)
  const void *l2_base;
  size_t l2_bytes;
};

// Launches the persistent trace kernel on `stream`.
svo_status launch_trace(const TraceLaunch &a, bool with_stats, void *stream);
// The child-request queue of the pixel-order rule from a launch's staged
// requests: a.request_count = requests raised, a.requests[0 .. min(raised,
// request_cap)) = the staged records of the lowest pixels, in pixel order.
// total_pixels flags are read (the flag array is padded with zeros to whole
// chunks of kRequestChunk); chunk_offsets holds one word per chunk.
constexpr uint32_t kRequestChunk = 4096;
svo_status launch_request_compaction(const TraceLaunch &a, uint32_t total_pixels, uint32_t *chunk_offsets,
                                     void *stream);
// Dynamic shared memory the launch needs.
size_t trace_smem_bytes(const TraceLaunch &a, bool bases_in_smem);
int trace_occupancy(const TraceLaunch &a, bool with_stats);

// A terrain scene's column height pyramids, for generating graft payloads on
// the device (tree_builder.cpp holds the scene).
constexpr int kMaxTerrainLevels = 18;
struct TerrainInfo {
  uint64_t id;  // unique per scene object of this process
  int base_depth, scene_depth, leaf;
  uint32_t res, seed;
  const uint16_t *lo[kMaxTerrainLevels], *hi[kMaxTerrainLevels];  // level l: 4^l columns, min / max height
};
// False when `scene` (an svo_scene_create handle) is not a terrain scene.
bool scene_terrain_info(const void *scene, TerrainInfo *out);

}  // namespace svo
