// Internal declarations of the megakernel path (kernel.cl's `trace`), shared by
// mega_kernels.cu and the C ABI in svo_api.cu.
#pragma once

#include <cuda_runtime.h>

#include "svo_internal.h"

namespace svo {

// Per pixel slot (the view's warp tiles, 32 slots per tile) between the kernels.
enum : uint8_t { kMegaPad = 0, kMegaMiss = 1, kMegaSky = 2, kMegaSurface = 3 };
struct MegaPixel {
  uint64_t loc[3];   // primary's end location; after the fan kernel, the cones' start
  float origin[3];   // cones' Origin: ulongToFloat of the primary's end location
  float dir[3];      // primary direction
  uint32_t node;     // surface block, SVO_MISS for the sky
  uint32_t id;       // pixel index in the view
  uint16_t n_cones;  // cones of this pixel's fan
  uint8_t kind;      // kMega*
  uint8_t depth;     // RayData.Depth: the surface's level, 1 for the sky
  uint32_t _pad;
};
static_assert(sizeof(MegaPixel) == 64, "MegaPixel layout");

// spawnRays's per-launch constants (kernel.cl:1115-1253): one spine step of the
// fan (its cones' FoV and weighting, cos/sin(-spineAngle), 1 - cos) and its
// ring rotations (cos/sin(-ringAngle), 1 - cos).
struct MegaSpine {
  float fov, weighting, c, s, k;
  uint32_t ring_begin, n_rings, _pad;
};
struct MegaRing {
  float c, s, k, _pad;
};

struct MegaLaunch {
  TraceLaunch t;            // tree, queue, view and table of the primary cones
  MegaPixel *pix;           // per slot of the view
  float4 *cone_dw;          // per cone slot of the band: direction, weighting
  uint16_t *cone_s;         // per cone slot: spine step + 1 (0: the reflection cone)
  uint8_t *cone_sky;        // per cone slot: 1 when the cone reached the sky
  uint32_t *tile_cones;     // per tile of the band: its cones, then (scanned) its first entry
  uint32_t *entries;        // the band's cones compacted: cone slots by tile, cone k, lane
  uint32_t *queue;          // [0] entry queue head of the cone kernel, [1] entries of the band
  const float2 *normal_sc;  // normalVector's (sin, cos) of each int16 angle, index angle + 32768
  const MegaSpine *spine;
  const MegaRing *ring;
  unsigned long long *totals;   // [0] cones of the fans, [1] primary surfaces
  int32_t n_spines;
  int32_t k_max;                // cones per pixel at most: the cone slot stride
  float fov_c, weighting_c;     // FovConstant, WeightingConstant: the reflection cone's
  uint32_t band_tile0, band_tiles;  // tiles [band_tile0, band_tile0 + band_tiles)
  uint32_t max_entries;         // cone slots of a band (bounds the entry count)
  int32_t grid_cones;           // persistent grid of the cone kernel
  int32_t cone_schedule;        // SVO_SCHEDULE_WARP: 32 entries per warp claim; LANE: lanes refill
};

// The wavefront's secondary-cone stage as the reference wires it (see
// gi_kernels.cu), over every pixel of a traced batch.
struct GiLaunch {
  const ViewParams *views;  // device view table of the trace (hit_index set for every view)
  const float *tables;      // the trace's ray-setup tables
  const uint4 *blocks;
  svo_usage *usage;
  const float2 *normal_sc;
  const MegaSpine *spine;
  const MegaRing *ring;
  uint32_t n_blocks, n_groups, total_pixels;
  int32_t n_views, n_spines;
  float fov_c, weighting_c;   // FovConstant, WeightingConstant of every view
  uint32_t ambient;           // AmbientLightLevel of every view
  int32_t valid;              // 0: evaluateMaterial returns at once (FovConstant <= 0 or |FovMultiplier| >= 1)
};
svo_status launch_gi(const GiLaunch &g, void *stream);
// spawnRays's spine and ring constants for an input (cached in the context by
// its cone parameters); returns the cones per pixel of a fan without a break
// (0 when that exceeds SVO_MEGA_MAX_CONES: the reference's loops would not end).
struct Context;
int32_t ensure_cone_schedule(Context &c, const svo_trace_input &in, svo_status &st);
svo_status ensure_normal_table(Context &c);

svo_status launch_mega_primary(const MegaLaunch &m, void *stream);
svo_status launch_mega_band(const MegaLaunch &m, void *stream);
int mega_occupancy(const MegaLaunch &m);

}  // namespace svo
