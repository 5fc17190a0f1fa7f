// The wavefront's secondary-cone (material) stage, as the reference wires it.
//
// MainWindow.RunWavefront (SvoTracer.Window/MainWindow.cs:390-402) has the stage
// commented out: evaluateMaterial over the material queue (the primary hits),
// RunTraces, then evaluateBackground. Enabled as written, it behaves as follows:
//  * evaluateMaterial (wavefront.cl:1568-1739) stamps the hit block's usage and
//    builds the cone fan of the hit (the reflection cone, spine seeds, ring
//    pairs; the same fan as kernel.cl's spawnRays). A hit whose base weighting
//    times WeightingConstant is below 6 only sets FinalWeightings to 255; a hit
//    seen edge-on (dot(direction, normal) >= 0) gets one cone along the primary
//    direction with weighting 255. Cone weightings are (uchar)(ringWeighting *
//    255).
//  * saveAccumulator (:338-355) puts every cone of weighting > 5 straight on
//    the background queue, so no cone is traced through the octree, and the
//    RunTraces that follows finds its queues empty.
//  * evaluateBackground (:1741-1797) adds each such cone's sky light to its
//    pixel: the sky colour and luminosity of the cone's direction, blended with
//    the hit block's colour by the ambient light level (weighting < 255), times
//    the weighting.
//  * EvaluateMaterial's host call resets the material queue before the kernel
//    runs, so resolveRemainders adds nothing: a hit pixel's colour is its cones'
//    sky light only; with unusable cone parameters (the kernel returns at once)
//    its weighting stays 0 and drawTrace paints it red.
// Sky pixels keep the first evaluateBackground's colour (the trace wrote it).
// Here one thread per pixel evaluates its cones in registers after the trace:
// the reference's per-pixel atomic sums are integer sums, so their order does
// not matter. Out-of-range float-to-uchar conversions (undefined in C) saturate.
#include <cuda_runtime.h>

#include <string>

#include "trace_core.cuh"
#include "fan.cuh"

namespace svo {
namespace {

__device__ __forceinline__ uint32_t sat_u8(float x) { return min(__float2uint_rz(x), 255u); }

__global__ void __launch_bounds__(256) gi_kernel(const GiLaunch g) {
  const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
  if (pixel >= g.total_pixels) return;
  int lo = 0, hi = g.n_views - 1;  // the view of this pixel (views in pixel order)
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.views[mid].pixel_begin <= pixel)
      lo = mid;
    else
      hi = mid - 1;
  }
  const ViewParams &v = g.views[lo];
  const uint32_t id = pixel - v.pixel_begin;
  const uint32_t hit = v.hit_index[id];
  if (hit == SVO_MISS) return;  // background pixels keep the trace's colour
  uint32_t fw = 0, fr = 0, fg = 0, fb = 0;  // FinalWeightings, FinalColourRs/Gs/Bs
  if (g.valid) {
    // updateUsage of the hit block's group (wavefront.cl:1607)
    const uint32_t group = hit >> 3;
    if (g.usage && group < g.n_groups) {
      uint16_t *tick = reinterpret_cast<uint16_t *>(g.usage + group);
      const uint16_t cur = *tick;
      if (cur < 65534 && cur != v.tick) *tick = v.tick;
    }
    const uint4 nd = load_node(g.blocks, g.n_blocks, hit);
    const uint32_t base[3] = {(nd.z >> 16) & 0xffu, nd.z >> 24, nd.w & 0xffu};
    float n[3];
    block_normal(g.normal_sc, nd, n);
    float dx, dy, dz;
    ray_direction(v, g.tables, id % v.width, id / v.width, dx, dy, dz);
    // saveAccumulator + evaluateBackground of one cone
    auto cone = [&](float x, float y, float z, uint32_t w) {
      if (w <= 5) return;  // not queued
      const float dotp = dot3(x, y, z, 0.0f, 0.0f, -1.0f);
      uint32_t c[3], lum;
      if (dotp > 0.8f) {
        c[0] = c[1] = c[2] = 255;
        lum = sat_u8(__fmul_rn(dotp, 200.0f));
      } else {
        c[0] = 135;
        c[1] = 206;
        c[2] = 235;
        lum = 1;
      }
      if (w < 255) {
        const uint32_t boundary = lum > g.ambient ? 255u : 0u;
        const float q = __fdiv_rn(__uint2float_rn(lum > g.ambient ? lum - g.ambient : g.ambient - lum),
                                  __fmul_rn(__uint2float_rn(lum + g.ambient), 255.0f));
#pragma unroll
        for (int k = 0; k < 3; k++)
          c[k] = sat_u8(__fadd_rn(__uint2float_rn(base[k]),
                                  __fmul_rn(__fmul_rn(q, __uint2float_rn(c[k])), __uint2float_rn(boundary - base[k]))));
      }
      fw += w;
      if (lum > 0) {
        fr += c[0] * w;
        fg += c[1] * w;
        fb += c[2] * w;
      }
    };
    if (__fmul_rn(g.weighting_c, 255.0f) < 6.0f) {
      fw = 255;  // FinalWeightings[traceID] = baseWeighting
    } else if (dot3(dx, dy, dz, n[0], n[1], n[2]) >= 0.0f) {
      cone(dx, dy, dz, 255);
    } else {
      spawn_fan(n, dx, dy, dz, g.fov_c, g.weighting_c, g.spine, g.n_spines, g.ring,
                [&](float x, float y, float z, float rw, int) { cone(x, y, z, sat_u8(__fmul_rn(rw, 255.0f))); });
    }
  }
  // drawTrace (wavefront.cl:1835-1850)
  if (v.rgba) {
    float4 px;
    if (fw == 0) {
      px = make_float4(0.75f, 0.0f, 0.0f, 1.0f);
    } else {
      const float d = __fmul_rn(__uint2float_rn(fw), 255.0f);
      px.x = fminf(__fdiv_rn(__uint2float_rn(fr), d), 1.0f);
      px.y = fminf(__fdiv_rn(__uint2float_rn(fg), d), 1.0f);
      px.z = fminf(__fdiv_rn(__uint2float_rn(fb), d), 1.0f);
      px.w = 1.0f;
    }
    reinterpret_cast<float4 *>(v.rgba)[id] = px;
  }
}

}  // namespace

svo_status launch_gi(const GiLaunch &g, void *stream) {
  if (!g.total_pixels) return SVO_OK;
  gi_kernel<<<(g.total_pixels + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("material stage launch: ") + cudaGetErrorString(e));
  return SVO_OK;
}

}  // namespace svo
