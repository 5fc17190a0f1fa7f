// The secondary-cone fan of a surface hit, shared by the megakernel
// (kernel.cl's spawnRays, kernel.cl:1115-1217) and the wavefront's material
// stage (evaluateMaterial, wavefront.cl:1568-1739): the reflection cone, then
// per spine step a seed cone rotated about the axis D x N, and per ring step a
// pair of cones rotated about the reflection, each stopping at the first cone
// below the surface. The spine and ring constants (MegaSpine, MegaRing) depend
// only on the input's cone parameters and are computed on the host. Every
// operation is one IEEE round-to-nearest float operation in the reference's
// order, so the directions and weightings are bit-exact.
#pragma once

#include <cuda_runtime.h>

#include "mega_internal.h"

namespace svo {
namespace {

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// normalize (OpenCL C): v / sqrt(x*x + y*y + z*z); a zero vector stays zero.
__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
  if (x == 0.0f && y == 0.0f && z == 0.0f) return;
  const float l = __fsqrt_rn(dot3(x, y, z, x, y, z));
  x = __fdiv_rn(x, l);
  y = __fdiv_rn(y, l);
  z = __fdiv_rn(z, l);
}

// Rotation of v about the unit axis a (cos c, sin s, k = 1 - c) in the
// reference's product order (spineRotation / ringRotation); `transpose` rotates
// by the opposite angle (the second vector of a ring pair).
__device__ __forceinline__ void rotate3(float ax, float ay, float az, float c, float s, float k, float vx, float vy,
                                        float vz, bool transpose, float &ox, float &oy, float &oz) {
  const float r3 = __fmul_rn(__fmul_rn(k, ax), ax), r4 = __fmul_rn(__fmul_rn(k, ax), ay);
  const float r5 = __fmul_rn(__fmul_rn(k, ax), az), r6 = __fmul_rn(__fmul_rn(k, ay), ay);
  const float r7 = __fmul_rn(__fmul_rn(k, ay), az), r8 = __fmul_rn(__fmul_rn(k, az), az);
  const float r9 = __fmul_rn(s, ax), r10 = __fmul_rn(s, ay), r11 = __fmul_rn(s, az);
  const float sg = transpose ? -1.0f : 1.0f;  // exact: flips the sign of the sine terms
  const float q9 = __fmul_rn(sg, r9), q10 = __fmul_rn(sg, r10), q11 = __fmul_rn(sg, r11);
  ox = __fadd_rn(__fadd_rn(__fmul_rn(__fadd_rn(r3, c), vx), __fmul_rn(__fsub_rn(r4, q11), vy)),
                 __fmul_rn(__fadd_rn(r5, q10), vz));
  oy = __fadd_rn(__fadd_rn(__fmul_rn(__fadd_rn(r4, q11), vx), __fmul_rn(__fadd_rn(r6, c), vy)),
                 __fmul_rn(__fsub_rn(r7, q9), vz));
  oz = __fadd_rn(__fadd_rn(__fmul_rn(__fsub_rn(r5, q10), vx), __fmul_rn(__fadd_rn(r7, q9), vy)),
                 __fmul_rn(__fadd_rn(r8, c), vz));
}

// normalVector (kernel.cl:264-275, wavefront.cl:235-246) of a block's
// NormalPitch / NormalYaw: sin/cos of angle * pi / 32767 come from a table of
// (sin, cos) per int16 angle (index angle + 32768).
__device__ __forceinline__ void block_normal(const float2 *normal_sc, uint4 node, float n[3]) {
  const int16_t pitch = (int16_t)(node.y >> 16), yaw = (int16_t)(node.z & 0xffffu);
  const float2 sp = __ldg(normal_sc + (pitch + 32768)), sy = __ldg(normal_sc + (yaw + 32768));
  n[0] = __fmul_rn(sy.y, sp.y);
  n[1] = __fmul_rn(sy.x, sp.y);
  n[2] = sp.x;
}

// The fan of a hit with normal n seen along D: emit(x, y, z, ringWeighting,
// spine) for each cone in generation order (spine 0: the reflection cone,
// s + 1: the cones of spine step s). ringWeighting is the reference's float
// before its multiplication by the parent's weighting.
template <class Emit>
__device__ __forceinline__ void spawn_fan(const float n[3], float Dx, float Dy, float Dz, float fov_c, float weighting_c,
                                          const MegaSpine *spine, int n_spines, const MegaRing *ring, Emit &&emit) {
  float axx = __fsub_rn(__fmul_rn(Dy, n[2]), __fmul_rn(Dz, n[1]));
  float axy = __fsub_rn(__fmul_rn(Dz, n[0]), __fmul_rn(Dx, n[2]));
  float axz = __fsub_rn(__fmul_rn(Dx, n[1]), __fmul_rn(Dy, n[0]));
  normalize3(axx, axy, axz);
  const float d2 = __fmul_rn(2.0f, dot3(Dx, Dy, Dz, n[0], n[1], n[2]));
  const float rx = __fsub_rn(Dx, __fmul_rn(d2, n[0]));
  const float ry = __fsub_rn(Dy, __fmul_rn(d2, n[1]));
  const float rz = __fsub_rn(Dz, __fmul_rn(d2, n[2]));
  float fov = fov_c, weighting = weighting_c, rw = weighting;
  float dp = dot3(rx, ry, rz, n[0], n[1], n[2]);
  if (dp < fov) rw = __fdiv_rn(__fmul_rn(weighting, dp), fov);
  emit(rx, ry, rz, rw, 0);
  for (int s = 0; s < n_spines; s++) {
    const MegaSpine sp = spine[s];
    fov = sp.fov;
    weighting = sp.weighting;
    rw = weighting;
    float sx, sy, sz;
    rotate3(axx, axy, axz, sp.c, sp.s, sp.k, rx, ry, rz, false, sx, sy, sz);
    normalize3(sx, sy, sz);
    dp = dot3(sx, sy, sz, n[0], n[1], n[2]);
    if (dp < 0.0f) break;
    if (dp < fov) rw = __fdiv_rn(__fmul_rn(weighting, dp), fov);
    emit(sx, sy, sz, rw, s + 1);
    for (uint32_t j = 0; j < sp.n_rings; j++) {
      const MegaRing rg = ring[sp.ring_begin + j];
      rw = weighting;
      float vx, vy, vz;
      rotate3(rx, ry, rz, rg.c, rg.s, rg.k, sx, sy, sz, false, vx, vy, vz);
      normalize3(vx, vy, vz);
      dp = dot3(vx, vy, vz, n[0], n[1], n[2]);
      if (dp < 0.0f) break;
      if (dp < fov) rw = __fdiv_rn(__fmul_rn(weighting, dp), fov);
      emit(vx, vy, vz, rw, s + 1);
      rotate3(rx, ry, rz, rg.c, rg.s, rg.k, sx, sy, sz, true, vx, vy, vz);
      normalize3(vx, vy, vz);
      emit(vx, vy, vz, rw, s + 1);
    }
  }
}

}  // namespace
}  // namespace svo
