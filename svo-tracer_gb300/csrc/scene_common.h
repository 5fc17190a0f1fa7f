// Scene arithmetic shared by the host tree builder and the device graft
// generator, so that both produce the same blocks bit for bit: the integer
// hash of the seeded scenes, the terrain's cell classification against its
// column height range, the terrain's colour bands and normals, the normal
// encoding, and CanHaveChildren.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SVO_SCENE_FN __host__ __device__ __forceinline__
#else
#define SVO_SCENE_FN inline
#endif

namespace svo {
namespace scene {

SVO_SCENE_FN uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352dU;
  h ^= h >> 15;
  h *= 0x846ca68bU;
  h ^= h >> 16;
  return h;
}

SVO_SCENE_FN uint32_t hash4(uint32_t seed, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  uint32_t h = mix32(seed ^ 0x9e3779b9U);
  h = mix32(h ^ a);
  h = mix32(h + 0x632be5abU ^ b);
  h = mix32(h + 0x85157af5U ^ c);
  h = mix32(h + 0x2545f491U ^ d);
  return h;
}

// A terrain cell at `level` (column heights quantised to leaf cells, the
// column range of its footprint [mn, mx], up = -z): geometry when its deepest
// voxel row is solid somewhere, air when its top row is open somewhere.
SVO_SCENE_FN void terrain_classify(uint32_t mx, uint32_t mn, uint32_t res, int leaf, int level, uint32_t z,
                                   bool &geo, bool &air) {
  const uint32_t s = 1u << (leaf - level);
  geo = (int64_t)mx > (int64_t)res - (int64_t)(z + 1) * s;
  air = (int64_t)mn < (int64_t)res - (int64_t)z * s;
}

// Terrain colour: a band by height above the bottom face (sand, grass, rock,
// snow) plus a seeded +-8 jitter per channel.
SVO_SCENE_FN void terrain_colour(uint32_t seed, int level, uint32_t x, uint32_t y, uint32_t z, uint8_t rgb[3]) {
  const double zc = (z + 0.5) * (1.0 / (double)(1ull << level));
  const double h = 1.0 - zc;
  int base[3];
  if (h < 0.06) {
    base[0] = 194; base[1] = 178; base[2] = 128;  // sand
  } else if (h < 0.14) {
    base[0] = 86; base[1] = 125; base[2] = 70;    // grass
  } else if (h < 0.22) {
    base[0] = 120; base[1] = 110; base[2] = 100;  // rock
  } else {
    base[0] = 236; base[1] = 236; base[2] = 242;  // snow
  }
  const uint32_t hsh = hash4(seed ^ 0x3c6ef372U, (uint32_t)level, x, y, z);
  for (int k = 0; k < 3; k++) {
    const int j = (int)((hsh >> (8 * k)) % 17u) - 8;
    const int v = base[k] + j;
    rgb[k] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
  }
}

// atan2(y, x) from basic float operations only (two half-angle reductions
// atan t = 2 atan(t / (1 + sqrt(1 + t^2))) to |t| <= tan(pi/16), then the
// Taylor series of atan to t^11), so that the host builder and the device
// generator round every step alike. Single precision: the device's FP64 pipe is
// slow, and the result is truncated to 1/32767 of pi anyway.
SVO_SCENE_FN float atan2_basic(float y, float x) {
  const float pi = 3.14159265358979f;
  if (x == 0.0f && y == 0.0f) return 0.0f;
  const float ax = x < 0.0f ? -x : x, ay = y < 0.0f ? -y : y;
  float t = ay <= ax ? ay / ax : ax / ay;
  for (int i = 0; i < 2; i++) t = t / (1.0f + sqrtf(1.0f + t * t));
  const float t2 = t * t;
  float term = t, sum = t;
  for (int k = 1; k <= 5; k++) {
    term = -term * t2;
    sum = sum + term / (float)(2 * k + 1);
  }
  float a = 4.0f * sum;
  if (ay > ax) a = pi / 2.0f - a;
  if (x < 0.0f) a = pi - a;
  return y < 0.0f ? -a : a;
}

// NormalAngle (TreeBuilder.cs:328-334) of the surface normal n. The
// reference's geometry definitions hand it (n.y, -n.z, n.x)
// (SphereDefinition.Normal), which normalVector (kernel.cl:264-275) decodes
// back to n: pitch = asin(n.z) / pi, yaw = atan2(n.y, n.x) / pi, each times
// 32767 and truncated. A zero vector gives (0, 0).
SVO_SCENE_FN void normal_angles(float nx, float ny, float nz, int16_t &pitch, int16_t &yaw) {
  const float pi = 3.14159265358979f;
  const float l = sqrtf(nx * nx + ny * ny + nz * nz);
  if (!(l > 0.0f)) {
    pitch = yaw = 0;
    return;
  }
  nx = nx / l;
  ny = ny / l;
  nz = nz / l;
  const float c = 1.0f - nz * nz;
  pitch = (int16_t)(32767.0f * (atan2_basic(nz, sqrtf(c > 0.0f ? c : 0.0f)) / pi));
  yaw = (int16_t)(32767.0f * (atan2_basic(ny, nx) / pi));
}

// The terrain's surface normal at column (x, y) of `level` (up = -z), from
// central differences of that level's column maxima (one-sided at the border).
SVO_SCENE_FN void terrain_normal(const uint16_t *hi_level, int level, int leaf, uint32_t x, uint32_t y,
                                 int16_t &pitch, int16_t &yaw) {
  const uint32_t n = 1u << level;
  const uint32_t x0 = x ? x - 1 : x, x1 = x + 1 < n ? x + 1 : x;
  const uint32_t y0 = y ? y - 1 : y, y1 = y + 1 < n ? y + 1 : y;
  const float s = (float)(1u << (leaf - level));  // leaf cells per column side
  const float hx = x1 > x0 ? ((float)hi_level[(size_t)y * n + x1] - (float)hi_level[(size_t)y * n + x0]) /
                                 ((float)(x1 - x0) * s)
                           : 0.0f;
  const float hy = y1 > y0 ? ((float)hi_level[(size_t)y1 * n + x] - (float)hi_level[(size_t)y0 * n + x]) /
                                 ((float)(y1 - y0) * s)
                           : 0.0f;
  normal_angles(-hx, -hy, -1.0f, pitch, yaw);
}

// CanHaveChildren (TreeBuilder.cs): some octant holds both air and geometry.
SVO_SCENE_FN bool can_have_children(uint16_t chunk) {
  return ((chunk & (chunk >> 1)) & 0x5555u) != 0;
}

}  // namespace scene
}  // namespace svo
