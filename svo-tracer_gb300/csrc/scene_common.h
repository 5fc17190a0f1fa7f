// Scene arithmetic shared by the host tree builder and the device graft
// generator, so that both produce the same blocks bit for bit: the integer
// hash of the seeded scenes, the terrain's cell classification against its
// column height range, the terrain's colour bands, and CanHaveChildren.
#pragma once

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

// CanHaveChildren (TreeBuilder.cs): some octant holds both air and geometry.
SVO_SCENE_FN bool can_have_children(uint16_t chunk) {
  return ((chunk & (chunk >> 1)) & 0x5555u) != 0;
}

}  // namespace scene
}  // namespace svo
