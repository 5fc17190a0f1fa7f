// Procedural scenes and the octree builder (host side of libsvo).
//
// The builder produces the reference's device format (SvoTracer.Domain/
// TreeBuilder.cs:102-284): dense ushort base chunks for levels 1..B, a dense
// level B+2 of 16-byte nodes at baseLocation, and deeper levels as 8-node
// groups. Node addresses follow TreeBuilder's allocation order exactly:
//   * level B+2 nodes sit at (level-(B+1) cell index << 3) + octant and exist
//     only under level-(B+1) cells whose base chunk pair is air+geometry;
//   * groups are taken from a queue that holds the sorted unused level-(B+1)
//     slots first, then 8^(B+1), 8^(B+1)+1, ... (TreeBuilder.cs:113-118);
//   * level B+2 nodes are visited x-major, then y, then z (TreeBuilder.cs:
//     123-141), and each subtree is filled depth-first, a group being taken the
//     moment a node turns out to need children (BuildBlocks, :237-256).
// That order is sequential by nature; this builder gets the same addresses in
// parallel by building each level-(B+2) subtree with local group numbers on
// its own thread, prefix-summing the group counts in visiting order and then
// mapping local group j of subtree k to queue entry offset_k + j.
//
// Geometry is the seeded scene of the workload, not the reference's analytic
// spheres/cubes: a displaced SDF sphere or an fBm heightfield terrain. Cells
// are classified exactly with respect to a leaf grid one level below the
// deepest node level (a node's chunk describes its 8 children).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/svo.h"
#include "scene_common.h"
#include "svo_internal.h"

namespace svo {
namespace {

using scene::hash4;

inline double unit_hash(uint32_t h) { return (h >> 8) * (1.0 / 16777216.0); }

inline double quintic(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }

uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t out = 0;
  for (int i = 0; i < 11; i++) {
    out |= ((x >> i) & 1u) << (3 * i);
    out |= ((y >> i) & 1u) << (3 * i + 1);
    out |= ((z >> i) & 1u) << (3 * i + 2);
  }
  return out;
}

uint32_t pow_sum(int depth) {
  uint32_t s = 0, p = 1;
  for (int i = 1; i <= depth; i++) {
    p *= 8;
    s += p;
  }
  return s;
}

// Cell classification at `level` (coords in [0, 2^level)) against the leaf
// grid at level `leaf`: geo = some leaf cell inside is solid, air = some is not.
struct Scene {
  int leaf = 0;
  uint32_t seed = 0;
  virtual ~Scene() = default;
  virtual void classify(int level, uint32_t cx, uint32_t cy, uint32_t cz, bool &geo, bool &air) const = 0;
  virtual void colour(int level, uint32_t cx, uint32_t cy, uint32_t cz, uint8_t rgb[3]) const = 0;
  // GetNormal (TreeBuilder.cs:46-55): the encoded surface normal of a cell
  virtual void normal(int level, uint32_t cx, uint32_t cy, uint32_t cz, int16_t &pitch, int16_t &yaw) const = 0;
};

// Sphere of radius 0.2 (0.4 of the [-1,1] world) at the cube centre, displaced
// by 3 octaves of seeded value noise of amplitude 0.025 (0.05 world). A leaf
// cell is solid when the displaced SDF at its centre is <= 0. Coarser cells
// use a Lipschitz bound of the SDF to decide whole cells at once.
struct SphereScene final : Scene {
  double cx = 0.5, cy = 0.5, cz = 0.5, radius = 0.2, amp = 0.025, f0 = 4.0;
  double lip = 0.0;
  SphereScene(uint32_t s, int leaf_level) {
    seed = s;
    leaf = leaf_level;
    // |grad n| <= sqrt(3) * 1.875 * sum_o (2 a_o / sum a) f_o for value noise
    // in [-1,1] with quintic fade (max slope 1.875).
    double sum_a = 1.0 + 0.5 + 0.25, g = 0.0, f = f0, a = 1.0;
    for (int o = 0; o < 3; o++, f *= 2.0, a *= 0.5) g += 2.0 * a / sum_a * 1.875 * f;
    lip = (1.0 + amp * std::sqrt(3.0) * g) * 1.01;
  }
  double noise3(double x, double y, double z, uint32_t oct) const {
    double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int32_t ix = (int32_t)fx, iy = (int32_t)fy, iz = (int32_t)fz;
    double tx = quintic(x - fx), ty = quintic(y - fy), tz = quintic(z - fz);
    double v[8];
    for (int k = 0; k < 8; k++)
      v[k] = unit_hash(hash4(seed, oct, (uint32_t)(ix + (k & 1)), (uint32_t)(iy + ((k >> 1) & 1)),
                             (uint32_t)(iz + ((k >> 2) & 1))));
    double x00 = v[0] + (v[1] - v[0]) * tx, x10 = v[2] + (v[3] - v[2]) * tx;
    double x01 = v[4] + (v[5] - v[4]) * tx, x11 = v[6] + (v[7] - v[6]) * tx;
    double y0 = x00 + (x10 - x00) * ty, y1 = x01 + (x11 - x01) * ty;
    return y0 + (y1 - y0) * tz;
  }
  double sdf(double x, double y, double z) const {
    double n = 0.0, f = f0, a = 1.0, sum_a = 1.75;
    for (uint32_t o = 0; o < 3; o++, f *= 2.0, a *= 0.5) n += a * (2.0 * noise3(x * f, y * f, z * f, o) - 1.0);
    n /= sum_a;
    double dx = x - cx, dy = y - cy, dz = z - cz;
    return std::sqrt(dx * dx + dy * dy + dz * dz) - radius - amp * n;
  }
  void classify(int level, uint32_t x, uint32_t y, uint32_t z, bool &geo, bool &air) const override {
    geo = air = false;
    classify_rec(level, x, y, z, geo, air);
  }
  void classify_rec(int level, uint32_t x, uint32_t y, uint32_t z, bool &geo, bool &air) const {
    double s = std::ldexp(1.0, -level);
    double f = sdf((x + 0.5) * s, (y + 0.5) * s, (z + 0.5) * s);
    if (level >= leaf) {
      if (f <= 0.0)
        geo = true;
      else
        air = true;
      return;
    }
    double r = std::sqrt(3.0) * (0.5 * s - std::ldexp(0.5, -leaf));
    if (f < -lip * r) {
      geo = true;
      return;
    }
    if (f > lip * r) {
      air = true;
      return;
    }
    for (int k = 0; k < 8 && !(geo && air); k++)
      classify_rec(level + 1, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + ((k >> 2) & 1), geo, air);
  }
  // radial, like SphereDefinition.Normal
  void normal(int level, uint32_t x, uint32_t y, uint32_t z, int16_t &pitch, int16_t &yaw) const override {
    const double s = std::ldexp(1.0, -level);
    scene::normal_angles((float)((x + 0.5) * s - cx), (float)((y + 0.5) * s - cy), (float)((z + 0.5) * s - cz), pitch,
                         yaw);
  }
  void colour(int level, uint32_t x, uint32_t y, uint32_t z, uint8_t rgb[3]) const override {
    uint32_t h = hash4(seed ^ 0x51ed270bU, (uint32_t)level, x, y, z);
    rgb[0] = (uint8_t)(h & 0xff);
    rgb[1] = (uint8_t)((h >> 8) & 0xff);
    rgb[2] = (uint8_t)((h >> 16) & 0xff);
  }
};

// fBm heightfield: 6 octaves of seeded 2-D value noise, lacunarity 2, gain
// 0.5, heights 0..0.3 of the domain. Up is -z (the reference's sky is lit
// from -z, wavefront.cl:1756), so a column of height h is solid for
// z >= 1 - h. Heights are quantised to whole leaf cells; min/max pyramids
// over the columns make cell classification O(1).
struct TerrainScene final : Scene {
  uint32_t res = 0;  // 2^leaf columns per axis
  double f0 = 18.0, hmax = 0.3;
  std::vector<std::vector<uint16_t>> lo, hi;  // per level l: 4^l entries
  TerrainScene(uint32_t s, int leaf_level, int threads) {
    seed = s;
    leaf = leaf_level;
    res = 1u << leaf;
    lo.resize(leaf + 1);
    hi.resize(leaf + 1);
    lo[leaf].resize((size_t)res * res);
    hi[leaf].resize((size_t)res * res);
    parallel_for(threads, res, [&](uint32_t j) {
      for (uint32_t i = 0; i < res; i++) {
        double h = height((i + 0.5) / res, (j + 0.5) / res);
        uint32_t H = (uint32_t)std::floor(h * res + 0.5);
        if (H > res) H = res;
        lo[leaf][(size_t)j * res + i] = (uint16_t)H;
        hi[leaf][(size_t)j * res + i] = (uint16_t)H;
      }
    });
    for (int l = leaf - 1; l >= 0; l--) {
      uint32_t n = 1u << l;
      lo[l].resize((size_t)n * n);
      hi[l].resize((size_t)n * n);
      const auto &clo = lo[l + 1], &chi = hi[l + 1];
      parallel_for(threads, n, [&, n, l](uint32_t j) {
        for (uint32_t i = 0; i < n; i++) {
          size_t a = (size_t)(2 * j) * (2 * n) + 2 * i, b = a + 2 * n;
          lo[l][(size_t)j * n + i] = std::min(std::min(clo[a], clo[a + 1]), std::min(clo[b], clo[b + 1]));
          hi[l][(size_t)j * n + i] = std::max(std::max(chi[a], chi[a + 1]), std::max(chi[b], chi[b + 1]));
        }
      });
    }
  }
  template <class F>
  static void parallel_for(int threads, uint32_t n, F f) {
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
      for (;;) {
        uint32_t j = next.fetch_add(1);
        if (j >= n) break;
        f(j);
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
  }
  double noise2(double x, double y, uint32_t oct) const {
    double fx = std::floor(x), fy = std::floor(y);
    int32_t ix = (int32_t)fx, iy = (int32_t)fy;
    double tx = quintic(x - fx), ty = quintic(y - fy);
    double v00 = unit_hash(hash4(seed, oct, (uint32_t)ix, (uint32_t)iy, 7));
    double v10 = unit_hash(hash4(seed, oct, (uint32_t)(ix + 1), (uint32_t)iy, 7));
    double v01 = unit_hash(hash4(seed, oct, (uint32_t)ix, (uint32_t)(iy + 1), 7));
    double v11 = unit_hash(hash4(seed, oct, (uint32_t)(ix + 1), (uint32_t)(iy + 1), 7));
    double a = v00 + (v10 - v00) * tx, b = v01 + (v11 - v01) * tx;
    return a + (b - a) * ty;
  }
  double height(double x, double y) const {
    double n = 0.0, f = f0, a = 1.0, sum_a = 0.0;
    for (uint32_t o = 0; o < 6; o++, f *= 2.0, a *= 0.5) {
      n += a * noise2(x * f, y * f, o);
      sum_a += a;
    }
    return hmax * (n / sum_a);
  }
  void classify(int level, uint32_t x, uint32_t y, uint32_t z, bool &geo, bool &air) const override {
    size_t idx = (size_t)y * (1u << level) + x;
    scene::terrain_classify(hi[level][idx], lo[level][idx], res, leaf, level, z, geo, air);
  }
  void colour(int level, uint32_t x, uint32_t y, uint32_t z, uint8_t rgb[3]) const override {
    scene::terrain_colour(seed, level, x, y, z, rgb);
  }
  void normal(int level, uint32_t x, uint32_t y, uint32_t, int16_t &pitch, int16_t &yaw) const override {
    scene::terrain_normal(hi[level].data(), level, leaf, x, y, pitch, yaw);
  }
};

using scene::can_have_children;

// MakeChunk (TreeBuilder.cs:264-284) for the cell (x,y,z) at `level`.
uint16_t make_chunk(const Scene &sc, int level, uint32_t x, uint32_t y, uint32_t z) {
  uint16_t chunk = 0;
  for (int k = 0; k < 8; k++) {
    bool geo, air;
    sc.classify(level + 1, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + ((k >> 2) & 1), geo, air);
    chunk |= (uint16_t)((air ? 1 : 0) << (2 * k));
    chunk |= (uint16_t)((geo ? 1 : 0) << (2 * k + 1));
  }
  return chunk;
}

svo_block make_block(const Scene &sc, int level, uint32_t x, uint32_t y, uint32_t z) {
  svo_block b;
  std::memset(&b, 0, sizeof(b));
  b.child = SVO_NO_CHILD;
  b.chunk = make_chunk(sc, level, x, y, z);
  b.opacity = 255;
  sc.normal(level, x, y, z, b.normal_pitch, b.normal_yaw);
  uint8_t rgb[3];
  sc.colour(level, x, y, z, rgb);
  b.colour_r = rgb[0];
  b.colour_g = rgb[1];
  b.colour_b = rgb[2];
  return b;
}

// Colour of a node with children: integer mean over the children whose
// octant holds geometry (the node's own colour otherwise).
void mean_colour(svo_block &parent, const svo_block *children) {
  uint32_t s[3] = {0, 0, 0}, n = 0;
  for (int k = 0; k < 8; k++)
    if ((parent.chunk >> (2 * k + 1)) & 1) {
      s[0] += children[k].colour_r;
      s[1] += children[k].colour_g;
      s[2] += children[k].colour_b;
      n++;
    }
  if (n) {
    parent.colour_r = (uint8_t)(s[0] / n);
    parent.colour_g = (uint8_t)(s[1] / n);
    parent.colour_b = (uint8_t)(s[2] / n);
  }
}

// One level-(B+2) subtree with local group numbers (child = local group,
// SVO_NO_CHILD = none).
struct Subtree {
  std::vector<svo_block> blocks;  // 8 per local group, pre-order of groups
};

// BuildBlocks (TreeBuilder.cs:237-256) with local allocation: group numbers
// 0,1,2,... are handed out in the order the queue would be dequeued.
void build_children(const Scene &sc, Subtree &st, uint32_t group, int level, uint32_t px, uint32_t py, uint32_t pz,
                    int max_depth) {
  for (int i = 0; i < 8; i++) {
    uint32_t x = 2 * px + (i & 1), y = 2 * py + ((i >> 1) & 1), z = 2 * pz + ((i >> 2) & 1);
    svo_block b = make_block(sc, level, x, y, z);
    if (level < max_depth && can_have_children(b.chunk)) {
      uint32_t g = (uint32_t)(st.blocks.size() / 8);
      st.blocks.resize(st.blocks.size() + 8);
      b.child = g;
      build_children(sc, st, g, level + 1, x, y, z, max_depth);
      mean_colour(b, &st.blocks[(size_t)g * 8]);
    }
    st.blocks[(size_t)group * 8 + i] = b;
  }
}

}  // namespace

struct TreeHost {
  uint8_t base_depth = 0;
  uint32_t block_count = 0;  // TreeBuilder's BlockCount
  std::vector<uint16_t> bases;
  std::vector<svo_block> blocks;
};

// A scene whose leaf grid lies one level below node level `scene_depth`.
struct SceneHost {
  uint64_t id = 0;  // unique per scene object (keys device copies of its data)
  std::unique_ptr<Scene> scene;
  int scene_depth = 0;
  int threads = 1;
  uint8_t base_depth = 0;
  uint64_t max_size = 0;
};

svo_status make_scene(const svo_scene_params &p, SceneHost &out) {
  const int B = p.base_depth, D = p.max_depth;
  if (B < 1 || B > 6) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_tree_build: base_depth must be 1..6");
  if (D < B + 2 || D > 16) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_tree_build: max_depth must be base_depth+2..16");
  static std::atomic<uint64_t> next_id{1};
  out.id = next_id.fetch_add(1);
  out.threads = p.threads > 0 ? p.threads : (int)std::max(1u, std::thread::hardware_concurrency());
  out.scene_depth = D;
  out.base_depth = (uint8_t)B;
  out.max_size = p.max_size;
  if (p.kind == SVO_SCENE_SPHERE)
    out.scene.reset(new SphereScene(p.seed, D + 1));
  else if (p.kind == SVO_SCENE_TERRAIN)
    out.scene.reset(new TerrainScene(p.seed, D + 1, out.threads));
  else
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_tree_build: unknown scene kind");
  return SVO_OK;
}

// TreeBuilder.BuildTree with nodes down to level D (<= the scene's depth).
svo_status build_tree_with(const SceneHost &scene, int D, TreeHost &tree) {
  const int B = scene.base_depth;
  if (D < B + 2 || D > scene.scene_depth)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_scene_build_tree: max_depth must be base_depth+2..the scene's depth");
  const int threads = scene.threads;
  const Scene *sc = scene.scene.get();
  svo_scene_params p{};
  p.max_size = scene.max_size;

  uint64_t max_size = p.max_size ? p.max_size : 0xFFFFFFFFull / 64;
  const uint64_t dense = 1ull << (3 * (B + 2));
  if (max_size < dense) max_size = dense;  // TreeBuilder.cs:105
  const uint64_t queue_end = max_size >> 3;

  tree.base_depth = (uint8_t)B;
  tree.bases.assign(pow_sum(B), 0);
  // BuildBaseChunks, TreeBuilder.cs:152-172
  for (int d = 1; d <= B; d++) {
    uint32_t n = 1u << d, start = pow_sum(d - 1);
    TerrainScene::parallel_for(threads, n, [&, n, start, d](uint32_t z) {
      for (uint32_t y = 0; y < n; y++)
        for (uint32_t x = 0; x < n; x++) tree.bases[start + morton3(x, y, z)] = make_chunk(*sc, d, x, y, z);
    });
  }

  // PopulateInitialBlocks, TreeBuilder.cs:180-227
  const uint32_t scan_n = 1u << (B + 1), base_start = pow_sum(B - 1);
  std::vector<uint8_t> populated((size_t)1 << (3 * (B + 1)), 0);
  for (uint32_t z = 0; z < scan_n; z++)
    for (uint32_t y = 0; y < scan_n; y++)
      for (uint32_t x = 0; x < scan_n; x++) {
        uint32_t pos = morton3(x, y, z);
        populated[pos] = ((tree.bases[base_start + (pos >> 3)] >> ((pos & 7) * 2)) & 3) == 3;
      }
  std::vector<uint32_t> empty_slots;
  for (uint32_t pos = 0; pos < populated.size(); pos++)
    if (!populated[pos]) empty_slots.push_back(pos);  // already sorted
  std::vector<svo_block> level2(dense);
  std::memset(level2.data(), 0, dense * sizeof(svo_block));
  std::vector<uint8_t> need(dense, 0);
  uint32_t block_count = 0;
  const uint32_t n2 = 1u << (B + 2);
  TerrainScene::parallel_for(threads, scan_n, [&](uint32_t z) {
    for (uint32_t y = 0; y < scan_n; y++)
      for (uint32_t x = 0; x < scan_n; x++) {
        uint32_t pos = morton3(x, y, z);
        if (!populated[pos]) continue;
        for (int k = 0; k < 8; k++) {
          uint32_t bx = 2 * x + (k & 1), by = 2 * y + ((k >> 1) & 1), bz = 2 * z + ((k >> 2) & 1);
          uint32_t a = (pos << 3) + (uint32_t)k;
          level2[a] = make_block(*sc, B + 2, bx, by, bz);
          need[a] = D > B + 2 && can_have_children(level2[a].chunk);
        }
      }
  });
  for (uint32_t pos = 0; pos < populated.size(); pos++)
    if (populated[pos]) block_count = std::max(block_count, (pos << 3) + 8);

  // Level-(B+2) subtrees in TreeBuilder's x, y, z visiting order.
  std::vector<uint32_t> roots;
  for (uint32_t x = 0; x < n2; x++)
    for (uint32_t y = 0; y < n2; y++)
      for (uint32_t z = 0; z < n2; z++) {
        uint32_t a = morton3(x, y, z);
        if (need[a]) roots.push_back(a);
      }
  std::vector<Subtree> subs(roots.size());
  TerrainScene::parallel_for(threads, (uint32_t)roots.size(), [&](uint32_t r) {
    uint32_t a = roots[r];  // level-(B+2) node
    uint32_t x = 0, y = 0, z = 0;
    for (int i = 0; i < B + 2; i++) {
      x |= ((a >> (3 * i)) & 1u) << i;
      y |= ((a >> (3 * i + 1)) & 1u) << i;
      z |= ((a >> (3 * i + 2)) & 1u) << i;
    }
    Subtree &st = subs[r];
    st.blocks.resize(8);
    build_children(*sc, st, 0, B + 3, x, y, z, D);
    mean_colour(level2[a], st.blocks.data());
  });

  // Queue positions: subtree r owns [off[r], off[r] + groups_r).
  std::vector<uint64_t> off(roots.size() + 1, 0);
  for (size_t r = 0; r < roots.size(); r++) off[r + 1] = off[r] + subs[r].blocks.size() / 8;
  const uint64_t capacity = empty_slots.size() + (queue_end > (1ull << (3 * (B + 1))) ? queue_end - (1ull << (3 * (B + 1))) : 0);
  if (off.back() > capacity)
    return fail(SVO_ERR_BUDGET, "svo_tree_build: tree needs " + std::to_string(off.back()) +
                                    " block groups but max_size allows " + std::to_string(capacity));
  auto queue_at = [&](uint64_t q) -> uint32_t {
    return q < empty_slots.size() ? empty_slots[q] : (uint32_t)((1ull << (3 * (B + 1))) + (q - empty_slots.size()));
  };
  uint64_t max_group = dense / 8 - 1;
  if (off.back() > 0) max_group = std::max<uint64_t>(max_group, queue_at(off.back() - 1));
  for (uint64_t q = 0; q < off.back() && q < empty_slots.size(); q++) max_group = std::max<uint64_t>(max_group, queue_at(q));
  tree.blocks.assign((max_group + 1) * 8, svo_block{});
  std::memcpy(tree.blocks.data(), level2.data(), dense * sizeof(svo_block));
  TerrainScene::parallel_for(threads, (uint32_t)roots.size(), [&](uint32_t r) {
    const Subtree &st = subs[r];
    tree.blocks[roots[r]].child = queue_at(off[r]) << 3;
    size_t groups = st.blocks.size() / 8;
    for (size_t g = 0; g < groups; g++) {
      uint32_t dst = queue_at(off[r] + g) << 3;
      for (int i = 0; i < 8; i++) {
        svo_block b = st.blocks[g * 8 + i];
        if (b.child != SVO_NO_CHILD) b.child = queue_at(off[r] + b.child) << 3;
        tree.blocks[dst + i] = b;
      }
    }
  });

  // TreeBuilder's BlockCount bookkeeping (TreeBuilder.cs:216 and :254, with
  // its "<" comparison) replayed in the order BuildBlocks writes nodes.
  struct Rec {
    static void walk(const std::vector<svo_block> &bl, uint32_t addr, uint32_t &bc) {
      for (uint32_t i = 0; i < 8; i++) {
        uint32_t c = bl[addr + i].child;
        if (c != SVO_NO_CHILD) walk(bl, c, bc);
        if (bc < addr + i) bc = addr + i + 1;
      }
    }
  };
  for (uint32_t a : roots) Rec::walk(tree.blocks, tree.blocks[a].child, block_count);
  tree.block_count = block_count;
  // "Trim final tree size down to populated volume" (TreeBuilder.cs:144-145):
  // Blocks = Blocks.Take(BlockCount). With the bookkeeping's "<" comparison the
  // count can stop one short of the last node written, which the reference
  // then drops; reads of it see a missing node, here as in the reference.
  if (tree.blocks.size() > block_count) tree.blocks.resize(block_count);
  return SVO_OK;
}

svo_status build_tree(const svo_scene_params &p, TreeHost &tree) {
  SceneHost scene;
  svo_status st = make_scene(p, scene);
  if (st) return st;
  return build_tree_with(scene, p.max_depth, tree);
}

// Graft payloads for child requests: one record per distinct requesting node
// (ascending node address, largest TreeSize of its requests); the payload is
// the node's children (and, for TreeSize 1, their children), built like
// BuildBlocks with local pre-order groups and children given as payload block
// indices (what WorldManager.UpdateGrafting hands to the graft kernel,
// SvoTracer.Window/WorldManager.cs:84-103).
struct GraftHost {
  std::vector<svo_grafting> records;
  std::vector<svo_block> payload;
};

svo_status graft_payload(const SceneHost &scene, const svo_child_request *req, size_t n, GraftHost &out) {
  std::vector<std::pair<uint32_t, size_t>> order;
  order.reserve(n);
  for (size_t i = 0; i < n; i++) order.push_back({req[i].address, i});
  std::sort(order.begin(), order.end());
  struct Job {
    uint32_t address;
    int depth;
    int limit;
    uint32_t x, y, z;
  };
  std::vector<Job> jobs;
  for (size_t k = 0; k < order.size();) {
    size_t e = k;
    uint8_t ts = 0;
    while (e < order.size() && order[e].first == order[k].first) ts = std::max(ts, req[order[e++].second].tree_size);
    const svo_child_request &r = req[order[k].second];
    int d = r.depth;
    if (d >= scene.base_depth + 2 && d < scene.scene_depth) {
      Job j;
      j.address = r.address;
      j.depth = d;
      j.limit = std::min(scene.scene_depth, d + 1 + (ts ? 1 : 0));
      j.x = (uint32_t)(r.location[0] >> (64 - d));
      j.y = (uint32_t)(r.location[1] >> (64 - d));
      j.z = (uint32_t)(r.location[2] >> (64 - d));
      jobs.push_back(j);
    }
    k = e;
  }
  std::vector<Subtree> subs(jobs.size());
  TerrainScene::parallel_for(scene.threads, (uint32_t)jobs.size(), [&](uint32_t i) {
    const Job &j = jobs[i];
    subs[i].blocks.resize(8);
    build_children(*scene.scene, subs[i], 0, j.depth + 1, j.x, j.y, j.z, j.limit);
  });
  size_t total = 0;
  for (auto &st : subs) total += st.blocks.size();
  out.payload.resize(total);
  out.records.resize(jobs.size());
  size_t at = 0;
  for (size_t i = 0; i < jobs.size(); i++) {
    const Subtree &st = subs[i];
    svo_grafting g{};
    g.graft_data_address = (uint32_t)at;
    g.graft_total_size = (uint32_t)(st.blocks.size() / 8);
    g.depth = 255;
    g.graft_address = jobs[i].address;
    out.records[i] = g;
    for (size_t b = 0; b < st.blocks.size(); b++) {
      svo_block blk = st.blocks[b];
      if (blk.child != SVO_NO_CHILD) blk.child = (uint32_t)at + 8u * blk.child;
      out.payload[at + b] = blk;
    }
    at += st.blocks.size();
  }
  return SVO_OK;
}

bool scene_terrain_info(const void *scene, TerrainInfo *out) {
  const SceneHost *sh = static_cast<const SceneHost *>(scene);
  const TerrainScene *t = dynamic_cast<const TerrainScene *>(sh->scene.get());
  if (!t || t->leaf >= kMaxTerrainLevels) return false;
  out->id = sh->id;
  out->base_depth = sh->base_depth;
  out->scene_depth = sh->scene_depth;
  out->leaf = t->leaf;
  out->res = t->res;
  out->seed = t->seed;
  for (int l = 0; l <= t->leaf; l++) {
    out->lo[l] = t->lo[l].data();
    out->hi[l] = t->hi[l].data();
  }
  return true;
}

}  // namespace svo

using svo::GraftHost;
using svo::SceneHost;
using svo::TreeHost;

extern "C" {

SVO_API svo_status svo_tree_build(const svo_scene_params *params, void **tree) {
  if (!params || !tree) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_tree_build: null argument");
  try {
    std::unique_ptr<TreeHost> t(new TreeHost);
    svo_status st = svo::build_tree(*params, *t);
    if (st != SVO_OK) return st;
    *tree = t.release();
    return SVO_OK;
  } catch (const std::bad_alloc &) {
    return svo::fail(SVO_ERR_OUT_OF_MEMORY, "svo_tree_build: out of host memory");
  } catch (const std::exception &e) {
    return svo::fail(SVO_ERR_INTERNAL, std::string("svo_tree_build: ") + e.what());
  }
}

SVO_API svo_status svo_tree_info(void *tree, uint8_t *base_depth, size_t *n_bases, size_t *n_blocks,
                                 uint32_t *block_count) {
  if (!tree) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_tree_info: null tree");
  auto *t = static_cast<TreeHost *>(tree);
  if (base_depth) *base_depth = t->base_depth;
  if (n_bases) *n_bases = t->bases.size();
  if (n_blocks) *n_blocks = t->blocks.size();
  if (block_count) *block_count = t->block_count;
  return SVO_OK;
}

SVO_API svo_status svo_tree_data(void *tree, const uint16_t **bases, const svo_block **blocks) {
  if (!tree) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_tree_data: null tree");
  auto *t = static_cast<TreeHost *>(tree);
  if (bases) *bases = t->bases.data();
  if (blocks) *blocks = t->blocks.data();
  return SVO_OK;
}

SVO_API svo_status svo_tree_free(void *tree) {
  delete static_cast<TreeHost *>(tree);
  return SVO_OK;
}

namespace {

// powSum (TreeBuilder.PowSum): base chunks of levels 1..depth.
uint64_t oct_pow_sum(int depth) {
  uint64_t s = 0, p = 1;
  for (int i = 1; i <= depth; i++) s += (p *= 8);
  return s;
}

struct FileCloser {
  void operator()(FILE *f) const {
    if (f) std::fclose(f);
  }
};

// Base depths whose chunk table a file can reasonably hold (powSum(8) = 19.2M).
constexpr int kMaxOctBaseDepth = 8;

}  // namespace

SVO_API svo_status svo_oct_write(const char *path, uint8_t base_depth, uint32_t block_count, const uint16_t *bases,
                                 size_t n_bases, const svo_block *blocks, size_t n_blocks) {
  if (!path || (!bases && n_bases) || (!blocks && n_blocks))
    return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_oct_write: null argument");
  if (base_depth > kMaxOctBaseDepth || n_bases != oct_pow_sum(base_depth))
    return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_oct_write: n_bases must be powSum(base_depth)");
  std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "wb"));
  if (!f) return svo::fail(SVO_ERR_IO, std::string("svo_oct_write: cannot create ") + path);
  uint8_t head[5];
  head[0] = base_depth;
  for (int k = 0; k < 4; k++) head[1 + k] = (uint8_t)(block_count >> (8 * k));
  bool ok = std::fwrite(head, 1, 5, f.get()) == 5;
  // both hosts this library builds for are little-endian, like BinaryWriter
  ok = ok && std::fwrite(bases, 2, n_bases, f.get()) == n_bases;
  ok = ok && std::fwrite(blocks, sizeof(svo_block), n_blocks, f.get()) == n_blocks;
  ok = (std::fflush(f.get()) == 0) && ok;
  if (!ok) return svo::fail(SVO_ERR_IO, std::string("svo_oct_write: write failed: ") + path);
  return SVO_OK;
}

SVO_API svo_status svo_oct_read(const char *path, void **tree) {
  if (!path || !tree) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_oct_read: null argument");
  std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "rb"));
  if (!f) return svo::fail(SVO_ERR_IO, std::string("svo_oct_read: cannot open ") + path);
  uint8_t head[5];
  if (std::fread(head, 1, 5, f.get()) != 5) return svo::fail(SVO_ERR_IO, "svo_oct_read: truncated header");
  const int base_depth = head[0];
  uint32_t block_count = 0;
  for (int k = 0; k < 4; k++) block_count |= (uint32_t)head[1 + k] << (8 * k);
  if (base_depth > kMaxOctBaseDepth)
    return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_oct_read: base depth " + std::to_string(base_depth) +
                                                   " is larger than " + std::to_string(kMaxOctBaseDepth));
  // the file must hold what the header announces before anything is allocated
  if (std::fseek(f.get(), 0, SEEK_END) != 0) return svo::fail(SVO_ERR_IO, "svo_oct_read: cannot seek");
  long long size = std::ftell(f.get());
  const uint64_t n_bases = oct_pow_sum(base_depth);
  const uint64_t need = 5 + 2 * n_bases + (uint64_t)sizeof(svo_block) * block_count;
  if (size < 0 || (uint64_t)size < need)
    return svo::fail(SVO_ERR_IO, "svo_oct_read: file holds " + std::to_string(size) + " bytes, the header needs " +
                                     std::to_string(need));
  if (std::fseek(f.get(), 5, SEEK_SET) != 0) return svo::fail(SVO_ERR_IO, "svo_oct_read: cannot seek");
  std::unique_ptr<TreeHost> t(new (std::nothrow) TreeHost);
  if (!t) return svo::fail(SVO_ERR_OUT_OF_MEMORY, "svo_oct_read: allocation failed");
  try {
    t->bases.resize(n_bases);
    t->blocks.resize(block_count);
  } catch (const std::bad_alloc &) {
    return svo::fail(SVO_ERR_OUT_OF_MEMORY, "svo_oct_read: allocation failed");
  }
  if (std::fread(t->bases.data(), 2, n_bases, f.get()) != n_bases ||
      std::fread(t->blocks.data(), sizeof(svo_block), block_count, f.get()) != block_count)
    return svo::fail(SVO_ERR_IO, "svo_oct_read: read failed");
  t->base_depth = (uint8_t)base_depth;
  t->block_count = block_count;
  *tree = t.release();
  return SVO_OK;
}

SVO_API svo_status svo_scene_create(const svo_scene_params *params, void **scene) {
  if (!params || !scene) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_scene_create: null argument");
  try {
    std::unique_ptr<SceneHost> s(new SceneHost);
    svo_status st = svo::make_scene(*params, *s);
    if (st) return st;
    *scene = s.release();
    return SVO_OK;
  } catch (const std::bad_alloc &) {
    return svo::fail(SVO_ERR_OUT_OF_MEMORY, "svo_scene_create: out of host memory");
  }
}

SVO_API svo_status svo_scene_build_tree(void *scene, uint8_t max_depth, void **tree) {
  if (!scene || !tree) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_scene_build_tree: null argument");
  try {
    std::unique_ptr<TreeHost> t(new TreeHost);
    svo_status st = svo::build_tree_with(*static_cast<SceneHost *>(scene), max_depth, *t);
    if (st) return st;
    *tree = t.release();
    return SVO_OK;
  } catch (const std::bad_alloc &) {
    return svo::fail(SVO_ERR_OUT_OF_MEMORY, "svo_scene_build_tree: out of host memory");
  }
}

SVO_API svo_status svo_scene_graft_payload(void *scene, const svo_child_request *requests, size_t n, void **graft) {
  if (!scene || !graft || (n && !requests)) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_scene_graft_payload: null");
  try {
    std::unique_ptr<GraftHost> g(new GraftHost);
    svo_status st = svo::graft_payload(*static_cast<SceneHost *>(scene), requests, n, *g);
    if (st) return st;
    *graft = g.release();
    return SVO_OK;
  } catch (const std::bad_alloc &) {
    return svo::fail(SVO_ERR_OUT_OF_MEMORY, "svo_scene_graft_payload: out of host memory");
  }
}

SVO_API svo_status svo_graft_payload_data(void *graft, const svo_grafting **records, size_t *n_records,
                                          const svo_block **payload, size_t *n_payload) {
  if (!graft) return svo::fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft_payload_data: null");
  auto *g = static_cast<GraftHost *>(graft);
  if (records) *records = g->records.data();
  if (n_records) *n_records = g->records.size();
  if (payload) *payload = g->payload.data();
  if (n_payload) *n_payload = g->payload.size();
  return SVO_OK;
}

SVO_API svo_status svo_graft_payload_free(void *graft) {
  delete static_cast<GraftHost *>(graft);
  return SVO_OK;
}

SVO_API svo_status svo_scene_free(void *scene) {
  delete static_cast<SceneHost *>(scene);
  return SVO_OK;
}

}  // extern "C"
