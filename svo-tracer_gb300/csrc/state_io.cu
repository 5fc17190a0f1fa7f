// Streaming-state snapshot (checkpoint / resume) of a context.
//
// The reference persists only the octree (.oct, OctreeSerializer); the usage
// ticks, the free block groups and the tree's growth are lost. A stream of
// frames (trace, GC, grafts) depends on all of them, so resuming it needs the
// whole resident state: the base chunks, every block of the budget (grafted
// groups live past the uploaded tree), the usage array, the depth the tree has
// grown to and the free list of the last GC with the part of it grafts have
// claimed. svo_state_save writes that state to a file after the context's
// pending work; svo_state_load replaces a context's resident tree with it, after
// which the next frames give what the saved context's would have.
//
// File layout (little-endian):
//   "SVOSTAT1"                                        8 bytes
//   uint32 version (1), uint8 base_depth, uint8 tree_depth, uint16 0
//   uint64 n_bases, n_blocks, budget, n_free, free_used
//   uint32 free_valid, uint32 0
//   uint16 bases[n_bases], zero padding to a multiple of 8 bytes
//   svo_block blocks[budget]
//   svo_usage usage[budget / 8]
//   uint32 free_list[n_free]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

using svo::Context;
using svo::fail;

namespace {

uint64_t pow_sum_host(int depth) {  // powSum (wavefront.cl:224): base chunks of levels 1..depth
  uint64_t s = 0, p = 1;
  for (int i = 1; i <= depth; i++) s += (p *= 8);
  return s;
}

constexpr char kMagic[8] = {'S', 'V', 'O', 'S', 'T', 'A', 'T', '1'};
constexpr uint32_t kVersion = 1;

struct StateHeader {
  char magic[8];
  uint32_t version;
  uint8_t base_depth, tree_depth;
  uint16_t _pad0;
  uint64_t n_bases, n_blocks, budget, n_free, free_used;
  uint32_t free_valid, _pad1;
};
static_assert(sizeof(StateHeader) == 64, "state header layout");

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

bool write_all(FILE *f, const void *p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }
bool read_all(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

}  // namespace

#define STATE_CUDA(call, what)                                                              \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return fail(SVO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)

extern "C" {

SVO_API svo_status svo_state_save(void *ctx, const char *path) {
  if (!ctx) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_save: null context");
  if (!path) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_save: null path");
  Context &c = *static_cast<Context *>(ctx);
  try {
    if (!c.has_tree) return fail(SVO_ERR_NO_TREE, "svo_state_save: no octree uploaded");
    STATE_CUDA(cudaSetDevice(c.device), "svo_state_save: cudaSetDevice");
    STATE_CUDA(cudaStreamSynchronize(c.stream), "svo_state_save: synchronize");
    const size_t n_groups = c.budget / 8;
    const uint64_t n_free = c.free_valid ? c.n_free : 0;
    std::vector<uint16_t> bases(c.n_bases);
    std::vector<svo_block> blocks(c.budget);
    std::vector<svo_usage> usage(n_groups);
    std::vector<uint32_t> free_list(n_free);
    STATE_CUDA(cudaMemcpy(bases.data(), c.bases.p, c.n_bases * 2, cudaMemcpyDeviceToHost), "svo_state_save: bases");
    STATE_CUDA(cudaMemcpy(blocks.data(), c.blocks.p, c.budget * sizeof(svo_block), cudaMemcpyDeviceToHost),
               "svo_state_save: blocks");
    STATE_CUDA(cudaMemcpy(usage.data(), c.usage.p, n_groups * sizeof(svo_usage), cudaMemcpyDeviceToHost),
               "svo_state_save: usage");
    if (n_free)
      STATE_CUDA(cudaMemcpy(free_list.data(), c.free_list.p, n_free * 4, cudaMemcpyDeviceToHost),
                 "svo_state_save: free list");
    StateHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.base_depth = c.base_depth;
    h.tree_depth = (uint8_t)c.tree_depth;
    h.n_bases = c.n_bases;
    h.n_blocks = c.n_blocks;
    h.budget = c.budget;
    h.n_free = n_free;
    h.free_used = c.free_valid ? c.free_used : 0;
    h.free_valid = c.free_valid ? 1u : 0u;
    const std::string tmp = std::string(path) + ".tmp";
    {
      File f;
      f.f = fopen(tmp.c_str(), "wb");
      if (!f.f) return fail(SVO_ERR_IO, std::string("svo_state_save: cannot open ") + tmp);
      static const uint8_t zeros[8] = {0};
      const size_t pad = (8 - (c.n_bases * 2) % 8) % 8;
      if (!write_all(f.f, &h, sizeof(h)) || !write_all(f.f, bases.data(), c.n_bases * 2) ||
          !write_all(f.f, zeros, pad) || !write_all(f.f, blocks.data(), c.budget * sizeof(svo_block)) ||
          !write_all(f.f, usage.data(), n_groups * sizeof(svo_usage)) ||
          !write_all(f.f, free_list.data(), n_free * 4) || fflush(f.f) != 0)
        return fail(SVO_ERR_IO, std::string("svo_state_save: write failed: ") + tmp);
    }
    if (std::rename(tmp.c_str(), path) != 0) return fail(SVO_ERR_IO, std::string("svo_state_save: cannot rename to ") + path);
    return SVO_OK;
  } catch (const std::bad_alloc &) {
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_state_save: out of host memory");
  }
}

SVO_API svo_status svo_state_load(void *ctx, const char *path) {
  if (!ctx) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_load: null context");
  if (!path) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_load: null path");
  Context &c = *static_cast<Context *>(ctx);
  try {
    File f;
    f.f = fopen(path, "rb");
    if (!f.f) return fail(SVO_ERR_IO, std::string("svo_state_load: cannot open ") + path);
    StateHeader h;
    if (!read_all(f.f, &h, sizeof(h))) return fail(SVO_ERR_IO, "svo_state_load: truncated header");
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion)
      return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_load: not a state file of this version");
    const bool sane = h.base_depth >= 1 && h.base_depth <= 8 && h.n_bases == pow_sum_host(h.base_depth) &&
                      h.budget % 8 == 0 && h.budget >= ((uint64_t)1 << (3 * (h.base_depth + 2))) &&
                      h.budget <= 0xFFFFFFF8ull && h.n_blocks <= h.budget && h.tree_depth <= SVO_MAX_TREE_DEPTH &&
                      h.tree_depth >= h.base_depth + 2 && h.n_free <= h.budget / 8 && h.free_used <= h.n_free &&
                      h.free_valid <= 1;
    if (!sane) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_load: inconsistent header");
    const size_t n_groups = h.budget / 8;
    std::vector<uint16_t> bases(h.n_bases);
    std::vector<svo_block> blocks(h.budget);
    std::vector<svo_usage> usage(n_groups);
    std::vector<uint32_t> free_list(h.n_free);
    uint8_t pad[8];
    const size_t npad = (8 - (h.n_bases * 2) % 8) % 8;
    if (!read_all(f.f, bases.data(), h.n_bases * 2) || !read_all(f.f, pad, npad) ||
        !read_all(f.f, blocks.data(), h.budget * sizeof(svo_block)) ||
        !read_all(f.f, usage.data(), n_groups * sizeof(svo_usage)) || !read_all(f.f, free_list.data(), h.n_free * 4))
      return fail(SVO_ERR_IO, "svo_state_load: truncated file");
    for (uint32_t g : free_list)
      if (g >= n_groups) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_state_load: free-list entry out of range");

    STATE_CUDA(cudaSetDevice(c.device), "svo_state_load: cudaSetDevice");
    STATE_CUDA(cudaStreamSynchronize(c.stream), "svo_state_load: synchronize");
    // the cached graphs hold the previous buffers and tree shape
    if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
    c.graph_exec = nullptr;
    if (c.gc_exec) cudaGraphExecDestroy(c.gc_exec);
    c.gc_exec = nullptr;
    c.has_tree = false;
    c.has_params = false;
    c.budget = h.budget;
    c.n_groups = n_groups;
    if (c.bases.reserve(h.n_bases) || c.blocks.reserve(h.budget) || c.usage.reserve(n_groups))
      return fail(SVO_ERR_OUT_OF_MEMORY, "svo_state_load: device allocation failed");
    svo_status st = svo::ensure_tree_buffers(c);
    if (st) return st;
    STATE_CUDA(cudaMemcpy(c.bases.p, bases.data(), h.n_bases * 2, cudaMemcpyHostToDevice), "svo_state_load: bases");
    STATE_CUDA(cudaMemcpy(c.blocks.p, blocks.data(), h.budget * sizeof(svo_block), cudaMemcpyHostToDevice),
               "svo_state_load: blocks");
    STATE_CUDA(cudaMemcpy(c.usage.p, usage.data(), n_groups * sizeof(svo_usage), cudaMemcpyHostToDevice),
               "svo_state_load: usage");
    if (h.n_free)
      STATE_CUDA(cudaMemcpy(c.free_list.p, free_list.data(), h.n_free * 4, cudaMemcpyHostToDevice),
                 "svo_state_load: free list");
    c.base_depth = h.base_depth;
    c.n_bases = h.n_bases;
    c.n_blocks = h.n_blocks;
    c.tree_depth = h.tree_depth;
    c.free_valid = h.free_valid != 0;
    c.n_free = h.n_free;
    c.free_used = h.free_used;
    c.n_pruned = c.n_freed = c.n_claimed = 0;
    c.has_tree = true;
    return SVO_OK;
  } catch (const std::bad_alloc &) {
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_state_load: out of host memory");
  }
}

}  // extern "C"
