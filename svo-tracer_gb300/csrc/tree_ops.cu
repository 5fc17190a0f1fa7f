// Tree updates on the device: usage initialisation, block GC, grafting and
// pruning (the reference's prune/graft kernels, SvoTracer.Kernel/wavefront.cl:
// 1097-1350, restated as a specification the oracle shares):
//
//  * groups: 8-node block groups, one svo_usage each (Tick 0 free, 1..65533
//    last frame used, 65534 multi-parent, 65535 inviolate);
//  * dense-real groups: the level-(B+2) groups under air+geometry
//    level-(B+1) cells, addressed by baseLocation; never allocated or freed;
//  * reachable: an allocatable group whose first node is the Child of a node
//    of a dense-real or reachable group.
//
// GC detaches stale groups (age > threshold in the wrapping tick space) from
// their parent node, then frees every allocated group that is no longer
// reachable, and compacts the free groups into an ascending free list. Grafts
// claim groups from that list in record order. Pruning applies the reference's
// Pruning records in order and frees the groups CullChild orphaned. The
// reference serialises its dereferencing through a global spin lock
// (wavefront.cl:226-231); here reachability is recomputed breadth-first with
// one pass per tree level, so no thread ever waits on another.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <set>
#include <string>
#include <vector>

#include "context.h"
#include "scene_common.h"

namespace svo {
namespace cg = cooperative_groups;
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;

struct TreeView {
  const uint16_t *bases;
  svo_block *blocks;
  svo_usage *usage;
  uint32_t n_groups;
  uint32_t base_start;    // powSum(B-1): first level-B base chunk
  uint32_t dense_groups;  // 8^(B+1)
  int32_t base_depth;
};

__device__ __forceinline__ bool dense_real(const TreeView &t, uint32_t g) {
  if (g >= t.dense_groups) return false;
  uint16_t chunk = t.bases[t.base_start + (g >> 3)];
  return ((chunk >> ((g & 7) * 2)) & 3) == 3;
}

__device__ __forceinline__ uint32_t tick_age(uint32_t t, uint32_t now) {
  return now >= t ? now - t : now + 65533u - t;
}

// Appends v to a list at *count with one atomic per group of the warp's lanes
// that append at the same time (the list's order is not significant).
__device__ __forceinline__ void append(uint32_t *list, uint32_t *count, uint32_t v) {
  cg::coalesced_group g = cg::coalesced_threads();
  uint32_t base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(count, g.size());
  list[g.shfl(base, 0) + g.thread_rank()] = v;
}

__global__ void k_reach_seed(TreeView t, uint32_t *reach, uint32_t *parent_min, uint32_t *frontier,
                             uint32_t *count) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < t.n_groups; g += gridDim.x * blockDim.x) {
    reach[g] = 0;
    if (parent_min) parent_min[g] = kNone;
    if (dense_real(t, g)) append(frontier, count, g);
  }
}

// One breadth-first level: every node of every frontier group marks its child group.
// Visits one child link of the walk: marks the child group reached and appends
// it to the next frontier the first time.
__device__ __forceinline__ uint32_t reach_child(const TreeView &t, uint32_t node, uint32_t c, uint32_t *parent_min) {
  if (c == kNone || (c & 7u)) return kNone;
  const uint32_t h = c >> 3;
  if (h >= t.n_groups || dense_real(t, h)) return kNone;
  if (parent_min) atomicMin(parent_min + h, node);
  return h;
}

// One level of the walk: one node per thread (loads coalesced across the warp),
// each thread taking up to four nodes a grid apart whose loads and atomics are
// issued together (the walk is bound by the latency of these dependent loads
// and atomics, not by bandwidth).
__global__ void k_reach_expand(TreeView t, const uint32_t *frontier, const uint32_t *n_in, uint32_t *next,
                               uint32_t *n_out, uint32_t *reach, uint32_t *parent_min) {
  constexpr int kU = 4;
  const uint64_t total = 8ull * *n_in;
  const uint64_t threads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; base < total; base += kU * threads) {
    uint32_t node[kU], h[kU], first[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const uint64_t i = base + u * threads;
      node[u] = i < total ? frontier[i >> 3] * 8u + (uint32_t)(i & 7) : kNone;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) h[u] = node[u] != kNone ? t.blocks[node[u]].child : kNone;
#pragma unroll
    for (int u = 0; u < kU; u++) h[u] = node[u] != kNone ? reach_child(t, node[u], h[u], parent_min) : kNone;
#pragma unroll
    for (int u = 0; u < kU; u++) first[u] = h[u] != kNone ? atomicExch(reach + h[u], 1u) : 1u;
#pragma unroll
    for (int u = 0; u < kU; u++)
      if (first[u] == 0u) append(next, n_out, h[u]);
  }
}

__global__ void k_init_usage_tree(TreeView t, const uint32_t *reach, const uint32_t *parent_min, uint16_t tick) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < t.n_groups; g += gridDim.x * blockDim.x) {
    svo_usage u;
    u._pad = 0;
    if (dense_real(t, g)) {
      u.tick = 65535;
      u.parent = kNone;
    } else if (reach[g]) {
      u.tick = tick;
      u.parent = parent_min[g];
    } else {
      u.tick = 0;
      u.parent = kNone;
    }
    t.usage[g] = u;
  }
}

// Stale groups: flag and detach from the parent node that still points at them.
// params: [0] the frame's tick, [1] the staleness threshold (device memory, so
// that a captured GC graph replays with the current frame's values).
__global__ void k_stale_detach(TreeView t, const uint32_t *params, uint8_t *flags) {
  const uint16_t now = (uint16_t)params[0];
  const uint32_t threshold = params[1];
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < t.n_groups; g += gridDim.x * blockDim.x) {
    uint8_t f = 0;
    uint32_t tk = t.usage[g].tick;
    if (tk >= 1 && tk <= 65533 && !dense_real(t, g) && tick_age(tk, now) > threshold) {
      f = 1;
      uint32_t p = t.usage[g].parent;
      if (p != kNone && p < t.n_groups * 8u && t.blocks[p].child == g * 8u) t.blocks[p].child = kNone;
    }
    flags[g] = f;
  }
}

// Frees allocated groups that are no longer reachable; flags them.
// `unfinished`: the frontier left after the last breadth-first level; when it is
// not empty the tree is deeper than the levels run, reachability is incomplete,
// and nothing is freed (the host reports the error).
__global__ void k_sweep(TreeView t, const uint32_t *reach, uint8_t *flags, const uint32_t *unfinished) {
  const bool ok = *unfinished == 0;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < t.n_groups; g += gridDim.x * blockDim.x) {
    if (!ok) {
      flags[g] = 0;
      continue;
    }
    uint8_t f = 0;
    uint32_t tk = t.usage[g].tick;
    if (tk >= 1 && tk <= 65533 && !reach[g] && !dense_real(t, g)) {
      svo_usage u;
      u.tick = 0;
      u._pad = 0;
      u.parent = kNone;
      t.usage[g] = u;
      f = 1;
    }
    flags[g] = f;
  }
}

__global__ void k_free_flags(TreeView t, uint8_t *flags) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < t.n_groups; g += gridDim.x * blockDim.x)
    flags[g] = (t.usage[g].tick == 0 && !dense_real(t, g)) ? 1 : 0;
}

// ---- stream compaction of a flag array into the ascending list of indices ----
constexpr int kScanBlock = 1024;

template <class T>
__global__ void k_count(const T *flags, uint32_t n, uint32_t *block_counts) {
  uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  int c = __syncthreads_count(i < n && flags[i]);
  if (threadIdx.x == 0) block_counts[blockIdx.x] = (uint32_t)c;
}

// Exclusive scan of n block counts (in place) by one CTA; writes the total.
// Exclusive scan in place of n counts by one CTA of kScanBlock threads, total to *total.
__device__ void scan_in_place(uint32_t *counts, uint32_t n, uint32_t *total) {
  __shared__ uint32_t part[kScanBlock];
  uint32_t per = (n + kScanBlock - 1) / kScanBlock;
  uint32_t b = threadIdx.x * per, e = min(n, b + per), s = 0;
  for (uint32_t i = b; i < e; i++) s += counts[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    uint32_t v = threadIdx.x >= (uint32_t)off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - s;  // exclusive prefix of this thread's range
  for (uint32_t i = b; i < e; i++) {
    uint32_t c = counts[i];
    counts[i] = run;
    run += c;
  }
  if (threadIdx.x == kScanBlock - 1) *total = part[kScanBlock - 1];
}

__global__ void k_scan_counts(uint32_t *counts, uint32_t n, uint32_t *total) { scan_in_place(counts, n, total); }

template <class T>
__global__ void k_scatter(const T *flags, uint32_t n, const uint32_t *offsets, uint32_t *out) {
  __shared__ uint32_t warp_base[kScanBlock / 32];
  uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  bool f = i < n && flags[i];
  unsigned m = __ballot_sync(0xffffffffu, f);
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_base[warp] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int w = 0; w < kScanBlock / 32; w++) {
      uint32_t c = warp_base[w];
      warp_base[w] = run;
      run += c;
    }
  }
  __syncthreads();
  if (f) out[offsets[blockIdx.x] + warp_base[warp] + __popc(m & ((1u << lane) - 1u))] = i;
}

// ---- grafting ------------------------------------------------------------------
struct GraftJob {
  uint32_t payload_block;  // first payload block of this group
  uint32_t record;
  uint32_t k;              // group index within the record's subtree
};

struct GraftRec {
  uint32_t P, G, q, target;  // payload block, groups, first free-list slot, target node
};

__global__ void k_graft_usage(TreeView t, const GraftJob *jobs, uint32_t n_jobs, const GraftRec *recs,
                              const uint32_t *free_list, uint16_t now) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_jobs; j += gridDim.x * blockDim.x) {
    uint32_t g = free_list[recs[jobs[j].record].q + jobs[j].k];
    svo_usage u;
    u.tick = now;
    u._pad = 0;
    u.parent = kNone;
    t.usage[g] = u;
  }
}

__global__ void k_graft_nodes(TreeView t, const GraftJob *jobs, uint32_t n_jobs, const GraftRec *recs,
                              const uint32_t *free_list, const svo_block *payload) {
  for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < 8ull * n_jobs;
       x += (uint64_t)gridDim.x * blockDim.x) {
    const GraftJob jb = jobs[x >> 3];
    const GraftRec r = recs[jb.record];
    uint32_t i = (uint32_t)(x & 7);
    svo_block b = payload[jb.payload_block + i];
    uint32_t node = free_list[r.q + jb.k] * 8u + i;
    uint32_t c = b.child;
    if (c != kNone) {
      uint32_t rel = c - r.P;
      if (c < r.P || (rel & 7u) || rel / 8u >= r.G) {
        b.child = kNone;
      } else {
        uint32_t h = free_list[r.q + rel / 8u];
        b.child = h * 8u;
        atomicMin(&t.usage[h].parent, node);
      }
    }
    t.blocks[node] = b;
  }
}

__global__ void k_graft_link(TreeView t, const GraftRec *recs, uint32_t n, const uint32_t *free_list) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    uint32_t g = free_list[recs[r].q];
    t.usage[g].parent = recs[r].target;
    t.blocks[recs[r].target].child = g * 8u;
  }
}

__device__ __forceinline__ uint32_t loc_octant(const uint64_t *loc, int d) {
  int s = 63 - d;
  return (uint32_t)(((loc[0] >> s) & 1) | (((loc[1] >> s) & 1) << 1) | (((loc[2] >> s) & 1) << 2));
}

// Location walk of getBlockAddress for graft targets given by Location.
__global__ void k_resolve_targets(TreeView t, const svo_grafting *rec, uint32_t n, const uint64_t *locs,
                                  uint64_t n_locs, uint32_t *targets) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    if (rec[r].depth == 255) {
      targets[r] = rec[r].graft_address;
      continue;
    }
    if ((uint64_t)rec[r].graft_address * 3 + 3 > n_locs) {
      targets[r] = kNone;
      continue;
    }
    const uint64_t *loc = locs + 3ull * rec[r].graft_address;
    uint32_t a = 0;
    for (int i = 0; i < t.base_depth + 2; i++) a = (a << 3) + loc_octant(loc, i);
    for (int d = t.base_depth + 2; d < rec[r].depth; d++) {
      if (a >= t.n_groups * 8u || t.blocks[a].child == kNone) {
        a = kNone;
        break;
      }
      a = t.blocks[a].child + loc_octant(loc, d);
    }
    targets[r] = a;
  }
}

// ---- pruning: the records are applied in order by one thread -------------------
__global__ void k_prune(TreeView t, uint16_t *bases_rw, uint32_t n_bases, uint16_t now, const svo_pruning *rec,
                        uint32_t n_rec, const svo_block *surface, uint32_t n_surface, const uint64_t *locs,
                        uint64_t n_locs, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                        uint32_t *culled) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  uint32_t n_blocks = t.n_groups * 8u;
  for (uint32_t r = 0; r < n_rec; r++) {
    const svo_pruning p = rec[r];
    uint32_t address = p.address;
    if ((p.properties >> 4) & 1) {  // BaseBlock
      if (address < n_bases) bases_rw[address] = p.chunk;
      continue;
    }
    if (p.depth != 255) {  // findAddress (wavefront.cl:1191-1211)
      if ((uint64_t)address * 3 + 3 > n_locs) continue;
      const uint64_t *loc = locs + 3ull * address;
      uint32_t a = 0;
      for (int i = 0; i < t.base_depth + 2; i++) a = (a << 3) + loc_octant(loc, i);
      bool missing = false;
      for (int i = t.base_depth + 2; i < p.depth; i++) {
        if (a >= n_blocks) {
          missing = true;
          break;
        }
        if (t.usage[a >> 3].tick < 65534) t.usage[a >> 3].tick = now;
        if (t.blocks[a].child == kNone) {
          uint32_t slot = (*n_req)++;
          if (req && slot < req_cap) {
            svo_child_request q;
            memset(&q, 0, sizeof(q));
            q.address = a;
            q.tick = now;
            q.depth = (uint8_t)i;
            q.location[0] = loc[0];
            q.location[1] = loc[1];
            q.location[2] = loc[2];
            q.tree_size = (uint8_t)(p.depth - i);
            req[slot] = q;
          }
          missing = true;
          break;
        }
        a = t.blocks[a].child + loc_octant(loc, i);
      }
      if (missing) continue;
      address = a;
    } else {
      if (address >= n_blocks || t.usage[address >> 3].tick == 0) continue;  // dereferenced
      if (t.usage[address >> 3].tick < 65534) t.usage[address >> 3].tick = now;
    }
    if (address >= n_blocks) continue;
    if (p.properties & 1) {  // CullChild
      t.blocks[address].child = p.child_address;
      *culled = 1;
    }
    uint32_t v = (p.properties >> 1) & 3;  // AlterViolability / MakeInviolate
    if (v == 3)
      t.usage[address >> 3].tick = 65535;
    else if (v == 1)
      t.usage[address >> 3].tick = now;
    if ((p.properties >> 3) & 1) {  // UpdateChunk
      if (p.colour_address < n_surface) t.blocks[address] = surface[p.colour_address];
      t.blocks[address].chunk = p.chunk;
    }
  }
}

int grid_for(uint64_t n, int bs = 256) {
  uint64_t g = (n + bs - 1) / bs;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, 152ull * 64));
}

TreeView view_of(Context &c) {
  TreeView t;
  t.bases = c.bases.p;
  t.blocks = c.blocks.p;
  t.usage = c.usage.p;
  t.n_groups = (uint32_t)c.n_groups;
  uint32_t s = 0, p = 1;
  for (int i = 1; i <= c.base_depth - 1; i++) s += (p *= 8);
  t.base_start = s;
  t.dense_groups = 1u << (3 * (c.base_depth + 1));
  t.base_depth = c.base_depth;
  return t;
}


// Breadth-first reachability from the dense-real groups, one launch per tree
// level below B+2 without reading the frontier sizes back: each launch reads
// its frontier size on the device (an empty frontier makes it a no-op). The
// tree's nodes lie at depths <= c.tree_depth, so tree_depth - B - 1 levels end
// with an empty frontier; the returned pointer holds the frontier left after
// the last level (0 when reachability is complete).
// scan_tmp = [block counts | ... | n-8, n-7: frontier sizes | n-6: compact total
//             | n-5: prune flag | n-4..n-2: GC totals]
uint32_t *reachability_async(Context &c, const TreeView &t, bool with_parents) {
  uint32_t *cnt = c.scan_tmp.p + (c.scan_tmp.n - 8);
  // the smallest parent node of each group is needed only for the usage
  // initialisation; without it the walk takes one scattered atomic per group, not two
  uint32_t *parents = with_parents ? c.parent_min.p : nullptr;
  cudaMemsetAsync(cnt, 0, 2 * sizeof(uint32_t), c.stream);
  k_reach_seed<<<grid_for(t.n_groups), 256, 0, c.stream>>>(t, c.reach.p, parents, c.frontier_a.p, cnt);
  uint32_t *in = c.frontier_a.p, *out = c.frontier_b.p;
  uint32_t *n_in = cnt, *n_out = cnt + 1;
  const int levels = std::max(1, std::min(c.tree_depth, SVO_MAX_TREE_DEPTH) - (int)c.base_depth - 1);
  for (int level = 0; level < levels; level++) {
    cudaMemsetAsync(n_out, 0, 4, c.stream);
    k_reach_expand<<<152 * 8, 256, 0, c.stream>>>(t, in, n_in, out, n_out, c.reach.p, parents);
    std::swap(in, out);
    std::swap(n_in, n_out);
  }
  return n_in;
}

svo_status reachability(Context &c, const TreeView &t) {
  uint32_t *left = reachability_async(c, t, true);
  SVO_CUDA(cudaGetLastError(), "reachability");
  uint32_t n = 0;
  SVO_CUDA(cudaMemcpyAsync(&n, left, 4, cudaMemcpyDeviceToHost, c.stream), "reachability: frontier size");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "reachability: synchronize");
  if (n) return fail(SVO_ERR_INTERNAL, "reachability: tree deeper than its recorded depth");
  return SVO_OK;
}

// Ascending indices of flags[i] != 0 into out; the count goes to *total on the device.
void compact_async(Context &c, const uint8_t *flags, uint32_t n, uint32_t *out, uint32_t *total) {
  uint32_t nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb == 0) {
    cudaMemsetAsync(total, 0, 4, c.stream);
    return;
  }
  uint32_t *counts = c.scan_tmp.p;
  k_count<<<nb, kScanBlock, 0, c.stream>>>(flags, n, counts);
  k_scan_counts<<<1, kScanBlock, 0, c.stream>>>(counts, nb, total);
  k_scatter<<<nb, kScanBlock, 0, c.stream>>>(flags, n, counts, out);
}


// Reachability, the sweep of unreachable allocated groups and the free list,
// enqueued without a synchronisation (a GC graph captures it): the freed count,
// the free-list length, the frontier left and (with `pruned_total`, a device
// slot already written) the pruned count go to the pinned h_out[0..3].
svo_status enqueue_sweep(Context &c, const TreeView &t, const uint32_t *pruned_total, uint32_t *h_out) {
  uint32_t *left = reachability_async(c, t, false);
  uint32_t *totals = c.scan_tmp.p + (c.scan_tmp.n - 4);  // [0] freed, [1] free, [2] frontier left
  k_sweep<<<grid_for(t.n_groups), 256, 0, c.stream>>>(t, c.reach.p, c.flags.p, left);
  compact_async(c, c.flags.p, t.n_groups, c.freed_list.p, totals);
  k_free_flags<<<grid_for(t.n_groups), 256, 0, c.stream>>>(t, c.flags.p);
  compact_async(c, c.flags.p, t.n_groups, c.free_list.p, totals + 1);
  SVO_CUDA(cudaMemcpyAsync(totals + 2, left, 4, cudaMemcpyDeviceToDevice, c.stream), "tree update: frontier");
  SVO_CUDA(cudaGetLastError(), "tree update: kernels");
  SVO_CUDA(cudaMemcpyAsync(h_out, totals, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream), "tree update: counts");
  if (pruned_total)
    SVO_CUDA(cudaMemcpyAsync(h_out + 3, pruned_total, 4, cudaMemcpyDeviceToHost, c.stream), "tree update: counts");
  return SVO_OK;
}

// The host side of a completed sweep: the counts read back into h[0..3].
svo_status finish_sweep(Context &c, const uint32_t *h, uint64_t *n_freed, uint64_t *n_pruned) {
  if (h[2]) {
    c.free_valid = false;
    return fail(SVO_ERR_INTERNAL, "tree update: tree deeper than its recorded depth; nothing was freed");
  }
  *n_freed = h[0];
  if (n_pruned) *n_pruned = h[3];
  c.n_free = h[1];
  c.free_used = 0;
  c.free_valid = true;
  return SVO_OK;
}

svo_status sweep_and_free_list(Context &c, const TreeView &t, uint64_t *n_freed, uint64_t *n_pruned = nullptr,
                               const uint32_t *pruned_total = nullptr) {
  uint32_t *h = c.h_gc_out.p;
  h[0] = h[1] = h[2] = h[3] = 0;
  svo_status st = enqueue_sweep(c, t, pruned_total, h);
  if (st) return st;
  SVO_CUDA(cudaStreamSynchronize(c.stream), "tree update: synchronize");
  return finish_sweep(c, h, n_freed, n_pruned);
}

// ---- graft payloads generated on the device (terrain scenes) -------------------
//
// The same payload the host generator builds for a frame's child requests
// (one job per distinct requesting node in ascending address order, its eight
// children and, for TreeSize 1, the children of those that can have children,
// BuildBlocks-style), grafted with svo_graft's rules, but without the host
// round trip: requests are deduplicated through a per-node marker, jobs sized
// and claimed from the free list in record order, and the nodes generated
// straight into the claimed groups from the terrain's column pyramids.

struct DevTerrain {
  const uint16_t *lo, *hi;  // all levels concatenated
  uint64_t off[kMaxTerrainLevels];
  int leaf;
  uint32_t res, seed;
};

struct GenJob {
  uint32_t address;  // requesting node: the graft target
  uint32_t x, y, z;  // its cell at `depth`
  uint32_t q;        // first free-list slot of its groups, or kNone when skipped
  uint8_t depth, mask, groups, _pad;  // mask: children that get a group of their own
};
static_assert(sizeof(GenJob) == 24, "GenJob layout");

__device__ __forceinline__ uint16_t terrain_chunk(const DevTerrain &T, int level, uint32_t x, uint32_t y, uint32_t z) {
  // MakeChunk: classify the eight level+1 cells
  const int l1 = level + 1;
  uint16_t chunk = 0;
  for (int k = 0; k < 8; k++) {
    const uint32_t cx = 2 * x + (k & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + ((k >> 2) & 1);
    const uint64_t idx = T.off[l1] + (uint64_t)cy * (1u << l1) + cx;
    bool geo, air;
    scene::terrain_classify(T.hi[idx], T.lo[idx], T.res, T.leaf, l1, cz, geo, air);
    chunk |= (uint16_t)((air ? 1 : 0) << (2 * k));
    chunk |= (uint16_t)((geo ? 1 : 0) << (2 * k + 1));
  }
  return chunk;
}

// MakeBlock of the host builder for a terrain cell (no children yet).
__device__ __forceinline__ svo_block terrain_block(const DevTerrain &T, int level, uint32_t x, uint32_t y, uint32_t z) {
  svo_block b;
  b.child = kNone;
  b.chunk = terrain_chunk(T, level, x, y, z);
  scene::terrain_normal(T.hi + T.off[level], level, T.leaf, x, y, b.normal_pitch, b.normal_yaw);
  uint8_t rgb[3];
  scene::terrain_colour(T.seed, level, x, y, z, rgb);
  b.colour_r = rgb[0];
  b.colour_g = rgb[1];
  b.colour_b = rgb[2];
  b.opacity = 255;
  b.specularity = 0;
  b.gloss = 0;
  return b;
}

// Marks every requesting node with (TreeSize != 0) << 31 | (request + 1),
// keeping the largest: any request of a node gives its depth and cell.
// The marked node's group also gets its bit in `group_bits` (one bit per group).
__global__ void k_gen_mark(const svo_child_request *req, const uint32_t *n_req, uint32_t cap, uint32_t *marker,
                           uint32_t *group_bits, uint32_t n_nodes, int min_depth, int scene_depth) {
  const uint32_t n = min(*n_req, cap);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const svo_child_request r = req[i];
    if (r.depth >= min_depth && r.depth < scene_depth && r.address < n_nodes) {
      atomicMax(&marker[r.address], ((r.tree_size ? 1u : 0u) << 31) | (i + 1));
      atomicOr(&group_bits[r.address >> 8], 1u << ((r.address >> 3) & 31u));
    }
  }
}

// Stream compaction of a group bitmap into the ascending list of marked groups
// (which clears the bitmap): set bits counted per CTA of 1024 words, then each
// word's bits written at its exclusive offset.
__global__ void k_bits_count(const uint32_t *bits, uint32_t n_words, uint32_t *block_counts) {
  __shared__ uint32_t wsum[32];
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  uint32_t c = __reduce_add_sync(0xffffffffu, i < n_words ? (uint32_t)__popc(bits[i]) : 0u);
  if ((threadIdx.x & 31u) == 0) wsum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    c = __reduce_add_sync(0xffffffffu, wsum[threadIdx.x]);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = c;
  }
}

__global__ void k_bits_scatter(uint32_t *bits, uint32_t n_words, const uint32_t *offsets, uint32_t *out) {
  __shared__ uint32_t wsum[32];
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t word = i < n_words ? bits[i] : 0u;
  const uint32_t c = __popc(word);
  uint32_t x = c;  // inclusive scan within the warp
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t own = wsum[lane];
    uint32_t incl = own;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    wsum[lane] = incl - own;  // exclusive prefix of the warps' counts
  }
  __syncthreads();
  uint32_t off = offsets[blockIdx.x] + wsum[warp] + (x - c);
  for (uint32_t m = word; m; m &= m - 1u) out[off++] = i * 32u + (uint32_t)(__ffs(m) - 1);
  if (word) bits[i] = 0;
}

// Marked nodes of each listed group (counts[j] for group list entry j).
__global__ void k_group_node_count(const uint32_t *groups, const uint32_t *n_groups, uint32_t cap,
                                   const uint32_t *marker, uint32_t *counts) {
  const uint32_t n = min(*n_groups, cap);
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t *m = marker + 8ull * groups[j];
    uint32_t c = 0;
    for (int k = 0; k < 8; k++) c += m[k] != 0;
    counts[j] = c;
  }
}

// The same scan of *n_ptr (read on the device, at most cap) counts.
__global__ void __launch_bounds__(kScanBlock) k_scan_device_n(uint32_t *counts, const uint32_t *n_ptr, uint32_t cap,
                                                              uint32_t *total) {
  scan_in_place(counts, min(*n_ptr, cap), total);
}

// The marked nodes of the listed groups in ascending order.
__global__ void k_group_node_emit(const uint32_t *groups, const uint32_t *n_groups, uint32_t cap,
                                  const uint32_t *marker, const uint32_t *offsets, uint32_t *out) {
  const uint32_t n = min(*n_groups, cap);
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t node0 = 8u * groups[j];
    uint32_t off = offsets[j];
    for (uint32_t k = 0; k < 8; k++)
      if (marker[node0 + k]) out[off++] = node0 + k;
  }
}

// One job per marked node (ascending): its cell, depth and groups; clears the marker.
__global__ void k_gen_size(const DevTerrain T, const uint32_t *addr, const uint32_t *n_jobs, uint32_t cap,
                           uint32_t *marker, const svo_child_request *req, int scene_depth, GenJob *jobs) {
  const uint32_t n = min(*n_jobs, cap);
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t a = addr[j];
    const uint32_t m = marker[a];
    marker[a] = 0;
    const svo_child_request r = req[(m & 0x7FFFFFFFu) - 1];
    const int d = r.depth;
    GenJob g;
    g.address = a;
    g.x = (uint32_t)(r.location[0] >> (64 - d));
    g.y = (uint32_t)(r.location[1] >> (64 - d));
    g.z = (uint32_t)(r.location[2] >> (64 - d));
    g.q = kNone;
    g.depth = (uint8_t)d;
    g._pad = 0;
    const int limit = min(scene_depth, d + 1 + (int)(m >> 31));
    uint32_t mask = 0;
    if (d + 1 < limit)
      for (int o = 0; o < 8; o++) {
        uint16_t ch = terrain_chunk(T, d + 1, 2 * g.x + (o & 1), 2 * g.y + ((o >> 1) & 1), 2 * g.z + ((o >> 2) & 1));
        if (scene::can_have_children(ch)) mask |= 1u << o;
      }
    g.mask = (uint8_t)mask;
    g.groups = (uint8_t)(1 + __popc(mask));
    jobs[j] = g;
  }
}

// Claims, one CTA: jobs in order take `groups` free-list slots each; a job that
// no longer fits is skipped and later ones still try (svo_graft's rule).
// Before the first job that overflows, claims are a prefix sum; from it on one
// thread applies the rule in order. scalars[1] = applied jobs, [2] = groups.
__global__ void __launch_bounds__(1024) k_gen_claim(GenJob *jobs, const uint32_t *n_jobs, uint32_t cap,
                                                    uint64_t avail, uint32_t *scalars) {
  __shared__ uint32_t part[1024];
  __shared__ uint32_t first_over, used_at_first;
  const uint32_t n = min(*n_jobs, cap);
  const uint32_t per = (n + 1023) / 1024, b = threadIdx.x * per, e = min(n, b + per);
  uint32_t sum = 0;
  for (uint32_t j = b; j < e; j++) sum += jobs[j].groups;
  part[threadIdx.x] = sum;
  if (threadIdx.x == 0) {
    first_over = n;
    used_at_first = 0;
  }
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t v = threadIdx.x >= (uint32_t)off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  const uint32_t excl = part[threadIdx.x] - sum;
  uint64_t run = excl;
  for (uint32_t j = b; j < e; j++) {
    run += jobs[j].groups;
    if (run > avail) {
      atomicMin(&first_over, j);
      break;
    }
  }
  __syncthreads();
  const uint32_t k = first_over;
  run = excl;
  for (uint32_t j = b; j < e && j <= k; j++) {
    if (j == k) {
      used_at_first = (uint32_t)run;
      break;
    }
    jobs[j].q = (uint32_t)run;
    run += jobs[j].groups;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t used = k < n ? used_at_first : (n ? part[1023] : 0);
    uint32_t applied = k;
    for (uint32_t j = k; j < n; j++) {
      const uint32_t gsz = jobs[j].groups;
      if (used + gsz <= avail) {
        jobs[j].q = (uint32_t)used;
        used += gsz;
        applied++;
      }
    }
    scalars[1] = applied;
    scalars[2] = (uint32_t)used;
  }
}

// Eight threads per claimed job: child o of the requesting node, its own
// children when it gets a group, usage entries and the link to the target.
__global__ void k_gen_write(const DevTerrain T, TreeView t, const GenJob *jobs, const uint32_t *n_jobs, uint32_t cap,
                            const uint32_t *free_list, uint64_t free_base, uint16_t now) {
  const uint32_t n = min(*n_jobs, cap);
  for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < 8ull * n;
       x += (uint64_t)gridDim.x * blockDim.x) {
    const GenJob g = jobs[x >> 3];
    if (g.q == kNone) continue;
    const uint32_t o = (uint32_t)(x & 7);
    const uint32_t g0 = free_list[free_base + g.q];
    const uint32_t node = g0 * 8u + o;
    const int level = g.depth + 1;
    const uint32_t cx = 2 * g.x + (o & 1), cy = 2 * g.y + ((o >> 1) & 1), cz = 2 * g.z + ((o >> 2) & 1);
    svo_block b = terrain_block(T, level, cx, cy, cz);
    if ((g.mask >> o) & 1u) {
      const uint32_t k = 1 + __popc(g.mask & ((1u << o) - 1u));
      const uint32_t gk = free_list[free_base + g.q + k];
      uint32_t sr = 0, sg = 0, sb = 0, cnt = 0;
      for (int i = 0; i < 8; i++) {
        svo_block c = terrain_block(T, level + 1, 2 * cx + (i & 1), 2 * cy + ((i >> 1) & 1), 2 * cz + ((i >> 2) & 1));
        t.blocks[gk * 8u + i] = c;
        if ((b.chunk >> (2 * i + 1)) & 1) {  // the mean over the geometry octants
          sr += c.colour_r;
          sg += c.colour_g;
          sb += c.colour_b;
          cnt++;
        }
      }
      svo_usage u;
      u.tick = now;
      u._pad = 0;
      u.parent = node;
      t.usage[gk] = u;
      b.child = gk * 8u;
      if (cnt) {
        b.colour_r = (uint8_t)(sr / cnt);
        b.colour_g = (uint8_t)(sg / cnt);
        b.colour_b = (uint8_t)(sb / cnt);
      }
    }
    t.blocks[node] = b;
    if (o == 0) {
      svo_usage u;
      u.tick = now;
      u._pad = 0;
      u.parent = g.address;
      t.usage[g0] = u;
      t.blocks[g.address].child = g0 * 8u;
    }
  }
}

}  // namespace

// The tree updates' scratch (reachability, flags, lists) for the context's budget.
svo_status ensure_tree_buffers(Context &c) {
  size_t g = c.n_groups;
  size_t nb = (g + kScanBlock - 1) / kScanBlock + 1;
  if (c.reach.reserve(g) || c.parent_min.reserve(g) || c.frontier_a.reserve(g) || c.frontier_b.reserve(g) ||
      c.flags.reserve(g) || c.scan_tmp.reserve(nb + 12) || c.free_list.reserve(g) || c.pruned_list.reserve(g) ||
      c.freed_list.reserve(g) || c.gc_params.reserve(2) || c.h_gc_params.reserve(2) || c.h_gc_out.reserve(4))
    return fail(SVO_ERR_OUT_OF_MEMORY, "tree update: device allocation failed");
  return SVO_OK;
}
}  // namespace svo

using svo::Context;
using svo::fail;

#define CTX(ptr, fn)                                                                          \
  if (!(ptr)) return fail(SVO_ERR_INVALID_ARGUMENT, std::string(fn) + ": null context"); \
  Context &c = *static_cast<Context *>(ptr);                                                \
  if (!c.has_tree) return fail(SVO_ERR_NO_TREE, std::string(fn) + ": no octree uploaded");   \
  SVO_CUDA(cudaSetDevice(c.device), "cudaSetDevice")

extern "C" {

SVO_API svo_status svo_init_usage_tree(void *ctx, uint16_t tick) {
  CTX(ctx, "svo_init_usage_tree");
  if (tick < 1 || tick > 65533) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_init_usage_tree: tick must be 1..65533");
  svo_status st = svo::ensure_tree_buffers(c);
  if (st) return st;
  svo::TreeView t = svo::view_of(c);
  st = svo::reachability(c, t);
  if (st) return st;
  svo::k_init_usage_tree<<<svo::grid_for(t.n_groups), 256, 0, c.stream>>>(t, c.reach.p, c.parent_min.p, tick);
  SVO_CUDA(cudaGetLastError(), "svo_init_usage_tree");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_init_usage_tree: synchronize");
  c.free_valid = false;
  return SVO_OK;
}

SVO_API svo_status svo_gc(void *ctx, const svo_update_input *in, svo_gc_report *report) {
  CTX(ctx, "svo_gc");
  if (!in) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_gc: null input");
  if (in->tick < 1 || in->tick > 65533) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_gc: tick must be 1..65533");
  svo_status st = svo::ensure_tree_buffers(c);
  if (st) return st;
  svo::TreeView t = svo::view_of(c);
  // The GC's ~30 launches (stale detach, one reachability level per tree level,
  // sweep, three compactions) and count read-backs replay from a CUDA graph,
  // captured for the tree's shape and buffers; the frame's tick and threshold
  // reach it through a pinned word its first node copies.
  c.h_gc_params.p[0] = in->tick;
  c.h_gc_params.p[1] = in->offset;
  uint32_t *pruned_total = c.scan_tmp.p + (c.scan_tmp.n - 5 + 4);  // the slot after the GC totals
  const std::vector<uint64_t> key = {c.n_groups, (uint64_t)c.tree_depth, c.base_depth, (uintptr_t)c.blocks.p,
                                     (uintptr_t)c.usage.p, (uintptr_t)c.bases.p, (uintptr_t)c.reach.p,
                                     (uintptr_t)c.flags.p, (uintptr_t)c.scan_tmp.p, c.scan_tmp.n,
                                     (uintptr_t)c.free_list.p, (uintptr_t)c.pruned_list.p, (uintptr_t)c.freed_list.p,
                                     (uintptr_t)c.frontier_a.p, (uintptr_t)c.frontier_b.p, (uintptr_t)c.stream};
  if (!c.gc_exec || c.gc_key != key) {
    if (c.gc_exec) cudaGraphExecDestroy(c.gc_exec);
    c.gc_exec = nullptr;
    SVO_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal), "svo_gc: capture");
    cudaMemcpyAsync(c.gc_params.p, c.h_gc_params.p, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream);
    svo::k_stale_detach<<<svo::grid_for(t.n_groups), 256, 0, c.stream>>>(t, c.gc_params.p, c.flags.p);
    svo::compact_async(c, c.flags.p, t.n_groups, c.pruned_list.p, pruned_total);
    svo_status est = svo::enqueue_sweep(c, t, pruned_total, c.h_gc_out.p);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(c.stream, &g);
    if (est) {
      if (g) cudaGraphDestroy(g);
      return est;
    }
    if (ce != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("svo_gc: end capture: ") + cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&c.gc_exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      c.gc_exec = nullptr;
      return fail(SVO_ERR_CUDA, std::string("svo_gc: instantiate: ") + cudaGetErrorString(ce));
    }
    c.gc_key = key;
  }
  SVO_CUDA(cudaGraphLaunch(c.gc_exec, c.stream), "svo_gc: launch");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_gc: synchronize");
  st = svo::finish_sweep(c, c.h_gc_out.p, &c.n_freed, &c.n_pruned);
  if (st) return st;
  if (report) {
    report->pruned = c.n_pruned;
    report->freed = c.n_freed;
    report->free = c.n_free;
  }
  return SVO_OK;
}

SVO_API svo_status svo_read_gc_lists(void *ctx, uint32_t *pruned, size_t cap_pruned, uint32_t *freed,
                                     size_t cap_freed, uint32_t *free_list, size_t cap_free) {
  CTX(ctx, "svo_read_gc_lists");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_gc_lists: synchronize");
  size_t np = std::min<size_t>(cap_pruned, c.n_pruned), nf = std::min<size_t>(cap_freed, c.n_freed);
  size_t nl = c.free_valid ? std::min<size_t>(cap_free, c.n_free - c.free_used) : 0;
  if (pruned && np) SVO_CUDA(cudaMemcpy(pruned, c.pruned_list.p, np * 4, cudaMemcpyDeviceToHost), "svo_read_gc_lists");
  if (freed && nf) SVO_CUDA(cudaMemcpy(freed, c.freed_list.p, nf * 4, cudaMemcpyDeviceToHost), "svo_read_gc_lists");
  if (free_list && nl)
    SVO_CUDA(cudaMemcpy(free_list, c.free_list.p + c.free_used, nl * 4, cudaMemcpyDeviceToHost), "svo_read_gc_lists");
  return SVO_OK;
}

// Node levels that a graft record's payload hangs below its target: the longest
// chain of child groups from the record's group 0 (links outside the record's
// groups are dropped, as k_graft_nodes drops them); -1 when the links form a cycle.
static int payload_levels(const svo_block *payload, uint32_t P, uint32_t G) {
  std::vector<uint32_t> frontier{0}, next, mark(G, 0);
  for (uint32_t level = 1; level <= G; level++) {
    next.clear();
    for (uint32_t g : frontier)
      for (uint32_t i = 0; i < 8; i++) {
        const uint32_t c = payload[P + 8ull * g + i].child;
        if (c == SVO_NO_CHILD || c < P) continue;
        const uint32_t rel = c - P;
        if ((rel & 7u) || rel / 8u >= G) continue;
        if (mark[rel / 8u] != level + 1) {
          mark[rel / 8u] = level + 1;
          next.push_back(rel / 8u);
        }
      }
    if (next.empty()) return (int)level;
    frontier.swap(next);
  }
  return -1;  // a group is still reached after G levels
}

SVO_API svo_status svo_graft(void *ctx, const svo_update_input *in, const svo_grafting *records, uint32_t n_records,
                             const svo_block *payload, size_t n_payload, const uint64_t *locations,
                             size_t n_locations, svo_graft_report *report) {
  CTX(ctx, "svo_graft");
  if (!in || (n_records && !records) || (n_payload && !payload))
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft: null argument");
  if (in->tick < 1 || in->tick > 65533) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft: tick must be 1..65533");
  if (n_payload > 0xFFFFFFF0ull) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft: payload too large");
  svo_status st = svo::ensure_tree_buffers(c);
  if (st) return st;
  svo::TreeView t = svo::view_of(c);
  if (!c.free_valid) {  // no GC ran since the tree changed: build the free list now
    uint64_t dummy = 0;
    st = svo::sweep_and_free_list(c, t, &dummy);
    if (st) return st;
    c.n_freed = dummy;
  }
  if (report) std::memset(report, 0, sizeof(*report));
  if (n_records == 0) return SVO_OK;
  // resolve targets on the device (Location walks), then assign free-list ranges in record order
  if (c.graft_records.reserve(n_records) || c.graft_targets.reserve(n_records) ||
      (n_locations && c.locations.reserve(n_locations)))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft: device allocation failed");
  SVO_CUDA(cudaMemcpyAsync(c.graft_records.p, records, sizeof(svo_grafting) * n_records, cudaMemcpyHostToDevice,
                           c.stream), "svo_graft: records");
  if (n_locations)
    SVO_CUDA(cudaMemcpyAsync(c.locations.p, locations, sizeof(uint64_t) * n_locations, cudaMemcpyHostToDevice,
                             c.stream), "svo_graft: locations");
  svo::k_resolve_targets<<<svo::grid_for(n_records), 256, 0, c.stream>>>(
      t, c.graft_records.p, n_records, c.locations.p, n_locations, c.graft_targets.p);
  std::vector<uint32_t> targets(n_records);
  SVO_CUDA(cudaMemcpyAsync(targets.data(), c.graft_targets.p, 4ull * n_records, cudaMemcpyDeviceToHost, c.stream),
           "svo_graft: targets");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_graft: synchronize");
  std::vector<svo::GraftRec> recs;
  std::vector<svo::GraftJob> jobs;
  std::vector<uint8_t> applied(n_records, 0);
  std::set<uint32_t> seen;
  uint64_t q = c.free_used;
  uint64_t n_blocks = (uint64_t)c.n_groups * 8;
  int deepest = c.tree_depth;  // deepest node level once the applied records are grafted
  for (uint32_t r = 0; r < n_records; r++) {
    uint32_t G = records[r].graft_total_size, P = records[r].graft_data_address;
    if (G == 0 || (P & 7u) || (uint64_t)P + 8ull * G > n_payload) continue;
    if (q + G > c.n_free) continue;
    uint32_t target = targets[r];
    if (target == svo::kNone || target >= n_blocks) continue;
    if (!seen.insert(target).second)
      return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft: two records graft onto node " + std::to_string(target));
    svo::GraftRec gr{P, G, (uint32_t)q, target};
    // the target of a Location record is the node at level max(depth, B+2); a
    // target given as a node index has no known level
    const int levels = records[r].depth == 255 ? -1 : payload_levels(payload, P, G);
    deepest = levels < 0 ? SVO_MAX_TREE_DEPTH
                         : std::max(deepest, std::max<int>(records[r].depth, c.base_depth + 2) + levels);
    uint32_t rec_index = (uint32_t)recs.size();
    recs.push_back(gr);
    for (uint32_t k = 0; k < G; k++) jobs.push_back(svo::GraftJob{P + 8 * k, rec_index, k});
    applied[r] = 1;
    q += G;
  }
  uint64_t claimed = q - c.free_used;
  if (!recs.empty()) {
    static_assert(sizeof(svo::GraftJob) == 12 && sizeof(svo::GraftRec) == 16, "graft job layout");
    size_t job_words = jobs.size() * 3, rec_words = recs.size() * 4;
    if (c.payload.reserve(n_payload) || c.graft_jobs.reserve(job_words + rec_words) ||
        c.claimed_list.reserve(std::max<uint64_t>(claimed, 1)))
      return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft: device allocation failed");
    svo::GraftRec *d_recs = reinterpret_cast<svo::GraftRec *>(c.graft_jobs.p + job_words);
    SVO_CUDA(cudaMemcpyAsync(c.payload.p, payload, sizeof(svo_block) * n_payload, cudaMemcpyHostToDevice, c.stream),
             "svo_graft: payload");
    SVO_CUDA(cudaMemcpyAsync(c.graft_jobs.p, jobs.data(), sizeof(svo::GraftJob) * jobs.size(),
                             cudaMemcpyHostToDevice, c.stream), "svo_graft: jobs");
    SVO_CUDA(cudaMemcpyAsync(d_recs, recs.data(), sizeof(svo::GraftRec) * recs.size(), cudaMemcpyHostToDevice,
                             c.stream), "svo_graft: records");
    const svo::GraftJob *d_jobs = reinterpret_cast<const svo::GraftJob *>(c.graft_jobs.p);
    uint32_t nj = (uint32_t)jobs.size();
    svo::k_graft_usage<<<svo::grid_for(nj), 256, 0, c.stream>>>(t, d_jobs, nj, d_recs, c.free_list.p, in->tick);
    svo::k_graft_nodes<<<svo::grid_for(8ull * nj), 256, 0, c.stream>>>(t, d_jobs, nj, d_recs, c.free_list.p,
                                                                      c.payload.p);
    svo::k_graft_link<<<svo::grid_for(recs.size()), 256, 0, c.stream>>>(t, d_recs, (uint32_t)recs.size(),
                                                                        c.free_list.p);
    SVO_CUDA(cudaGetLastError(), "svo_graft: kernels");
    SVO_CUDA(cudaMemcpyAsync(c.claimed_list.p, c.free_list.p + c.free_used, claimed * 4, cudaMemcpyDeviceToDevice,
                             c.stream), "svo_graft: claimed list");
    SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_graft: synchronize");
  }
  c.n_claimed = claimed;
  c.free_used = q;
  // grafted subtrees can reach below the deepest level seen so far
  if (claimed) c.tree_depth = std::min(SVO_MAX_TREE_DEPTH, std::max(c.tree_depth, deepest));
  if (report) {
    report->applied = (uint32_t)recs.size();
    report->skipped = n_records - (uint32_t)recs.size();
    report->claimed = claimed;
    report->free_left = c.n_free - c.free_used;
  }
  return SVO_OK;
}

SVO_API svo_status svo_read_graft_claims(void *ctx, uint32_t *claimed, size_t cap) {
  CTX(ctx, "svo_read_graft_claims");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_read_graft_claims: synchronize");
  size_t n = std::min<size_t>(cap, c.n_claimed);
  if (claimed && n)
    SVO_CUDA(cudaMemcpy(claimed, c.claimed_list.p, n * 4, cudaMemcpyDeviceToHost), "svo_read_graft_claims");
  return SVO_OK;
}

SVO_API svo_status svo_prune(void *ctx, const svo_update_input *in, const svo_pruning *records, uint32_t n_records,
                             const svo_block *surface, size_t n_surface, const uint64_t *locations,
                             size_t n_locations, svo_prune_report *report) {
  CTX(ctx, "svo_prune");
  if (!in || (n_records && !records)) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_prune: null argument");
  if (in->tick < 1 || in->tick > 65533) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_prune: tick must be 1..65533");
  svo_status st = svo::ensure_tree_buffers(c);
  if (st) return st;
  svo::TreeView t = svo::view_of(c);
  if (report) std::memset(report, 0, sizeof(*report));
  if (n_records == 0) return SVO_OK;
  uint32_t cap = std::max<uint32_t>(c.request_cap, 4096);
  if (c.prune_records.reserve(n_records) || c.payload.reserve(std::max<size_t>(n_surface, 1)) ||
      (n_locations && c.locations.reserve(n_locations)) || c.requests.reserve(cap))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_prune: device allocation failed");
  c.request_cap = cap;
  SVO_CUDA(cudaMemcpyAsync(c.prune_records.p, records, sizeof(svo_pruning) * n_records, cudaMemcpyHostToDevice,
                           c.stream), "svo_prune: records");
  if (n_surface)
    SVO_CUDA(cudaMemcpyAsync(c.payload.p, surface, sizeof(svo_block) * n_surface, cudaMemcpyHostToDevice, c.stream),
             "svo_prune: surface");
  if (n_locations)
    SVO_CUDA(cudaMemcpyAsync(c.locations.p, locations, sizeof(uint64_t) * n_locations, cudaMemcpyHostToDevice,
                             c.stream), "svo_prune: locations");
  uint32_t *culled = c.scan_tmp.p + (c.scan_tmp.n - 5);
  uint32_t before = 0;
  SVO_CUDA(cudaMemcpyAsync(&before, c.counters.p + 1, 4, cudaMemcpyDeviceToHost, c.stream), "svo_prune: requests");
  SVO_CUDA(cudaMemsetAsync(culled, 0, 4, c.stream), "svo_prune: reset");
  svo::k_prune<<<1, 1, 0, c.stream>>>(t, c.bases.p, (uint32_t)c.n_bases, in->tick, c.prune_records.p, n_records,
                                     c.payload.p, (uint32_t)n_surface, c.locations.p, n_locations, c.requests.p, cap,
                                     c.counters.p + 1, culled);
  SVO_CUDA(cudaGetLastError(), "svo_prune: kernel");
  uint32_t was_culled = 0, after = 0;
  SVO_CUDA(cudaMemcpyAsync(&was_culled, culled, 4, cudaMemcpyDeviceToHost, c.stream), "svo_prune: flag");
  SVO_CUDA(cudaMemcpyAsync(&after, c.counters.p + 1, 4, cudaMemcpyDeviceToHost, c.stream), "svo_prune: requests");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_prune: synchronize");
  // CullChild can point a node at any group: the tree's depth is no longer known
  c.tree_depth = SVO_MAX_TREE_DEPTH;
  uint64_t freed = 0;
  if (was_culled) {
    st = svo::sweep_and_free_list(c, t, &freed);
    if (st) return st;
  } else {
    c.free_valid = false;
  }
  c.n_freed = freed;
  c.n_pruned = 0;
  if (report) {
    report->freed = freed;
    report->requests = after - before;
  }
  return SVO_OK;
}

}  // extern "C"

SVO_API svo_status svo_graft_generate(void *ctx, void *scene, const svo_update_input *in, svo_graft_report *report) {
  CTX(ctx, "svo_graft_generate");
  if (!scene || !in) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft_generate: null argument");
  if (in->tick < 1 || in->tick > 65533) return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft_generate: tick must be 1..65533");
  svo::TerrainInfo ti;
  if (!svo::scene_terrain_info(scene, &ti))
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft_generate: device generation needs a terrain scene");
  if (ti.base_depth != c.base_depth)
    return fail(SVO_ERR_INVALID_ARGUMENT, "svo_graft_generate: scene and resident tree differ in base depth");
  svo_status st = svo::ensure_tree_buffers(c);
  if (st) return st;
  svo::TreeView t = svo::view_of(c);
  if (!c.free_valid) {  // no GC ran since the tree changed: build the free list now
    uint64_t dummy = 0;
    st = svo::sweep_and_free_list(c, t, &dummy);
    if (st) return st;
    c.n_freed = dummy;
  }
  if (report) std::memset(report, 0, sizeof(*report));
  const uint32_t cap = c.request_cap;
  if (cap == 0 || !c.requests.p) {
    c.n_claimed = 0;
    return SVO_OK;
  }
  // the scene's column pyramids, once per scene
  svo::DevTerrain T{};
  uint64_t total = 0;
  for (int l = 0; l <= ti.leaf; l++) {
    T.off[l] = total;
    total += 1ull << (2 * l);
  }
  if (c.terrain_id != ti.id) {
    c.terrain_id = 0;
    if (c.terrain_lo.reserve(total) || c.terrain_hi.reserve(total))
      return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft_generate: terrain allocation failed");
    for (int l = 0; l <= ti.leaf; l++) {
      size_t bytes = (1ull << (2 * l)) * sizeof(uint16_t);
      SVO_CUDA(cudaMemcpyAsync(c.terrain_lo.p + T.off[l], ti.lo[l], bytes, cudaMemcpyHostToDevice, c.stream),
               "svo_graft_generate: terrain");
      SVO_CUDA(cudaMemcpyAsync(c.terrain_hi.p + T.off[l], ti.hi[l], bytes, cudaMemcpyHostToDevice, c.stream),
               "svo_graft_generate: terrain");
    }
    SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_graft_generate: terrain");
    c.terrain_id = ti.id;
  }
  T.lo = c.terrain_lo.p;
  T.hi = c.terrain_hi.p;
  T.leaf = ti.leaf;
  T.res = ti.res;
  T.seed = ti.seed;
  // marker (zero between calls), compaction counts, jobs
  const uint32_t n_nodes = (uint32_t)(c.n_groups * 8);
  if (c.gen_marker.n < n_nodes) {
    if (c.gen_marker.reserve(n_nodes)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft_generate: allocation failed");
    SVO_CUDA(cudaMemsetAsync(c.gen_marker.p, 0, (size_t)n_nodes * 4, c.stream), "svo_graft_generate: marker");
  }
  // the group bitmap (one bit per group, zero between calls)
  const uint32_t n_words = (uint32_t)((c.n_groups + 31) / 32);
  if (c.gen_bits.n < n_words) {
    if (c.gen_bits.reserve(n_words)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft_generate: allocation failed");
    SVO_CUDA(cudaMemsetAsync(c.gen_bits.p, 0, (size_t)n_words * 4, c.stream), "svo_graft_generate: bitmap");
  }
  const uint32_t nb = (n_words + svo::kScanBlock - 1) / svo::kScanBlock;
  const uint32_t list_cap = std::max(1u, cap);  // marked groups and nodes never exceed the stored requests
  if (c.gen_counts.reserve(std::max(nb + 1, list_cap)) || c.gen_addr.reserve(list_cap) ||
      c.gen_groups.reserve(list_cap) || c.gen_scalars.reserve(4) ||
      c.gen_jobs.reserve(sizeof(svo::GenJob) * (size_t)list_cap))
    return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft_generate: allocation failed");
  uint32_t *scalars = c.gen_scalars.p;  // [0] jobs, [1] applied, [2] claimed groups, [3] marked groups
  svo::GenJob *jobs = reinterpret_cast<svo::GenJob *>(c.gen_jobs.p);
  const uint32_t *n_req = c.counters.p + 1;  // the last trace's request count
  svo::k_gen_mark<<<svo::grid_for(cap), 256, 0, c.stream>>>(c.requests.p, n_req, cap, c.gen_marker.p, c.gen_bits.p,
                                                            n_nodes, ti.base_depth + 2, ti.scene_depth);
  // marked groups (ascending), then their marked nodes (ascending): the jobs
  svo::k_bits_count<<<nb, svo::kScanBlock, 0, c.stream>>>(c.gen_bits.p, n_words, c.gen_counts.p);
  svo::k_scan_counts<<<1, svo::kScanBlock, 0, c.stream>>>(c.gen_counts.p, nb, scalars + 3);
  svo::k_bits_scatter<<<nb, svo::kScanBlock, 0, c.stream>>>(c.gen_bits.p, n_words, c.gen_counts.p, c.gen_groups.p);
  svo::k_group_node_count<<<svo::grid_for(cap), 256, 0, c.stream>>>(c.gen_groups.p, scalars + 3, list_cap,
                                                                    c.gen_marker.p, c.gen_counts.p);
  svo::k_scan_device_n<<<1, svo::kScanBlock, 0, c.stream>>>(c.gen_counts.p, scalars + 3, list_cap, scalars);
  svo::k_group_node_emit<<<svo::grid_for(cap), 256, 0, c.stream>>>(c.gen_groups.p, scalars + 3, list_cap,
                                                                   c.gen_marker.p, c.gen_counts.p, c.gen_addr.p);
  svo::k_gen_size<<<svo::grid_for(cap), 256, 0, c.stream>>>(T, c.gen_addr.p, scalars, cap, c.gen_marker.p,
                                                            c.requests.p, ti.scene_depth, jobs);
  const uint64_t avail = c.n_free - c.free_used;
  svo::k_gen_claim<<<1, 1024, 0, c.stream>>>(jobs, scalars, cap, avail, scalars);
  svo::k_gen_write<<<svo::grid_for(8ull * cap), 256, 0, c.stream>>>(T, t, jobs, scalars, cap, c.free_list.p,
                                                                    c.free_used, in->tick);
  SVO_CUDA(cudaGetLastError(), "svo_graft_generate: kernels");
  uint32_t sc[3] = {0, 0, 0};
  SVO_CUDA(cudaMemcpyAsync(sc, scalars, sizeof(sc), cudaMemcpyDeviceToHost, c.stream), "svo_graft_generate: counts");
  SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_graft_generate: synchronize");
  const uint64_t claimed = sc[2];
  if (claimed) {
    if (c.claimed_list.reserve(claimed)) return fail(SVO_ERR_OUT_OF_MEMORY, "svo_graft_generate: allocation failed");
    SVO_CUDA(cudaMemcpyAsync(c.claimed_list.p, c.free_list.p + c.free_used, claimed * 4, cudaMemcpyDeviceToDevice,
                             c.stream), "svo_graft_generate: claimed list");
    SVO_CUDA(cudaStreamSynchronize(c.stream), "svo_graft_generate: synchronize");
    // generated nodes lie at most at the scene's depth
    c.tree_depth = std::max(c.tree_depth, ti.scene_depth);
  }
  c.n_claimed = claimed;
  c.free_used += claimed;
  if (report) {
    report->applied = sc[1];
    report->skipped = sc[0] - sc[1];
    report->claimed = claimed;
    report->free_left = c.n_free - c.free_used;
  }
  return SVO_OK;
}
