/*
 * svo_tree_oracle.c -- TEST INFRASTRUCTURE ONLY: parity checker of the tree
 * update kernels (usage initialisation, block GC, grafting, pruning).
 *
 * The reference's prune/graft kernels (SvoTracer/SvoTracer.Kernel/
 * wavefront.cl:1097-1350) are unreachable as wired (MainWindow.cs:284-326 bind
 * the wrong buffers, the GC loop's condition is false on entry, Usages is
 * indexed by block address). This file restates the specification the CUDA
 * path implements, which keeps the reference's records and their meaning:
 *
 *   groups        8-node block groups, one svo_usage each. Tick 0 = free,
 *                 1..65533 = last frame used, 65534 multi-parent, 65535
 *                 inviolate.
 *   dense-real    group g < 8^(B+1) whose level-(B+1) cell has an
 *                 air+geometry base pair: the real level-(B+2) nodes, addressed
 *                 by baseLocation. Never allocated, freed or pruned.
 *   allocatable   every other group below n_groups.
 *   reachable     an allocatable group whose first node is the Child of a node
 *                 in a dense-real or reachable group.
 *   age(t, now)   (now - t) in the wrapping tick space 1..65533.
 *
 * init_usage_tree: dense-real -> {65535, ~0}; reachable -> {tick, parent node}
 *   (the smallest parent address if several); others -> {0, ~0}.
 * gc: stale = allocatable groups with 1 <= tick <= 65533 and age > threshold;
 *   each stale group is detached from its parent node (Child := ~0 when the
 *   parent still points at it); then every allocatable group with a tick in
 *   1..65533 that is no longer reachable is freed ({0, ~0}); the free list is
 *   the ascending list of allocatable groups with tick 0.
 * graft: records in order claim GraftTotalSize groups each from the free list
 *   (skipped, not partially applied, when too few remain); payload group k of a
 *   record becomes claimed group k; children (payload block indices) are
 *   remapped; every claimed group gets {now, parent node or ~0}; the target
 *   node's Child points at the first claimed group.
 * prune: Pruning records (wavefront.cl:24-36, 1215-1266) in order, then a
 *   reachability sweep frees the groups CullChild orphaned.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/svo.h"

#define NONE 0xFFFFFFFFu

static uint32_t pow_sum(int d) {
  uint32_t s = 0, p = 1;
  for (int i = 1; i <= d; i++) s += (p *= 8);
  return s;
}

static int dense_real(const uint16_t *bases, int B, uint32_t g) {
  uint32_t dense_groups = 1u << (3 * (B + 1));
  if (g >= dense_groups) return 0;
  uint16_t chunk = bases[pow_sum(B - 1) + (g >> 3)];
  return ((chunk >> ((g & 7) * 2)) & 3) == 3;
}

/* Marks reachable allocatable groups (reach[g] = 1) and records the smallest
 * parent node address of each. Returns the number reached. */
static uint64_t reach_from_dense(const uint16_t *bases, int B, const svo_block *blocks, size_t n_groups,
                                 uint8_t *reach, uint32_t *parent) {
  uint32_t dense_groups = 1u << (3 * (B + 1));
  memset(reach, 0, n_groups);
  for (size_t g = 0; g < n_groups; g++) parent[g] = NONE;
  uint32_t *stack = (uint32_t *)malloc(sizeof(uint32_t) * (n_groups + 1));
  size_t top = 0;
  uint64_t count = 0;
  for (uint32_t g = 0; g < dense_groups && g < n_groups; g++)
    if (dense_real(bases, B, g)) stack[top++] = g;
  /* depth-first over groups; a group is expanded once */
  uint8_t *expanded = (uint8_t *)calloc(n_groups, 1);
  while (top) {
    uint32_t g = stack[--top];
    if (expanded[g]) continue;
    expanded[g] = 1;
    for (uint32_t i = 0; i < 8; i++) {
      uint32_t node = g * 8 + i;
      uint32_t c = blocks[node].child;
      if (c == NONE || (c & 7) != 0) continue;
      uint32_t h = c >> 3;
      if (h >= n_groups || dense_real(bases, B, h)) continue;
      if (node < parent[h]) parent[h] = node;
      if (!reach[h]) {
        reach[h] = 1;
        count++;
        stack[top++] = h;
      }
    }
  }
  free(expanded);
  free(stack);
  return count;
}

void oracle_init_usage_tree(const uint16_t *bases, int B, const svo_block *blocks, size_t n_groups, svo_usage *usage,
                            uint16_t tick) {
  uint8_t *reach = (uint8_t *)malloc(n_groups);
  uint32_t *parent = (uint32_t *)malloc(sizeof(uint32_t) * n_groups);
  reach_from_dense(bases, B, blocks, n_groups, reach, parent);
  for (size_t g = 0; g < n_groups; g++) {
    usage[g]._pad = 0;
    if (dense_real(bases, B, (uint32_t)g)) {
      usage[g].tick = 65535;
      usage[g].parent = NONE;
    } else if (reach[g]) {
      usage[g].tick = tick;
      usage[g].parent = parent[g];
    } else {
      usage[g].tick = 0;
      usage[g].parent = NONE;
    }
  }
  free(reach);
  free(parent);
}

static uint32_t age(uint32_t t, uint32_t now) { return now >= t ? now - t : now + 65533u - t; }

/* Frees allocatable, allocated (tick 1..65533), unreachable groups; appends
 * them (ascending) to freed. Returns the count. */
static uint64_t sweep(const uint16_t *bases, int B, const svo_block *blocks, size_t n_groups, svo_usage *usage,
                      uint32_t *freed) {
  uint8_t *reach = (uint8_t *)malloc(n_groups);
  uint32_t *parent = (uint32_t *)malloc(sizeof(uint32_t) * n_groups);
  reach_from_dense(bases, B, blocks, n_groups, reach, parent);
  uint64_t n = 0;
  for (size_t g = 0; g < n_groups; g++) {
    if (dense_real(bases, B, (uint32_t)g) || reach[g]) continue;
    if (usage[g].tick >= 1 && usage[g].tick <= 65533) {
      usage[g].tick = 0;
      usage[g].parent = NONE;
      if (freed) freed[n] = (uint32_t)g;
      n++;
    }
  }
  free(reach);
  free(parent);
  return n;
}

/* Block GC. pruned/freed/free_list may be NULL; counts returned in out[3]. */
void oracle_gc(const uint16_t *bases, int B, svo_block *blocks, size_t n_groups, svo_usage *usage, uint16_t now,
               uint32_t threshold, uint32_t *pruned, uint32_t *freed, uint32_t *free_list, uint64_t out[3]) {
  uint64_t np = 0, nf = 0;
  for (size_t g = 0; g < n_groups; g++) {
    if (dense_real(bases, B, (uint32_t)g)) continue;
    uint32_t t = usage[g].tick;
    if (t < 1 || t > 65533 || age(t, now) <= threshold) continue;
    if (pruned) pruned[np] = (uint32_t)g;
    np++;
    uint32_t p = usage[g].parent;
    if (p != NONE && p < n_groups * 8 && blocks[p].child == (uint32_t)g * 8) blocks[p].child = NONE;
  }
  uint64_t nfreed = sweep(bases, B, blocks, n_groups, usage, freed);
  for (size_t g = 0; g < n_groups; g++)
    if (!dense_real(bases, B, (uint32_t)g) && usage[g].tick == 0) {
      if (free_list) free_list[nf] = (uint32_t)g;
      nf++;
    }
  out[0] = np;
  out[1] = nfreed;
  out[2] = nf;
}

/* Walks from level B+2 to `depth` along `loc` (getBlockAddress without the
 * stamps); returns the node or NONE when a node on the way has no child. */
static uint32_t walk(const svo_block *blocks, size_t n_blocks, int B, int depth, const uint64_t loc[3]) {
  uint32_t addr = 0;
  for (int i = 0; i < B + 2; i++) {
    int s = 63 - i;
    addr = (addr << 3) + (uint32_t)(((loc[0] >> s) & 1) | (((loc[1] >> s) & 1) << 1) | (((loc[2] >> s) & 1) << 2));
  }
  for (int d = B + 2; d < depth; d++) {
    if (addr >= n_blocks || blocks[addr].child == NONE) return NONE;
    int s = 63 - d;
    addr = blocks[addr].child +
           (uint32_t)(((loc[0] >> s) & 1) | (((loc[1] >> s) & 1) << 1) | (((loc[2] >> s) & 1) << 2));
  }
  return addr;
}

/* Grafting: claims from free_list (n_free entries) in record order. claimed
 * receives the claimed groups in claim order; applied[r] = 1 if record r was
 * applied. Returns the number of claimed groups. */
uint64_t oracle_graft(int B, svo_block *blocks, size_t n_groups, svo_usage *usage, uint16_t now,
                      const svo_grafting *rec, uint32_t n_rec, const svo_block *payload, size_t n_payload,
                      const uint64_t *locations, size_t n_locations, const uint32_t *free_list, uint64_t n_free,
                      uint32_t *claimed, uint8_t *applied) {
  uint64_t q = 0;
  size_t n_blocks = n_groups * 8;
  for (uint32_t r = 0; r < n_rec; r++) {
    applied[r] = 0;
    uint32_t G = rec[r].graft_total_size, P = rec[r].graft_data_address;
    if (G == 0 || (P & 7) || (uint64_t)P + 8ull * G > n_payload) continue;
    if (q + G > n_free) continue;
    uint32_t target;
    if (rec[r].depth == 255) {
      target = rec[r].graft_address;
    } else {
      if ((uint64_t)rec[r].graft_address * 3 + 3 > n_locations) continue;
      target = walk(blocks, n_blocks, B, rec[r].depth, locations + 3ull * rec[r].graft_address);
    }
    if (target == NONE || target >= n_blocks) continue;
    const uint32_t *C = free_list + q;
    for (uint32_t k = 0; k < G; k++) {
      usage[C[k]].tick = now;
      usage[C[k]].parent = NONE;
      usage[C[k]]._pad = 0;
    }
    for (uint32_t k = 0; k < G; k++)
      for (uint32_t i = 0; i < 8; i++) {
        svo_block b = payload[P + 8 * k + i];
        uint32_t node = C[k] * 8 + i;
        uint32_t c = b.child;
        if (c != NONE) {
          uint32_t rel = c - P;
          if (c < P || (rel & 7) || rel / 8 >= G) {
            b.child = NONE;
          } else {
            uint32_t h = C[rel / 8];
            b.child = h * 8;
            if (node < usage[h].parent) usage[h].parent = node; /* smallest referencing node */
          }
        }
        blocks[node] = b;
      }
    usage[C[0]].parent = target;
    blocks[target].child = C[0] * 8;
    for (uint32_t k = 0; k < G; k++) claimed[q + k] = C[k];
    q += G;
    applied[r] = 1;
  }
  return q;
}

/* Pruning records (wavefront.cl:1215-1266) in order; child requests of
 * missing paths are appended to req (count in *n_req); orphans are freed and
 * listed in freed (count returned). */
uint64_t oracle_prune(uint16_t *bases, size_t n_bases, int B, svo_block *blocks, size_t n_groups, svo_usage *usage,
                      uint16_t now, const svo_pruning *rec, uint32_t n_rec, const svo_block *surface,
                      size_t n_surface, const uint64_t *locations, size_t n_locations, svo_child_request *req,
                      uint32_t req_cap, uint32_t *n_req, uint32_t *freed) {
  size_t n_blocks = n_groups * 8;
  int culled = 0;
  for (uint32_t r = 0; r < n_rec; r++) {
    const svo_pruning *p = &rec[r];
    uint32_t address = p->address;
    if ((p->properties >> 4) & 1) { /* BaseBlock */
      if (address < n_bases) bases[address] = p->chunk;
      continue;
    }
    if (p->depth != 255) { /* findAddress, wavefront.cl:1191-1211 */
      if ((uint64_t)address * 3 + 3 > n_locations) continue;
      const uint64_t *loc = locations + 3ull * address;
      uint32_t a = 0;
      for (int i = 0; i < B + 2; i++) {
        int s = 63 - i;
        a = (a << 3) + (uint32_t)(((loc[0] >> s) & 1) | (((loc[1] >> s) & 1) << 1) | (((loc[2] >> s) & 1) << 2));
      }
      int missing = 0;
      for (int i = B + 2; i < p->depth; i++) {
        if (a >= n_blocks) {
          missing = 1;
          break;
        }
        if ((a >> 3) < n_groups && usage[a >> 3].tick < 65534) usage[a >> 3].tick = now;
        if (blocks[a].child == NONE) {
          uint32_t slot = (*n_req)++;
          if (req && slot < req_cap) {
            svo_child_request *q = &req[slot];
            memset(q, 0, sizeof(*q));
            q->address = a;
            q->tick = now;
            q->depth = (uint8_t)i;
            q->location[0] = loc[0];
            q->location[1] = loc[1];
            q->location[2] = loc[2];
            q->tree_size = (uint8_t)(p->depth - i);
          }
          missing = 1;
          break;
        }
        int s = 63 - i;
        a = blocks[a].child +
            (uint32_t)(((loc[0] >> s) & 1) | (((loc[1] >> s) & 1) << 1) | (((loc[2] >> s) & 1) << 2));
      }
      if (missing) continue;
      address = a;
    } else {
      if (address >= n_blocks || usage[address >> 3].tick == 0) continue; /* dereferenced */
      if (usage[address >> 3].tick < 65534) usage[address >> 3].tick = now;
    }
    if (address >= n_blocks) continue;
    if (p->properties & 1) { /* CullChild */
      blocks[address].child = p->child_address;
      culled = 1;
    }
    uint32_t v = (p->properties >> 1) & 3; /* AlterViolability, MakeInviolate */
    if (v == 3)
      usage[address >> 3].tick = 65535;
    else if (v == 1)
      usage[address >> 3].tick = now;
    if ((p->properties >> 3) & 1) { /* UpdateChunk */
      if (p->colour_address < n_surface) blocks[address] = surface[p->colour_address];
      blocks[address].chunk = p->chunk;
    }
  }
  if (!culled) return 0;
  return sweep(bases, B, blocks, n_groups, usage, freed);
}
