/*
 * svo_oracle.c -- TEST INFRASTRUCTURE ONLY: the parity checker of the CUDA
 * tracer. Not linked into, loaded by or called from the product.
 *
 * A plain-C restatement of the reference's wavefront cone tracer hot path
 * (SvoTracer/SvoTracer.Kernel/wavefront.cl). The reference runs every ray as a
 * sequence of queued kernel launches; each ray's state transitions depend only
 * on that ray and the (read-only during a trace) octree, and the per-pixel
 * accumulation is a commutative integer sum, so this file runs each ray's
 * state machine to completion, one ray at a time. The results are the ones
 * the queued passes produce in any order.
 *
 * Numerics (the parity contract for OpenCL's implementation-defined
 * built-ins): every float operation is a single IEEE round-to-nearest
 * operation in source order, built with -ffp-contract=off; native_divide is a
 * correctly rounded division; native_sin/cos of the ray setup are the
 * per-column/per-row tables (float)sin((double)angle); fast_length is
 * sqrtf((x*x + y*y) + z*z); and every comparison of ConeDepth = -half_log2(c)
 * with an integer k is evaluated exactly as a comparison of c with 2^-k, so no
 * logarithm is evaluated. Float-to-integer conversions that the reference
 * leaves undefined (out of range, NaN) saturate (NaN -> 0).
 */
#include "svo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ULMAX 0xFFFFFFFFFFFFFFFFull

/* wavefront.cl:200-207 floatToUlong. 0.999999911f is the float 1 - 2^-24. */
uint64_t oracle_float_to_ulong(float x) {
  if (x >= 0.999999911f) return ULMAX;
  float v = fabsf(x) * 18446744073709551616.0f; /* (float)ULONG_MAX == 2^64 */
  if (v != v) return 0;
  if (!(v < 18446744073709551616.0f)) return ULMAX;
  return (uint64_t)v;
}

/* wavefront.cl:209 ulongToFloat: (float)x / 2^64, exact scaling. */
float oracle_ulong_to_float(uint64_t x) { return (float)x / 18446744073709551616.0f; }

/* wavefront.cl:211-221 roundUlong: distance to the next level-(depth+1)
 * boundary in the travel direction. */
uint64_t oracle_round_ulong(uint64_t value, uint8_t depth, int round_up) {
  uint64_t mask = ULMAX - (ULMAX >> (depth + 1));
  if (round_up) return ((value & mask) + ((ULMAX - (ULMAX >> 1)) >> depth)) - value;
  uint64_t output = value - ((value & mask) - 1);
  if (output >= value) return value;
  return output;
}

/* wavefront.cl:224 powSum: sum of 8^i for i = 1..depth. */
uint32_t oracle_pow_sum(uint8_t depth) {
  uint32_t s = 0, p = 1;
  for (int i = 1; i <= depth; i++) {
    p *= 8;
    s += p;
  }
  return s;
}

/* wavefront.cl:428-430 chunkPosition: child octant below level `depth`. */
uint8_t oracle_chunk_position(uint8_t depth, const uint64_t loc[3]) {
  int s = 64 - depth - 1;
  return (uint8_t)(((loc[0] >> s) & 1) + (((loc[1] >> s) & 1) << 1) + (((loc[2] >> s) & 1) << 2));
}

/* wavefront.cl:405-411 baseLocation: dense index of the level-`depth` cell. */
uint32_t oracle_base_location(uint8_t depth, const uint64_t loc[3]) {
  uint32_t out = 0;
  for (uint8_t i = 0; i < depth; i++) out = (out << 3) + oracle_chunk_position(i, loc);
  return out;
}

/* wavefront.cl:440-497 traverseChunk (without the trailing setConeDepth,
 * whose value is recomputed where it is read). */
void oracle_traverse_chunk(uint8_t depth, const float dir[3], const float inv[3], const int sign[3], uint64_t loc[3]) {
  uint64_t d[3];
  float a[3];
  for (int k = 0; k < 3; k++) {
    d[k] = oracle_round_ulong(loc[k], depth, sign[k]);
    a[k] = fabsf((float)d[k] * inv[k]);
  }
  if (a[0] <= a[1] && a[0] <= a[2]) {
    float u = oracle_ulong_to_float(d[0]);
    d[1] = oracle_float_to_ulong(dir[1] * inv[0] * u);
    d[2] = oracle_float_to_ulong(dir[2] * inv[0] * u);
  } else if (a[1] <= a[0] && a[1] <= a[2]) {
    float u = oracle_ulong_to_float(d[1]);
    d[0] = oracle_float_to_ulong(dir[0] * inv[1] * u);
    d[2] = oracle_float_to_ulong(dir[2] * inv[1] * u);
  } else {
    float u = oracle_ulong_to_float(d[2]);
    d[0] = oracle_float_to_ulong(dir[0] * inv[2] * u);
    d[1] = oracle_float_to_ulong(dir[1] * inv[2] * u);
  }
  for (int k = 0; k < 3; k++) {
    if (sign[k])
      loc[k] += d[k];
    else
      loc[k] -= d[k];
  }
  for (int k = 0; k < 3; k++) {
    if (sign[k] && loc[k] == 0)
      loc[k] = ULMAX;
    else if (!sign[k] && loc[k] == ULMAX)
      loc[k] = 0;
  }
}

/* wavefront.cl:413-426 comparePositions: pop while the step left the cell. */
uint8_t oracle_compare_positions(uint8_t depth, const uint64_t prev[3], const uint64_t loc[3], const int sign[3]) {
  for (;;) {
    uint8_t np = oracle_chunk_position(depth, loc);
    uint8_t pp = oracle_chunk_position(depth, prev);
    int left = 0;
    for (int k = 0; k < 3; k++) {
      int pb = (pp >> k) & 1, nb = (np >> k) & 1;
      if (pb == sign[k] && nb != sign[k]) left = 1;
    }
    if (!left) return depth;
    if (depth == 1) return depth;
    depth--;
  }
}

/* wavefront.cl:433-437 leaving. */
static int leaving(const uint64_t loc[3], const int sign[3]) {
  for (int k = 0; k < 3; k++) {
    if (!sign[k] && loc[k] == 0) return 1;
    if (sign[k] && loc[k] == ULMAX) return 1;
  }
  return 0;
}

/* wavefront.cl:387-391 coneSize, max() as "y if x < y else x". */
static float cone_size(float m, float fov, const float dof[2]) {
  float eye = fov * m;
  float f = fabsf(dof[0] * (dof[1] - m));
  return eye < f ? f : eye;
}

/* wavefront.cl:394-399 setConeDepth's distance: fast_length(Origin - Location). */
static float cone_distance(const float origin[3], const uint64_t loc[3]) {
  float x = origin[0] - oracle_ulong_to_float(loc[0]);
  float y = origin[1] - oracle_ulong_to_float(loc[1]);
  float z = origin[2] - oracle_ulong_to_float(loc[2]);
  return fabsf(sqrtf(x * x + y * y + z * z));
}

/* 2^-k as a float (k <= 126). */
static float pow2_neg(int k) { return ldexpf(1.0f, -k); }

/* wavefront.cl:639-1088 traceIntoVolume. The 27-way switch picks, among the
 * axes whose slab the origin is outside of, the one with the largest entry
 * distance (ties to x, then y), enters the cube on that face and rejects the
 * ray when the entry point lies outside the cube grown by the cone size. */
int oracle_trace_into_volume(const float o[3], const float dir[3], const float inv[3], float fov, const float dof[2],
                             uint64_t loc[3]) {
  int lo[3], hi[3];
  int any = 0;
  for (int k = 0; k < 3; k++) {
    lo[k] = o[k] < 0;
    hi[k] = o[k] > 1;
    any |= lo[k] | hi[k];
  }
  if (!any) {
    for (int k = 0; k < 3; k++) loc[k] = oracle_float_to_ulong(o[k]);
    return 1;
  }
  for (int k = 0; k < 3; k++)
    if ((lo[k] | hi[k]) && dir[k] == 0) return 0;
  for (int k = 0; k < 3; k++) {
    int pos = dir[k] >= 0;
    if (lo[k] && !pos) return 0;
    if (hi[k] && pos) return 0;
  }
  float mk[3] = {0, 0, 0};
  int out[3], n = 0;
  for (int k = 0; k < 3; k++) {
    if (lo[k] | hi[k]) {
      float bound = hi[k] ? 1.0f : 0.0f;
      mk[k] = fabsf((bound - o[k]) * inv[k]);
      out[n++] = k;
    }
  }
  int axis;
  if (n == 1) {
    axis = out[0];
  } else if (n == 2) {
    axis = mk[out[0]] >= mk[out[1]] ? out[0] : out[1];
  } else {
    if (mk[0] >= mk[1] && mk[0] >= mk[2])
      axis = 0;
    else if (mk[1] >= mk[0] && mk[1] >= mk[2])
      axis = 1;
    else
      axis = 2;
  }
  float m = mk[axis];
  float p[3];
  for (int k = 0; k < 3; k++) {
    if (k == axis)
      p[k] = hi[k] ? 1.0f : 0.0f;
    else
      p[k] = o[k] + (dir[k] * m);
  }
  for (int k = 0; k < 3; k++) loc[k] = oracle_float_to_ulong(p[k]);
  float c = cone_size(m, fov, dof);
  for (int k = 0; k < 3; k++)
    if (p[k] < -c || p[k] > 1 + c) return 0;
  return 1;
}

void oracle_view_tables(const svo_trace_input *in, float *sin_u, float *cos_u, float *sin_v, float *cos_v) {
  float w = (float)in->screen_size[0], h = (float)in->screen_size[1];
  /* wavefront.cl:566-572 */
  for (uint32_t x = 0; x < in->screen_size[0]; x++) {
    float u = in->fov[0] * ((w / 2.0f - (float)x) / w);
    sin_u[x] = (float)sin((double)u);
    cos_u[x] = (float)cos((double)u);
  }
  for (uint32_t y = 0; y < in->screen_size[1]; y++) {
    float v = in->fov[1] * ((h / 2.0f - (float)y) / h);
    sin_v[y] = (float)sin((double)v);
    cos_v[y] = (float)cos((double)v);
  }
}

static const svo_block zero_block;

static const svo_block *node_at(const svo_block *blocks, size_t n_blocks, uint32_t addr) {
  return addr < n_blocks ? &blocks[addr] : &zero_block;
}

/* wavefront.cl:296-304 getBlockAddress; *reads counts the node loads of the
 * walk plus the load of the returned node. */
static uint32_t block_address(const svo_block *blocks, size_t n_blocks, uint8_t base_depth, uint8_t depth,
                              const uint64_t loc[3], uint32_t *reads) {
  uint32_t addr = oracle_base_location((uint8_t)(base_depth + 2), loc);
  for (uint8_t d = (uint8_t)(base_depth + 2); d < depth; d++) {
    addr = node_at(blocks, n_blocks, addr)->child + oracle_chunk_position(d, loc);
    (*reads)++;
  }
  (*reads)++;
  return addr;
}

static uint8_t sat_u8(float v) {
  if (v != v) return 0;
  if (v <= 0.0f) return 0;
  if (v >= 255.0f) return 255;
  return (uint8_t)v;
}

void oracle_init_usage(const uint16_t *bases, uint8_t base_depth, svo_usage *usage, size_t n_groups) {
  /* MainWindow.cs:129-141: entries [0, 8^B) look at the level-B base chunk of
   * the same index and become inviolate when one of its low four octants is
   * both air and geometry (j = 3, 12, 48, 192). */
  memset(usage, 0, n_groups * sizeof(svo_usage));
  uint32_t base_start = oracle_pow_sum((uint8_t)(base_depth - 1));
  uint32_t range = oracle_pow_sum(base_depth);
  for (uint32_t i = 0; i < range - base_start && i < n_groups; i++)
    for (uint32_t j = 3; j <= 255; j <<= 2)
      if ((bases[i + base_start] & j) == j) {
        usage[i].tick = 65535;
        usage[i].parent = 0xFFFFFFFFu;
        break;
      }
}

typedef struct ray_result {
  uint32_t hit_index;
  uint8_t hit_depth;
  float t;
  uint32_t acc[4];
  uint32_t v_block, v_base, steps;
  int step_limited;
  int requested; /* the ray stopped with a child request (at most one per ray) */
  svo_child_request request;
  float dir[3];  /* setupInitialTrace's direction */
} ray_result;

static void trace_ray(const uint16_t *bases, uint8_t B, const svo_block *blocks, size_t n_blocks, svo_usage *usage,
                      size_t n_groups, const svo_trace_input *in, const float *su, const float *cu, const float *sv,
                      const float *cv, uint32_t px, uint32_t py, int32_t max_steps, svo_child_request *req,
                      uint32_t req_cap, uint32_t *n_req, ray_result *r) {
  memset(r, 0, sizeof(*r));
  r->hit_index = SVO_MISS;
  r->t = INFINITY;
  /* setupInitialTrace, wavefront.cl:563-595 */
  float m0 = cu[px] * cv[py];
  float m1 = (0.0f - su[px]) * cv[py];
  float m2 = sv[py];
  const float *F = in->facing;
  float dir[3], inv[3], o[3];
  int sign[3];
  dir[0] = F[0] * m0 + F[3] * m1 + F[6] * m2;
  dir[1] = F[1] * m0 + F[4] * m1 + F[7] * m2;
  dir[2] = F[2] * m0 + F[5] * m1 + F[8] * m2;
  for (int k = 0; k < 3; k++) {
    r->dir[k] = dir[k];
    inv[k] = 1.0f / dir[k];
    sign[k] = dir[k] >= 0;
    o[k] = in->origin[k];
  }
  float fov = in->fov[0] / (float)in->screen_size[0];
  const float zero_dof[2] = {0.0f, 0.0f};
  uint64_t loc[3];
  int background = 1;
  uint8_t depth = 1;
  int hit = 0;
  /* init, wavefront.cl:1376-1384: enter the cube or go to the background queue. */
  if (oracle_trace_into_volume(o, dir, inv, fov, zero_dof, loc)) {
    background = 0;
    for (;;) {
      if (max_steps > 0 && (int32_t)r->steps >= max_steps) {
        r->step_limited = 1;
        background = 1;
        break;
      }
      r->steps++;
      if (depth <= B) {
        /* runBaseTrace, wavefront.cl:1400-1463 */
        uint16_t chunk = bases[oracle_pow_sum((uint8_t)(depth - 1)) + oracle_base_location(depth, loc)];
        r->v_base++;
        if (((chunk >> (oracle_chunk_position(depth, loc) * 2)) & 2) != 2) {
          uint64_t prev[3] = {loc[0], loc[1], loc[2]};
          oracle_traverse_chunk(depth, dir, inv, sign, loc);
          if (leaving(loc, sign)) {
            background = 1;
            break;
          }
          depth = oracle_compare_positions(depth, prev, loc, sign);
        } else {
          depth = depth < B ? (uint8_t)(depth + 1) : (uint8_t)(B + 2);
          if (depth == B + 1) depth = B;
        }
        continue;
      }
      /* runBlockTrace, wavefront.cl:1465-1566 */
      uint32_t addr = block_address(blocks, n_blocks, B, depth, loc, &r->v_block);
      const svo_block *blk = node_at(blocks, n_blocks, addr);
      if (usage && (addr >> 3) < n_groups) {
        svo_usage *u = &usage[addr >> 3];
        if (u->tick < 65534 && u->tick != in->tick) u->tick = in->tick;
      }
      int complete = 0;
      if (((blk->chunk >> (oracle_chunk_position(depth, loc) * 2)) & 2) != 2) {
        uint64_t prev[3] = {loc[0], loc[1], loc[2]};
        oracle_traverse_chunk(depth, dir, inv, sign, loc);
        if (leaving(loc, sign)) {
          background = 1;
          break;
        }
        depth = oracle_compare_positions(depth, prev, loc, sign);
      } else {
        /* ConeDepth = -half_log2(c): "ConeDepth < k" <=> c > 2^-k,
         * "ConeDepth > k" <=> c < 2^-k. */
        float c = cone_size(cone_distance(o, loc), fov, in->dof);
        if (c > pow2_neg(B + 2)) {
          depth = (uint8_t)(B + 2);
          complete = 1;
        } else if (c > pow2_neg(depth)) {
          depth--;
        } else if (blk->child == SVO_NO_CHILD) {
          /* requestChild, wavefront.cl:362-375 with the call of :1539.
           * TreeSize = min(1, (uchar)ConeDepth - Depth) is 1 exactly when
           * ConeDepth >= Depth + 1; Tick is the unset TraceData.Tick (0). */
          svo_child_request *q = &r->request;
          memset(q, 0, sizeof(*q));
          q->address = addr;
          q->tick = 0;
          q->depth = depth;
          q->location[0] = loc[0];
          q->location[1] = loc[1];
          q->location[2] = loc[2];
          q->tree_size = c <= pow2_neg(depth + 1) ? 1 : 0;
          r->requested = 1;
          uint32_t slot;
#ifdef _OPENMP
#pragma omp atomic capture
#endif
          slot = (*n_req)++;
          if (req && slot < req_cap) req[slot] = *q;
          complete = 1;
        } else if (c < pow2_neg(depth + 1)) {
          depth++;
        } else {
          complete = 1;
        }
      }
      if (complete) {
        hit = 1;
        break;
      }
      if (depth == B + 1) depth = B;
    }
  }
  if (hit) {
    /* resolveRemainders, wavefront.cl:1799-1833 */
    uint32_t addr = block_address(blocks, n_blocks, B, depth, loc, &r->v_block);
    const svo_block *blk = node_at(blocks, n_blocks, addr);
    r->hit_index = addr;
    r->hit_depth = depth;
    r->acc[0] = 255;
    r->acc[1] = (uint32_t)blk->colour_r * 255u;
    r->acc[2] = (uint32_t)blk->colour_g * 255u;
    r->acc[3] = (uint32_t)blk->colour_b * 255u;
    /* hit distance as kernel.cl's resolveRayData: length(Location - Origin) */
    float x = oracle_ulong_to_float(loc[0]) - o[0];
    float y = oracle_ulong_to_float(loc[1]) - o[1];
    float z = oracle_ulong_to_float(loc[2]) - o[2];
    r->t = sqrtf(x * x + y * y + z * z);
  } else if (background) {
    /* evaluateBackground, wavefront.cl:1741-1797, for a primary ray
     * (Weighting 255, so the ambient blend does not apply). */
    float dotp = dir[0] * 0.0f + dir[1] * 0.0f + dir[2] * -1.0f;
    uint32_t cr, cg, cb;
    uint8_t lum;
    if (dotp > 0.8f) {
      cr = cg = cb = 255;
      lum = sat_u8(dotp * 200.0f);
    } else {
      cr = 135;
      cg = 206;
      cb = 235;
      lum = 1;
    }
    r->acc[0] = 255;
    if (lum > 0) {
      r->acc[1] = cr * 255u;
      r->acc[2] = cg * 255u;
      r->acc[3] = cb * 255u;
    }
  }
}

int64_t oracle_trace_view(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                          svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                          const oracle_view_out *out, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                          int32_t threads) {
  return oracle_trace_rows_gi(bases, base_depth, blocks, n_blocks, usage, n_groups, in, max_steps, out, req, req_cap,
                              n_req, threads, 0, in->screen_size[1], 0);
}

int64_t oracle_trace_rows(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                          svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                          const oracle_view_out *out, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                          int32_t threads, uint32_t row_begin, uint32_t row_end) {
  return oracle_trace_rows_gi(bases, base_depth, blocks, n_blocks, usage, n_groups, in, max_steps, out, req, req_cap,
                              n_req, threads, row_begin, row_end, 0);
}

typedef struct mega_schedule mega_schedule;
static int gi_schedule(const svo_trace_input *in, mega_schedule **S);
static void gi_free_schedule(mega_schedule *S);
static void gi_pixel(const svo_block *blk, const float dir[3], const svo_trace_input *in, const mega_schedule *S,
                     uint32_t acc[4]);

int64_t oracle_trace_rows_gi(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                             svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                             const oracle_view_out *out, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                             int32_t threads, uint32_t row_begin, uint32_t row_end, int32_t gi) {
  uint32_t W = in->screen_size[0], H = in->screen_size[1];
  /* the material stage: evaluateMaterial returns at once for unusable cone
   * parameters (wavefront.cl:1575-1576); a schedule whose loops would not end is
   * refused (-2) */
  const int gi_valid = gi && !(in->fov_constant <= 0 || in->fov_multiplier >= 1 || in->fov_multiplier <= -1);
  mega_schedule *S = NULL;
  if (gi_valid && !gi_schedule(in, &S)) return -2;
  if (row_end > H) row_end = H;
  if (row_begin > row_end) row_begin = row_end;
  float *su = (float *)malloc(sizeof(float) * (W + 1));
  float *cu = (float *)malloc(sizeof(float) * (W + 1));
  float *sv = (float *)malloc(sizeof(float) * (H + 1));
  float *cv = (float *)malloc(sizeof(float) * (H + 1));
  oracle_view_tables(in, su, cu, sv, cv);
  int64_t limited = 0;
  int64_t n = (int64_t)W * (row_end - row_begin);
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt) reduction(+ : limited)
#endif
  for (int64_t id = 0; id < n; id++) {
    ray_result r;
    trace_ray(bases, base_depth, blocks, n_blocks, usage, n_groups, in, su, cu, sv, cv, (uint32_t)(id % W),
              row_begin + (uint32_t)(id / W), max_steps, req, req_cap, n_req, &r);
    limited += r.step_limited;
    if (out->hit_index) out->hit_index[id] = r.hit_index;
    if (out->hit_depth) out->hit_depth[id] = r.hit_depth;
    if (out->t) out->t[id] = r.t;
    if (out->acc)
      for (int k = 0; k < 4; k++) out->acc[4 * id + k] = r.acc[k];
    if (out->v_block) out->v_block[id] = r.v_block;
    if (out->v_base) out->v_base[id] = r.v_base;
    if (out->steps) out->steps[id] = r.steps;
    if (out->requested) out->requested[id] = (uint8_t)r.requested;
    if (out->pixel_request && r.requested) out->pixel_request[id] = r.request;
    if (gi && r.hit_index != SVO_MISS) {
      /* the secondary-cone stage replaces a hit's accumulators (resolveRemainders
       * then finds the material queue empty) and stamps the hit block's usage */
      if (gi_valid) {
        uint32_t g = r.hit_index >> 3;
        if (usage && g < n_groups && usage[g].tick < 65534 && usage[g].tick != in->tick) usage[g].tick = in->tick;
        gi_pixel(node_at(blocks, n_blocks, r.hit_index), r.dir, in, S, r.acc);
      } else {
        r.acc[0] = r.acc[1] = r.acc[2] = r.acc[3] = 0;
      }
      if (out->acc)
        for (int k = 0; k < 4; k++) out->acc[4 * id + k] = r.acc[k];
    }
    if (out->rgba) {
      /* drawTrace, wavefront.cl:1835-1850 */
      float *px = &out->rgba[4 * id];
      if (r.acc[0] == 0) {
        px[0] = 0.75f;
        px[1] = 0.0f;
        px[2] = 0.0f;
        px[3] = 1.0f;
      } else {
        float fw = (float)r.acc[0] * 255.0f;
        px[0] = fminf((float)r.acc[1] / fw, 1.0f);
        px[1] = fminf((float)r.acc[2] / fw, 1.0f);
        px[2] = fminf((float)r.acc[3] / fw, 1.0f);
        px[3] = 1.0f;
      }
    }
  }
  free(su);
  free(cu);
  free(sv);
  free(cv);
  if (S) gi_free_schedule(S);
  return limited;
}


/* ---- differentiable forward model: LOD hit lists ------------------------- */

/* For each ray of the view: the sequence of LOD hit nodes (up to max_hits),
 * continuing past every hit as if its octant were empty (the traversal of
 * svo_diff_forward), whether the ray ended by leaving the cube (then the sky
 * colour contributes) and that sky colour (drawTrace's float of c/255). */
void oracle_hit_lists(const uint16_t *bases, uint8_t B, const svo_block *blocks, size_t n_blocks,
                      const svo_trace_input *in, int32_t max_steps, int32_t max_hits, uint32_t *hits, uint8_t *n_hits,
                      uint8_t *leaves, float *sky, int32_t threads) {
  uint32_t W = in->screen_size[0], H = in->screen_size[1];
  float *su = (float *)malloc(sizeof(float) * (W + 1));
  float *cu = (float *)malloc(sizeof(float) * (W + 1));
  float *sv = (float *)malloc(sizeof(float) * (H + 1));
  float *cv = (float *)malloc(sizeof(float) * (H + 1));
  oracle_view_tables(in, su, cu, sv, cv);
  int64_t n = (int64_t)W * H;
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
  for (int64_t id = 0; id < n; id++) {
    uint32_t px = (uint32_t)(id % W), py = (uint32_t)(id / W);
    float m0 = cu[px] * cv[py], m1 = (0.0f - su[px]) * cv[py], m2 = sv[py];
    const float *F = in->facing;
    float dir[3], inv[3], o[3];
    int sign[3];
    dir[0] = F[0] * m0 + F[3] * m1 + F[6] * m2;
    dir[1] = F[1] * m0 + F[4] * m1 + F[7] * m2;
    dir[2] = F[2] * m0 + F[5] * m1 + F[8] * m2;
    for (int k = 0; k < 3; k++) {
      inv[k] = 1.0f / dir[k];
      sign[k] = dir[k] >= 0;
      o[k] = in->origin[k];
    }
    float fov = in->fov[0] / (float)in->screen_size[0];
    const float zero_dof[2] = {0.0f, 0.0f};
    uint64_t loc[3];
    int nh = 0, leave = 0, steps = 0;
    uint32_t reads = 0;
    uint8_t depth = 1;
    if (!oracle_trace_into_volume(o, dir, inv, fov, zero_dof, loc)) {
      leave = 1;
    } else {
      for (;;) {
        if (max_steps > 0 && steps >= max_steps) {
          leave = 1;
          break;
        }
        steps++;
        int occupied, block = depth > B, hit = 0;
        uint32_t addr = 0;
        const svo_block *blk = &zero_block;
        if (!block) {
          uint16_t chunk = bases[oracle_pow_sum((uint8_t)(depth - 1)) + oracle_base_location(depth, loc)];
          occupied = ((chunk >> (oracle_chunk_position(depth, loc) * 2)) & 2) == 2;
        } else {
          addr = block_address(blocks, n_blocks, B, depth, loc, &reads);
          blk = node_at(blocks, n_blocks, addr);
          occupied = ((blk->chunk >> (oracle_chunk_position(depth, loc) * 2)) & 2) == 2;
        }
        if (occupied && !block) {
          depth = depth < B ? (uint8_t)(depth + 1) : (uint8_t)(B + 2);
          continue;
        }
        if (occupied) {
          float c = cone_size(cone_distance(o, loc), fov, in->dof);
          if (c > pow2_neg(B + 2)) {
            depth = (uint8_t)(B + 2);
            hit = 1;
          } else if (c > pow2_neg(depth)) {
            depth--;
            if (depth == B + 1) depth = B;
            continue;
          } else if (blk->child == SVO_NO_CHILD) {
            hit = 1;
          } else if (c < pow2_neg(depth + 1)) {
            depth++;
            continue;
          } else {
            hit = 1;
          }
          if (hit) {
            hits[id * max_hits + nh] = block_address(blocks, n_blocks, B, depth, loc, &reads);
            if (++nh >= max_hits) break;
          }
        }
        /* empty octant, or stepping past a hit */
        uint64_t prev[3] = {loc[0], loc[1], loc[2]};
        oracle_traverse_chunk(depth, dir, inv, sign, loc);
        if (leaving(loc, sign)) {
          leave = 1;
          break;
        }
        depth = oracle_compare_positions(depth, prev, loc, sign);
        if (depth == B + 1) depth = B;
      }
    }
    n_hits[id] = (uint8_t)nh;
    leaves[id] = (uint8_t)leave;
    float dotp = dir[0] * 0.0f + dir[1] * 0.0f + dir[2] * -1.0f;
    uint32_t cr = 135, cg = 206, cb = 235;
    if (dotp > 0.8f) cr = cg = cb = 255;
    sky[3 * id + 0] = (float)(cr * 255u) / 65025.0f;
    sky[3 * id + 1] = (float)(cg * 255u) / 65025.0f;
    sky[3 * id + 2] = (float)(cb * 255u) / 65025.0f;
  }
  free(su);
  free(cu);
  free(sv);
  free(cv);
}

/* FP64 compositing over hit lists: colour, loss sum((C - target)^2) / rays and,
 * if grad != NULL, its gradient with respect to the per-node RGBA (4 doubles
 * per node, accumulated). rgb (3 doubles per ray) may be NULL. */
double oracle_diff_eval(const uint32_t *hits, const uint8_t *n_hits, const uint8_t *leaves, const float *sky,
                        int64_t n_rays, int32_t max_hits, const double *params, const double *target, double *rgb,
                        double *grad, int32_t threads) {
  double loss = 0.0;
  double inv_n = 1.0 / (double)n_rays;
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt) reduction(+ : loss)
#endif
  for (int64_t r = 0; r < n_rays; r++) {
    const uint32_t *h = hits + r * max_hits;
    double C[3] = {0, 0, 0}, T = 1.0;
    for (int i = 0; i < n_hits[r]; i++) {
      const double *p = params + 4ull * h[i];
      for (int k = 0; k < 3; k++) C[k] += T * p[3] * p[k];
      T *= 1.0 - p[3];
    }
    if (leaves[r])
      for (int k = 0; k < 3; k++) C[k] += T * (double)sky[3 * r + k];
    double G[3];
    for (int k = 0; k < 3; k++) {
      double e = C[k] - (target ? target[3 * r + k] : 0.0);
      loss += e * e * inv_n;
      G[k] = 2.0 * e * inv_n;
      if (rgb) rgb[3 * r + k] = C[k];
    }
    if (!grad) continue;
    double S[3] = {0, 0, 0};
    T = 1.0;
    for (int i = 0; i < n_hits[r]; i++) {
      const double *p = params + 4ull * h[i];
      double *g = grad + 4ull * h[i];
      double a = p[3], ta = T * a, da = 0.0;
      for (int k = 0; k < 3; k++) {
        S[k] += ta * p[k];
        double behind = C[k] - S[k];
        da += G[k] * (T * p[k] - (1.0 - a > 0.0 ? behind / (1.0 - a) : 0.0));
        double gk = ta * G[k];
#ifdef _OPENMP
#pragma omp atomic
#endif
        g[k] += gk;
      }
#ifdef _OPENMP
#pragma omp atomic
#endif
      g[3] += da;
      T *= 1.0 - a;
    }
  }
  return loss;
}

/* FP64 central finite differences of the loss of oracle_diff_eval with respect
 * to the 4 parameters of each node in `nodes` (step h). Only the rays whose hit
 * list holds the node change with its parameters, so each difference is summed
 * over those rays alone; nodes[] must be sorted ascending and fd receives 4
 * doubles per listed node. */
void oracle_diff_fd(const uint32_t *hits, const uint8_t *n_hits, const uint8_t *leaves, const float *sky,
                    int64_t n_rays, int32_t max_hits, const double *params, const double *target, const uint32_t *nodes,
                    int32_t n_nodes, double h, double *fd, int32_t threads) {
  double inv_n = 1.0 / (double)n_rays;
  memset(fd, 0, sizeof(double) * 4 * (size_t)n_nodes);
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
  for (int64_t r = 0; r < n_rays; r++) {
    const uint32_t *hl = hits + r * max_hits;
    for (int i0 = 0; i0 < n_hits[r]; i0++) {
      /* nodes[] is sorted ascending; each listed node is differenced once per ray */
      int32_t lo = 0, hi = n_nodes;
      while (lo < hi) {
        int32_t mid = (lo + hi) / 2;
        if (nodes[mid] < hl[i0])
          lo = mid + 1;
        else
          hi = mid;
      }
      if (lo >= n_nodes || nodes[lo] != hl[i0]) continue;
      int seen = 0;
      for (int i = 0; i < i0; i++) seen |= hl[i] == hl[i0];
      if (seen) continue;
      int32_t j = lo;
      for (int ch = 0; ch < 4; ch++) {
        double side[2];
        for (int sgn = 0; sgn < 2; sgn++) {
          double delta = sgn ? -h : h;
          double C[3] = {0, 0, 0}, T = 1.0;
          for (int i = 0; i < n_hits[r]; i++) {
            double p[4];
            for (int k = 0; k < 4; k++) p[k] = params[4ull * hl[i] + k];
            if (hl[i] == nodes[j]) p[ch] += delta;
            for (int k = 0; k < 3; k++) C[k] += T * p[3] * p[k];
            T *= 1.0 - p[3];
          }
          if (leaves[r])
            for (int k = 0; k < 3; k++) C[k] += T * (double)sky[3 * r + k];
          double l = 0.0;
          for (int k = 0; k < 3; k++) {
            double e = C[k] - target[3 * r + k];
            l += e * e * inv_n;
          }
          side[sgn] = l;
        }
        double v = (side[0] - side[1]) / (2.0 * h);
#ifdef _OPENMP
#pragma omp atomic
#endif
        fd[4 * j + ch] += v;
      }
    }
  }
}


/* ---- megakernel: kernel.cl's `trace` (kernel.cl:1531-1558) ----------------
 *
 * One work-item per pixel: the primary cone (the same fixed-point traversal as
 * the wavefront, with kernel.cl's differences noted below), then spawnRays's
 * fan of secondary cones from the hit (kernel.cl:1115-1253), each traced to
 * the sky or to a surface, their light accumulated in generation order, and
 * draw (kernel.cl:1264-1275). Extra parity-contract rules: length and
 * normalize use sqrtf((x*x + y*y) + z*z); normalize of a zero vector is that
 * vector (OpenCL C); the double literal of `dotprod > 0.8` is compared in
 * double; native_sin/cos of the spine and ring angles and of normalVector are
 * (float)sin((double)x), like the ray-setup tables. */

#define MEGA_PI_F 3.14159274101257324219f
#define MEGA_PI_2_F 1.57079637050628662109f

/* The cone fan's per-launch constants: spawnRays's spine and ring loops depend
 * only on TraceInput (FovMultiplier/Constant, WeightingMultiplier/Constant). */
typedef struct {
  float fov, weighting, c, s, one_minus_c; /* spine: cone FoV, weighting, cos/sin(-spineAngle), 1 - cos */
  int ring_begin, n_rings;
} mega_spine;
typedef struct {
  float c, s, one_minus_c; /* cos/sin(-ringAngle), 1 - cos */
} mega_ring;
struct mega_schedule {
  int n_spines, n_rings;
  mega_spine *spine;
  mega_ring *ring;
};

/* Returns 0 when the loops would not end within `limit` cones per pixel. */
static int mega_build_schedule(const svo_trace_input *in, int limit, mega_schedule *S) {
  S->n_spines = S->n_rings = 0;
  S->spine = NULL;
  S->ring = NULL;
  int cap_s = 16, cap_r = 64, cones = 1;
  S->spine = (mega_spine *)malloc(sizeof(mega_spine) * cap_s);
  S->ring = (mega_ring *)malloc(sizeof(mega_ring) * cap_r);
  float fov = in->fov_constant, oldfov = fov, spine = 0.0f;
  const float FM = in->fov_multiplier, FC = in->fov_constant;
  while (spine < MEGA_PI_F) {
    fov = (FM * (spine + fov) + FC) / (1 - FM);
    spine = (1 + FM) * (spine + oldfov) / (1 - FM);
    oldfov = fov;
    if (S->n_spines == cap_s) S->spine = (mega_spine *)realloc(S->spine, sizeof(mega_spine) * (cap_s *= 2));
    mega_spine *sp = &S->spine[S->n_spines++];
    sp->fov = fov;
    sp->weighting = spine * in->weighting_multiplier + in->weighting_constant;
    sp->c = (float)cos((double)(-spine));
    sp->s = (float)sin((double)(-spine));
    sp->one_minus_c = 1.0f - sp->c;
    sp->ring_begin = S->n_rings;
    sp->n_rings = 0;
    cones += 1;
    for (int j = 1; (float)j * fov < MEGA_PI_2_F; j++) {
      if (cones + 2 > limit) return 0;
      if (S->n_rings == cap_r) S->ring = (mega_ring *)realloc(S->ring, sizeof(mega_ring) * (cap_r *= 2));
      mega_ring *rg = &S->ring[S->n_rings++];
      float angle = (float)(j * 2) * fov;
      rg->c = (float)cos((double)(-angle));
      rg->s = (float)sin((double)(-angle));
      rg->one_minus_c = 1.0f - rg->c;
      sp->n_rings++;
      cones += 2;
    }
    if (cones > limit) return 0;
  }
  return 1;
}

static float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void normalize3(float v[3]) {
  if (v[0] == 0.0f && v[1] == 0.0f && v[2] == 0.0f) return;
  float l = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] = v[0] / l;
  v[1] = v[1] / l;
  v[2] = v[2] / l;
}

/* Rodrigues rotation of v about the unit axis a by the angle whose cos, sin
 * and 1 - cos are (c, s, k), in kernel.cl's product order (spineRotation /
 * ringRotation, :1142-1166, :1181-1206); transpose = 1 gives the rotation by
 * the opposite angle (the second ring vector, :1217-1222). */
static void rotate3(const float a[3], float c, float s, float k, const float v[3], int transpose, float out[3]) {
  float r3 = k * a[0] * a[0], r4 = k * a[0] * a[1], r5 = k * a[0] * a[2];
  float r6 = k * a[1] * a[1], r7 = k * a[1] * a[2], r8 = k * a[2] * a[2];
  float r9 = s * a[0], r10 = s * a[1], r11 = s * a[2];
  if (!transpose) {
    out[0] = (r3 + c) * v[0] + (r4 - r11) * v[1] + (r5 + r10) * v[2];
    out[1] = (r4 + r11) * v[0] + (r6 + c) * v[1] + (r7 - r9) * v[2];
    out[2] = (r5 - r10) * v[0] + (r7 + r9) * v[1] + (r8 + c) * v[2];
  } else {
    out[0] = (r3 + c) * v[0] + (r4 + r11) * v[1] + (r5 - r10) * v[2];
    out[1] = (r4 - r11) * v[0] + (r6 + c) * v[1] + (r7 + r9) * v[2];
    out[2] = (r5 + r10) * v[0] + (r7 - r9) * v[1] + (r8 + c) * v[2];
  }
}

typedef struct {
  float origin[3], dir[3], inv[3], dof[2], fov;
  int sign[3];
  int cone_set; /* ConeDepth is 0 until a traverse sets it (setupInitialTrace leaves it unset) */
  uint64_t loc[3];
  uint8_t depth;
} mega_ray;

/* traceVoxel (kernel.cl:1075-1089) with traceBase (:1058-1073) and traceBlock
 * (:1002-1056). Returns 1 at a surface (*node: the block resolveRayData reads),
 * 0 in the sky (including a trace stopped by max_steps). */
static int mega_trace_voxel(const uint16_t *bases, uint8_t B, const svo_block *blocks, size_t n_blocks,
                            svo_usage *usage, size_t n_groups, uint16_t tick, int32_t max_steps, mega_ray *r,
                            uint32_t *node, uint32_t *steps, svo_child_request *req, uint32_t req_cap,
                            uint32_t *n_req) {
  uint32_t heap[64];
  heap[B + 1] = SVO_NO_CHILD;
  int32_t n = 0;
  for (;;) {
    if (r->depth == B + 1) {
      r->depth = B;
      continue;
    }
    if (max_steps > 0 && n >= max_steps) return 0;
    n++;
    (*steps)++;
    if (r->depth <= B) {
      uint16_t chunk = bases[oracle_pow_sum((uint8_t)(r->depth - 1)) + oracle_base_location(r->depth, r->loc)];
      if (((chunk >> (oracle_chunk_position(r->depth, r->loc) * 2)) & 2) != 2) {
        uint64_t prev[3] = {r->loc[0], r->loc[1], r->loc[2]};
        oracle_traverse_chunk(r->depth, r->dir, r->inv, r->sign, r->loc);
        r->cone_set = 1;
        if (leaving(r->loc, r->sign)) return 0;
        r->depth = oracle_compare_positions(r->depth, prev, r->loc, r->sign);
      } else {
        r->depth = r->depth < B ? (uint8_t)(r->depth + 1) : (uint8_t)(B + 2);
      }
      continue;
    }
    uint32_t addr = r->depth == B + 2
                        ? oracle_base_location((uint8_t)(B + 2), r->loc)
                        : node_at(blocks, n_blocks, heap[r->depth - 1])->child +
                              oracle_chunk_position((uint8_t)(r->depth - 1), r->loc);
    heap[r->depth] = addr;
    if (usage && (addr >> 3) < n_groups) {
      svo_usage *u = &usage[addr >> 3];
      if (u->tick < 65534 && u->tick != tick) u->tick = tick;
    }
    const svo_block *blk = node_at(blocks, n_blocks, addr);
    if (((blk->chunk >> (oracle_chunk_position(r->depth, r->loc) * 2)) & 2) != 2) {
      uint64_t prev[3] = {r->loc[0], r->loc[1], r->loc[2]};
      oracle_traverse_chunk(r->depth, r->dir, r->inv, r->sign, r->loc);
      r->cone_set = 1;
      if (leaving(r->loc, r->sign)) return 0;
      r->depth = oracle_compare_positions(r->depth, prev, r->loc, r->sign);
      continue;
    }
    /* ConeDepth = -half_log2(c) compared exactly; an unset ConeDepth (0) is
     * below B+2, so the first branch takes it. */
    float c = r->cone_set ? cone_size(cone_distance(r->origin, r->loc), r->fov, r->dof) : 1.0f;
    if (c > pow2_neg(B + 2)) {
      r->depth = (uint8_t)(B + 2);
      *node = heap[B + 2];
      return 1;
    }
    if (c > pow2_neg(r->depth)) {
      r->depth--;
      continue;
    }
    if (blk->child == SVO_NO_CHILD) {
      /* requestChild with buildChildRequest(localAddress, Depth, Tick, 1, Location) */
      uint32_t slot;
#ifdef _OPENMP
#pragma omp atomic capture
#endif
      slot = (*n_req)++;
      if (req && slot < req_cap) {
        svo_child_request *q = &req[slot];
        memset(q, 0, sizeof(*q));
        q->address = addr;
        q->tick = tick;
        q->depth = r->depth;
        q->location[0] = r->loc[0];
        q->location[1] = r->loc[1];
        q->location[2] = r->loc[2];
        q->tree_size = 1;
      }
      *node = addr;
      return 1;
    }
    if (c < pow2_neg(r->depth + 1)) {
      r->depth++;
      continue;
    }
    *node = addr; /* average() returns the block itself */
    return 1;
  }
}

/* resolveBackgroundRayData (kernel.cl:1225-1240): colour and luminosity of the sky. */
static void mega_sky(const float dir[3], uint8_t rgb[3], float *lum) {
  float dotp = dir[0] * 0.0f + dir[1] * 0.0f + dir[2] * -1.0f;
  if ((double)dotp > 0.8) {
    rgb[0] = rgb[1] = rgb[2] = 255;
    *lum = dotp * 150.0f;
  } else {
    rgb[0] = 135;
    rgb[1] = 206;
    rgb[2] = 235;
    *lum = 10.0f;
  }
}

/* normalVector (kernel.cl:264-275). */
static void mega_normal(int16_t pitch, int16_t yaw, float n[3]) {
  float fy = (float)yaw * MEGA_PI_F / 32767.0f, fp = (float)pitch * MEGA_PI_F / 32767.0f;
  float sy = (float)sin((double)fy), cy = (float)cos((double)fy);
  float sp = (float)sin((double)fp), cp = (float)cos((double)fp);
  n[0] = cy * cp;
  n[1] = sy * cp;
  n[2] = sp;
}

/* traverseChunkNormal (kernel.cl:428-489): the cone's start, one level-`depth`
 * cell along the normal, choosing the axis of the largest distance. */
static void mega_step_normal(uint8_t depth, const float nrm[3], uint64_t loc[3]) {
  int s[3];
  float inv[3], a[3];
  uint64_t d[3];
  for (int k = 0; k < 3; k++) {
    s[k] = nrm[k] >= 0;
    inv[k] = 1.0f / nrm[k];
    d[k] = oracle_round_ulong(loc[k], depth, s[k]);
    a[k] = fabsf((float)d[k] * inv[k]);
  }
  if (a[0] >= a[1] && a[0] >= a[2]) {
    float u = oracle_ulong_to_float(d[0]);
    d[1] = oracle_float_to_ulong(nrm[1] * inv[0] * u);
    d[2] = oracle_float_to_ulong(nrm[2] * inv[0] * u);
  } else if (a[1] >= a[0] && a[1] >= a[2]) {
    float u = oracle_ulong_to_float(d[1]);
    d[0] = oracle_float_to_ulong(nrm[0] * inv[1] * u);
    d[2] = oracle_float_to_ulong(nrm[2] * inv[1] * u);
  } else {
    float u = oracle_ulong_to_float(d[2]);
    d[0] = oracle_float_to_ulong(nrm[0] * inv[2] * u);
    d[1] = oracle_float_to_ulong(nrm[1] * inv[2] * u);
  }
  for (int k = 0; k < 3; k++) loc[k] = s[k] ? loc[k] + d[k] : loc[k] - d[k];
  for (int k = 0; k < 3; k++) {
    if (s[k] && loc[k] == 0)
      loc[k] = ULMAX;
    else if (!s[k] && loc[k] == ULMAX)
      loc[k] = 0;
  }
}

typedef struct {
  float weight, r, g, b; /* RayAccumulator: TotalWeighting, ColourR/G/B */
} mega_acc;

/* accumulateRay (kernel.cl:1110-1113): setupTrace (:524-544), traceRay and
 * writeToAccumulator (:1255-1262) for one cone. */
static void mega_cone(const uint16_t *bases, uint8_t B, const svo_block *blocks, size_t n_blocks, svo_usage *usage,
                      size_t n_groups, uint16_t tick, int32_t max_steps, const uint64_t hit_loc[3], uint8_t hit_depth,
                      const float nrm[3], const float dir[3], float fov, float weighting, mega_acc *acc,
                      uint32_t *steps, svo_child_request *req, uint32_t req_cap, uint32_t *n_req) {
  mega_ray c;
  for (int k = 0; k < 3; k++) {
    c.origin[k] = oracle_ulong_to_float(hit_loc[k]);
    c.dir[k] = dir[k];
    c.inv[k] = 1.0f / dir[k];
    c.sign[k] = dir[k] >= 0;
    c.loc[k] = hit_loc[k];
  }
  c.dof[0] = c.dof[1] = 0.0f;
  c.fov = fov;
  c.depth = 1;
  mega_step_normal(hit_depth, nrm, c.loc);
  c.cone_set = 1;
  uint32_t node;
  int surface = mega_trace_voxel(bases, B, blocks, n_blocks, usage, n_groups, tick, max_steps, &c, &node, steps, req,
                                 req_cap, n_req);
  acc->weight += weighting;
  if (surface) return; /* Luminosity 0 */
  uint8_t rgb[3];
  float lum;
  mega_sky(dir, rgb, &lum);
  acc->r += ((float)rgb[0] / 255.0f) * weighting * lum;
  acc->g += ((float)rgb[1] / 255.0f) * weighting * lum;
  acc->b += ((float)rgb[2] / 255.0f) * weighting * lum;
}

int64_t oracle_mega_trace_rows(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                               svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                               int32_t cone_limit, const oracle_view_out *out, uint32_t *n_cones,
                               svo_child_request *req, uint32_t req_cap, uint32_t *n_req, int32_t threads,
                               uint32_t row_begin, uint32_t row_end) {
  /* kernel.cl:1533-1534: nothing is drawn for an unusable cone schedule */
  if (in->fov_constant <= 0 || in->fov_multiplier >= 1 || in->fov_multiplier <= -1) return 0;
  mega_schedule S;
  if (!mega_build_schedule(in, cone_limit, &S)) {
    free(S.spine);
    free(S.ring);
    return -1;
  }
  uint32_t W = in->screen_size[0], H = in->screen_size[1];
  if (row_end > H) row_end = H;
  if (row_begin > row_end) row_begin = row_end;
  const uint8_t B = base_depth;
  float *su = (float *)malloc(sizeof(float) * (W + 1));
  float *cu = (float *)malloc(sizeof(float) * (W + 1));
  float *sv = (float *)malloc(sizeof(float) * (H + 1));
  float *cv = (float *)malloc(sizeof(float) * (H + 1));
  oracle_view_tables(in, su, cu, sv, cv);
  int64_t n = (int64_t)W * (row_end - row_begin);
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
  for (int64_t id = 0; id < n; id++) {
    uint32_t px = (uint32_t)(id % W), py = row_begin + (uint32_t)(id / W);
    /* setupInitialTrace (kernel.cl:491-522): DoF and Tick come from the input */
    float m0 = cu[px] * cv[py], m1 = (0.0f - su[px]) * cv[py], m2 = sv[py];
    const float *F = in->facing;
    mega_ray p;
    p.dir[0] = F[0] * m0 + F[3] * m1 + F[6] * m2;
    p.dir[1] = F[1] * m0 + F[4] * m1 + F[7] * m2;
    p.dir[2] = F[2] * m0 + F[5] * m1 + F[8] * m2;
    for (int k = 0; k < 3; k++) {
      p.inv[k] = 1.0f / p.dir[k];
      p.sign[k] = p.dir[k] >= 0;
      p.origin[k] = in->origin[k];
    }
    p.dof[0] = in->dof[0];
    p.dof[1] = in->dof[1];
    p.fov = in->fov[0] / (float)W;
    p.cone_set = 0;
    p.depth = 1;
    uint32_t steps = 0, cones = 0, hit_index = SVO_MISS;
    uint8_t hit_depth = 0;
    float t = INFINITY;
    uint8_t rgb[3];
    mega_acc acc = {0.0f, 0.0f, 0.0f, 0.0f};
    if (!oracle_trace_into_volume(p.origin, p.dir, p.inv, p.fov, p.dof, p.loc)) {
      float lum;
      mega_sky(p.dir, rgb, &lum);
    } else {
      uint32_t node = 0;
      int surface = mega_trace_voxel(bases, B, blocks, n_blocks, usage, n_groups, in->tick, max_steps, &p, &node,
                                     &steps, req, req_cap, n_req);
      float nrm[3] = {0.0f, 0.0f, 0.0f};
      uint8_t depth = 1; /* RayData.Depth of a sky ray */
      if (surface) {
        /* resolveRayData (kernel.cl:1242-1253) */
        const svo_block *blk = node_at(blocks, n_blocks, node);
        rgb[0] = blk->colour_r;
        rgb[1] = blk->colour_g;
        rgb[2] = blk->colour_b;
        mega_normal(blk->normal_pitch, blk->normal_yaw, nrm);
        depth = p.depth;
        hit_index = node;
        hit_depth = p.depth;
        float x = oracle_ulong_to_float(p.loc[0]) - p.origin[0];
        float y = oracle_ulong_to_float(p.loc[1]) - p.origin[1];
        float z = oracle_ulong_to_float(p.loc[2]) - p.origin[2];
        t = sqrtf(x * x + y * y + z * z);
      } else {
        float lum;
        mega_sky(p.dir, rgb, &lum);
      }
      /* spawnRays (kernel.cl:1115-1253) with baseWeighting 1 */
      const float *D = p.dir;
      float axis[3] = {D[1] * nrm[2] - D[2] * nrm[1], D[2] * nrm[0] - D[0] * nrm[2], D[0] * nrm[1] - D[1] * nrm[0]};
      normalize3(axis);
      float d2 = 2.0f * dot3(D, nrm);
      float refl[3] = {D[0] - d2 * nrm[0], D[1] - d2 * nrm[1], D[2] - d2 * nrm[2]};
      float fov = in->fov_constant, weighting = in->weighting_constant, rw = weighting;
      float dp = dot3(refl, nrm);
      if (dp < fov) rw = weighting * dp / fov;
      mega_cone(bases, B, blocks, n_blocks, usage, n_groups, in->tick, max_steps, p.loc, depth, nrm, refl, fov,
                rw * 1.0f, &acc, &steps, req, req_cap, n_req);
      cones++;
      for (int s = 0; s < S.n_spines; s++) {
        const mega_spine *sp = &S.spine[s];
        fov = sp->fov;
        weighting = sp->weighting;
        rw = weighting;
        float seed[3];
        rotate3(axis, sp->c, sp->s, sp->one_minus_c, refl, 0, seed);
        normalize3(seed);
        dp = dot3(seed, nrm);
        if (dp < 0) break;
        if (dp < fov) rw = weighting * dp / fov;
        mega_cone(bases, B, blocks, n_blocks, usage, n_groups, in->tick, max_steps, p.loc, depth, nrm, seed, fov,
                  rw * 1.0f, &acc, &steps, req, req_cap, n_req);
        cones++;
        for (int j = 0; j < sp->n_rings; j++) {
          const mega_ring *rg = &S.ring[sp->ring_begin + j];
          rw = weighting;
          float v[3];
          rotate3(refl, rg->c, rg->s, rg->one_minus_c, seed, 0, v);
          normalize3(v);
          dp = dot3(v, nrm);
          if (dp < 0) break;
          if (dp < fov) rw = weighting * dp / fov;
          mega_cone(bases, B, blocks, n_blocks, usage, n_groups, in->tick, max_steps, p.loc, depth, nrm, v, fov,
                    rw * 1.0f, &acc, &steps, req, req_cap, n_req);
          rotate3(refl, rg->c, rg->s, rg->one_minus_c, seed, 1, v);
          normalize3(v);
          mega_cone(bases, B, blocks, n_blocks, usage, n_groups, in->tick, max_steps, p.loc, depth, nrm, v, fov,
                    rw * 1.0f, &acc, &steps, req, req_cap, n_req);
          cones += 2;
        }
      }
    }
    if (out->hit_index) out->hit_index[id] = hit_index;
    if (out->hit_depth) out->hit_depth[id] = hit_depth;
    if (out->t) out->t[id] = t;
    if (out->steps) out->steps[id] = steps;
    if (n_cones) n_cones[id] = cones;
    if (out->rgba) {
      /* draw (kernel.cl:1264-1275) */
      float *o = &out->rgba[4 * id];
      if (acc.weight > 0.01f) {
        o[0] = fminf(((float)rgb[0] + acc.r / acc.weight) / 255.0f, 1.0f);
        o[1] = fminf(((float)rgb[1] + acc.g / acc.weight) / 255.0f, 1.0f);
        o[2] = fminf(((float)rgb[2] + acc.b / acc.weight) / 255.0f, 1.0f);
      } else {
        o[0] = (float)rgb[0] / 255.0f;
        o[1] = (float)rgb[1] / 255.0f;
        o[2] = (float)rgb[2] / 255.0f;
      }
      o[3] = 1.0f;
    }
  }
  free(su);
  free(cu);
  free(sv);
  free(cv);
  free(S.spine);
  free(S.ring);
  return 0;
}


/* ---- the wavefront's secondary-cone stage, as the reference wires it --------
 *
 * MainWindow.RunWavefront (MainWindow.cs:390-402) has it commented out; enabled
 * as written, per primary hit: evaluateMaterial (wavefront.cl:1568-1739) builds
 * the hit's cone fan (the same fan as kernel.cl's spawnRays), saveAccumulator
 * (:338-355) puts every cone of weighting > 5 on the background queue without
 * tracing it, evaluateBackground (:1741-1797) adds its sky light (blended with
 * the hit block's colour by the ambient light level) to the pixel, and
 * resolveRemainders finds the material queue already reset, so the hit's own
 * colour is never added. Float-to-uchar conversions saturate. */

static int gi_schedule(const svo_trace_input *in, mega_schedule **S) {
  *S = (mega_schedule *)calloc(1, sizeof(mega_schedule));
  if (!mega_build_schedule(in, SVO_MEGA_MAX_CONES, *S)) {
    gi_free_schedule(*S);
    *S = NULL;
    return 0;
  }
  return 1;
}

static void gi_free_schedule(mega_schedule *S) {
  free(S->spine);
  free(S->ring);
  free(S);
}

/* saveAccumulator + evaluateBackground of one cone with weighting w. */
static void gi_cone(const float d[3], uint8_t w, const svo_block *blk, uint8_t ambient, uint32_t acc[4]) {
  if (w <= 5) return;
  float dotp = d[0] * 0.0f + d[1] * 0.0f + d[2] * -1.0f;
  uint8_t c[3], lum;
  if (dotp > 0.8f) {
    c[0] = c[1] = c[2] = 255;
    lum = sat_u8(dotp * 200.0f);
  } else {
    c[0] = 135;
    c[1] = 206;
    c[2] = 235;
    lum = 1;
  }
  if (w < 255) {
    uint32_t boundary = lum > ambient ? 255u : 0u;
    float q = (float)(lum > ambient ? lum - ambient : ambient - lum) / ((float)(lum + ambient) * 255.0f);
    const uint8_t base[3] = {blk->colour_r, blk->colour_g, blk->colour_b};
    for (int k = 0; k < 3; k++) c[k] = sat_u8((float)base[k] + q * (float)c[k] * (float)(uint32_t)(boundary - base[k]));
  }
  acc[0] += w;
  if (lum > 0)
    for (int k = 0; k < 3; k++) acc[1 + k] += (uint32_t)c[k] * w;
}

static void gi_pixel(const svo_block *blk, const float dir[3], const svo_trace_input *in, const mega_schedule *S,
                     uint32_t acc[4]) {
  acc[0] = acc[1] = acc[2] = acc[3] = 0;
  const float base_w = 255.0f; /* the primary's Weighting */
  float nrm[3];
  mega_normal(blk->normal_pitch, blk->normal_yaw, nrm);
  if (in->weighting_constant * base_w < 6) {
    acc[0] = 255; /* FinalWeightings[traceID] = baseWeighting */
    return;
  }
  if (dot3(dir, nrm) >= 0) { /* seen edge-on: one cone along the primary direction */
    gi_cone(dir, 255, blk, in->ambient_light_level, acc);
    return;
  }
  const float *D = dir;
  float axis[3] = {D[1] * nrm[2] - D[2] * nrm[1], D[2] * nrm[0] - D[0] * nrm[2], D[0] * nrm[1] - D[1] * nrm[0]};
  normalize3(axis);
  float d2 = 2.0f * dot3(D, nrm);
  float refl[3] = {D[0] - d2 * nrm[0], D[1] - d2 * nrm[1], D[2] - d2 * nrm[2]};
  float fov = in->fov_constant, weighting = in->weighting_constant, rw = weighting;
  float dp = dot3(refl, nrm);
  if (dp < fov) rw = weighting * dp / fov;
  gi_cone(refl, sat_u8(rw * base_w), blk, in->ambient_light_level, acc);
  for (int s = 0; s < S->n_spines; s++) {
    const mega_spine *sp = &S->spine[s];
    fov = sp->fov;
    weighting = sp->weighting;
    rw = weighting;
    float seed[3];
    rotate3(axis, sp->c, sp->s, sp->one_minus_c, refl, 0, seed);
    normalize3(seed);
    dp = dot3(seed, nrm);
    if (dp < 0) break;
    if (dp < fov) rw = weighting * dp / fov;
    gi_cone(seed, sat_u8(rw * base_w), blk, in->ambient_light_level, acc);
    for (int j = 0; j < sp->n_rings; j++) {
      const mega_ring *rg = &S->ring[sp->ring_begin + j];
      rw = weighting;
      float v[3];
      rotate3(refl, rg->c, rg->s, rg->one_minus_c, seed, 0, v);
      normalize3(v);
      dp = dot3(v, nrm);
      if (dp < 0) break;
      if (dp < fov) rw = weighting * dp / fov;
      gi_cone(v, sat_u8(rw * base_w), blk, in->ambient_light_level, acc);
      rotate3(refl, rg->c, rg->s, rg->one_minus_c, seed, 1, v);
      normalize3(v);
      gi_cone(v, sat_u8(rw * base_w), blk, in->ambient_light_level, acc);
    }
  }
}
