/*
 * svo_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's wavefront cone tracer
 * (SvoTracer/SvoTracer.Kernel/wavefront.cl) used as the parity checker of the
 * CUDA path. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it. Nothing in the product links or calls it.
 */
#ifndef SVO_ORACLE_H
#define SVO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/svo.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-pixel stats of one view (any pointer may be NULL). */
typedef struct oracle_view_out {
  uint32_t *hit_index;
  uint8_t *hit_depth;
  float *t;
  float *rgba;    /* 4 per pixel */
  uint32_t *acc;  /* 4 per pixel: FinalWeightings, FinalColourR, G, B */
  uint32_t *v_block; /* node reads of the reference's getBlockAddress walks */
  uint32_t *v_base;  /* base chunk reads */
  uint32_t *steps;   /* traversal steps (base + block) */
  /* The request each ray raised, by pixel: requested[pixel] = 1 and
   * pixel_request[pixel] = the record when the ray stopped with a child
   * request, requested[pixel] = 0 otherwise. The queue of the pixel-order rule
   * (SVO_REQUESTS_PIXEL) is the flagged records in pixel order, capped. */
  uint8_t *requested;
  svo_child_request *pixel_request;
} oracle_view_out;

/* Traces one view. usage (n_groups entries) is stamped like runBlockTrace;
 * child requests are appended at *n_req (slots >= req_cap are counted, not
 * written). Returns the number of rays stopped by max_steps. threads <= 0
 * uses all OpenMP threads. */
int64_t oracle_trace_view(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                          svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                          const oracle_view_out *out, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                          int32_t threads);
/* Same for rows [row_begin, row_end) of the view only; per-pixel outputs are
 * indexed within the band (pixel (x, y) at (y - row_begin) * W + x). */
int64_t oracle_trace_rows(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                          svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                          const oracle_view_out *out, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                          int32_t threads, uint32_t row_begin, uint32_t row_end);

/* Same, with gi = 1 also running the wavefront's secondary-cone stage as the
 * reference wires it (the hits' accumulators and colour, their usage stamps);
 * returns -2 when the cone schedule's loops would not end. */
int64_t oracle_trace_rows_gi(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                             svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                             const oracle_view_out *out, svo_child_request *req, uint32_t req_cap, uint32_t *n_req,
                             int32_t threads, uint32_t row_begin, uint32_t row_end, int32_t gi);

/* Ray-setup tables of the parity contract: sinU/cosU per column, sinV/cosV
 * per row, each (float)sin((double)angle). */
void oracle_view_tables(const svo_trace_input *in, float *sin_u, float *cos_u, float *sin_v, float *cos_v);

/* Fixed-point helpers, exported for unit tests. */
uint64_t oracle_float_to_ulong(float x);
float oracle_ulong_to_float(uint64_t x);
uint64_t oracle_round_ulong(uint64_t value, uint8_t depth, int round_up);
uint32_t oracle_pow_sum(uint8_t depth);
uint8_t oracle_chunk_position(uint8_t depth, const uint64_t loc[3]);
uint32_t oracle_base_location(uint8_t depth, const uint64_t loc[3]);
/* traverseChunk on a bare state; loc is updated in place. */
void oracle_traverse_chunk(uint8_t depth, const float dir[3], const float inv[3], const int sign[3], uint64_t loc[3]);
uint8_t oracle_compare_positions(uint8_t depth, const uint64_t prev[3], const uint64_t loc[3], const int sign[3]);
/* traceIntoVolume: returns 1 and the entry location when the ray enters. */
int oracle_trace_into_volume(const float origin[3], const float dir[3], const float inv[3], float fov,
                             const float dof[2], uint64_t loc[3]);

/* The megakernel (kernel.cl's `trace`) over rows [row_begin, row_end): per pixel
 * the primary cone, the spawnRays fan of secondary cones and draw's colour.
 * out->hit_index/hit_depth/t describe the primary's surface block, out->steps
 * counts the traversal steps of all the pixel's traces and n_cones its
 * secondary cones (either may be NULL). Returns -1 (nothing traced) when the
 * cone schedule has more than cone_limit cones per pixel, else 0; an unusable
 * schedule (FovConstant <= 0, |FovMultiplier| >= 1) draws nothing, as the
 * kernel does. */
int64_t oracle_mega_trace_rows(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                               svo_usage *usage, size_t n_groups, const svo_trace_input *in, int32_t max_steps,
                               int32_t cone_limit, const oracle_view_out *out, uint32_t *n_cones,
                               svo_child_request *req, uint32_t req_cap, uint32_t *n_req, int32_t threads,
                               uint32_t row_begin, uint32_t row_end);

/* Usage initialisation rule of MainWindow.cs:129-141. */
void oracle_init_usage(const uint16_t *bases, uint8_t base_depth, svo_usage *usage, size_t n_groups);

/* Differentiable forward model (no reference counterpart): per-ray LOD hit
 * lists of one view, the ray continuing past each hit as if its octant were
 * empty; then FP64 compositing, loss, analytic gradient and central finite
 * differences over those lists. */
void oracle_hit_lists(const uint16_t *bases, uint8_t base_depth, const svo_block *blocks, size_t n_blocks,
                      const svo_trace_input *in, int32_t max_steps, int32_t max_hits, uint32_t *hits, uint8_t *n_hits,
                      uint8_t *leaves, float *sky, int32_t threads);
double oracle_diff_eval(const uint32_t *hits, const uint8_t *n_hits, const uint8_t *leaves, const float *sky,
                        int64_t n_rays, int32_t max_hits, const double *params, const double *target, double *rgb,
                        double *grad, int32_t threads);
void oracle_diff_fd(const uint32_t *hits, const uint8_t *n_hits, const uint8_t *leaves, const float *sky,
                    int64_t n_rays, int32_t max_hits, const double *params, const double *target, const uint32_t *nodes,
                    int32_t n_nodes, double h, double *fd, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif
