/*
 * svo.h -- C ABI of the GB300 sparse-voxel-octree cone tracer (libsvo.so).
 *
 * Every entry point returns an svo_status (0 = success) and never lets a C++
 * exception cross the boundary. A non-zero status leaves a message that
 * svo_last_error_string() returns; the C# facade turns it into an exception
 * the way the reference's ComputeManager.HandleResultCode does
 * (SvoTracer.Kernel/ComputeManager.cs:283-287).
 *
 * Structs use the OpenCL layouts the reference kernels declare
 * (SvoTracer.Kernel/wavefront.cl:1-84), naturally aligned, with the sizes
 * checked by static_assert below. Several of the reference's C# serialisers
 * write shorter records than these OpenCL layouts; this ABI follows the
 * kernel side.
 *
 * Threading: a context is used from one host thread at a time. All device
 * work of a context runs on one CUDA stream (svo_set_stream may replace it).
 * Host buffers belong to the caller; device buffers made by the library
 * belong to the context and are released by svo_destroy.
 */
#ifndef SVO_H
#define SVO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SVO_API __attribute__((visibility("default")))
#else
#define SVO_API
#endif

typedef int32_t svo_status;

enum {
  SVO_OK = 0,
  SVO_ERR_INVALID_ARGUMENT = 1,
  SVO_ERR_CUDA = 2,
  SVO_ERR_OUT_OF_MEMORY = 3,
  SVO_ERR_QUEUE_FULL = 4,  /* reserved: no call returns it. A child-request queue past its cap is not an
                              error (the reference drops the requests past MaxChildRequestId); the raised
                              count that svo_read_child_requests returns then exceeds the cap */
  SVO_ERR_TIMEOUT = 5,     /* a bounded device wait ran out */
  SVO_ERR_NO_TREE = 6,     /* trace/prune/graft before svo_upload_octree */
  SVO_ERR_STEP_LIMIT = 7,  /* reserved: no call returns it. A ray that reaches max_steps ends in the sky,
                              as a ray the reference stops does, and is counted in
                              svo_trace_stats.step_limited */
  SVO_ERR_BUDGET = 8,      /* block budget exhausted (builder, graft) */
  SVO_ERR_NO_DEVICE = 9,   /* no usable CUDA device / kernel image */
  SVO_ERR_INTERNAL = 10,
  SVO_ERR_IO = 11          /* a file could not be opened, read or written, or is truncated */
};

/* Sentinels of the reference format. */
#define SVO_NO_CHILD 0xFFFFFFFFu      /* Block.Child with no children      */
#define SVO_TICK_MULTI_PARENT 65534u  /* Usage.Tick: multi-parent group    */
#define SVO_TICK_INVIOLATE 65535u     /* Usage.Tick: never collected       */
#define SVO_MISS 0xFFFFFFFFu          /* hit_index of a ray that hit nothing */
#define SVO_MAX_TREE_DEPTH 24         /* deepest node level a trace walks   */

/* 16-byte node: wavefront.cl:1-12, SvoTracer.Domain/Models/Block.cs:7-21.
 * chunk holds 2 bits per child octant k = x + 2y + 4z:
 * bit 2k = child contains air, bit 2k+1 = child contains geometry. */
typedef struct svo_block {
  uint32_t child;  /* first of 8 consecutive children, SVO_NO_CHILD = none */
  uint16_t chunk;
  int16_t normal_pitch;
  int16_t normal_yaw;
  uint8_t colour_r;
  uint8_t colour_g;
  uint8_t colour_b;
  uint8_t opacity;
  uint8_t specularity; /* "Spare" in wavefront.cl */
  uint8_t gloss;
} svo_block;

/* One per 8-node block group: wavefront.cl:14-17. Tick 0 = free. */
typedef struct svo_usage {
  uint16_t tick;
  uint16_t _pad;
  uint32_t parent; /* node address whose Child points at this group */
} svo_usage;

/* Camera/frame parameters, wavefront.cl:53-75 (104 bytes).
 * facing is column-major 3x3: columns forward, left, up. */
typedef struct svo_trace_input {
  float origin[3];
  float facing[9];
  float fov[2];  /* horizontal, vertical FoV in radians */
  float dof[2];  /* depth of field (angle, focal distance) */
  uint32_t screen_size[2];
  uint8_t max_opacity;
  uint8_t base_depth;
  uint16_t tick;
  uint32_t max_child_request_id;
  float fov_multiplier;
  float fov_constant;
  float weighting_multiplier;
  float weighting_constant;
  uint8_t ambient_light_level;
  uint8_t _pad[7];
} svo_trace_input;

/* Tree-update parameters, wavefront.cl:77-84 (20 bytes). */
typedef struct svo_update_input {
  uint8_t base_depth;
  uint8_t _pad;
  uint16_t tick;
  uint32_t max_child_request_id;
  uint32_t memory_size; /* block count */
  uint32_t offset;      /* stale threshold in ticks */
  uint32_t graft_size;  /* block groups to claim */
} svo_update_input;

/* Host-issued tree edit, wavefront.cl:24-36 (20 bytes).
 * properties: bit0 cull child subtree and set child_address; bits1-2 = 11
 * make inviolate, 01 stamp the tick; bit3 overwrite the node (colour from
 * the record's surface block) and its chunk; bit4 write a base chunk. */
typedef struct svo_pruning {
  uint8_t properties;
  uint8_t depth;   /* 255: address is a node index, else a Location index */
  uint8_t _pad0[2];
  uint32_t address;
  uint16_t chunk;
  uint8_t _pad1[2];
  uint32_t colour_address;
  uint32_t child_address;
} svo_pruning;

/* Subtree graft, wavefront.cl:38-43 (16 bytes). */
typedef struct svo_grafting {
  uint32_t graft_data_address; /* first group of this subtree in the payload */
  uint32_t graft_total_size;   /* groups in this subtree */
  uint8_t depth;               /* 255: graft_address is a node index */
  uint8_t _pad[3];
  uint32_t graft_address;
} svo_grafting;

/* Missing-child request raised by a trace, wavefront.cl:45-51 (40 bytes). */
typedef struct svo_child_request {
  uint32_t address;
  uint16_t tick;
  uint8_t depth;
  uint8_t _pad0;
  uint64_t location[3];
  uint8_t tree_size;
  uint8_t _pad1[7];
} svo_child_request;

/* Per-pixel results of a trace. Pointers are host memory unless on_device is
 * non-zero, then they are device pointers the caller owns. Any pointer may be
 * NULL to skip that output. When every host output of a call is pinned
 * (cudaMallocHost / cudaHostRegister), the kernel writes hit_index, t and rgba
 * directly, so their transfer overlaps the trace, and hit_depth (one byte per
 * pixel, too small a store to cross to host memory efficiently) goes through a
 * device buffer and one copy per view; other host memory goes through device
 * buffers and a copy after the trace. Either way the call returns with the
 * outputs written. */
typedef struct svo_trace_output {
  uint32_t *hit_index; /* node index of the hit, SVO_MISS for background */
  uint8_t *hit_depth;  /* level of the hit node, 0 for background */
  float *t;            /* distance origin->hit location, +inf for background */
  float *rgba;         /* 4 floats per pixel, drawTrace's colour */
  int32_t on_device;
  int32_t _pad;
} svo_trace_output;

/* Counters of the last trace (or batch). */
typedef struct svo_trace_stats {
  uint64_t rays;
  uint64_t hits;
  uint64_t base_steps;       /* V_base summed over rays */
  uint64_t block_node_reads; /* V_block summed over rays (reference walk) */
  uint64_t block_steps;
  uint64_t child_requests;   /* raised, may exceed the cap */
  uint64_t step_limited;     /* rays stopped by the step limit */
} svo_trace_stats;

/* Tuning of the persistent trace kernel (0 = library default). */
typedef struct svo_trace_config {
  int32_t block_size;   /* threads per CTA, multiple of 32 up to 256 (default 192) */
  int32_t ctas_per_sm;  /* resident CTAs per SM for the persistent grid */
  int32_t ray_chunk;    /* rays a thread claims per ray-queue fetch (1..64) */
  int32_t cadence;      /* steps a thread runs between ray retire/refill points (1..1024) */
  int32_t max_steps;    /* per-ray step limit */
  int32_t collect_stats; /* 0 none, 1 totals (svo_last_trace_stats), 2 totals and per-ray counts */
  int32_t max_hits;     /* differentiable forward: LOD hits composited per ray (1..1024) */
  int32_t schedule;     /* SVO_SCHEDULE_LANE, SVO_SCHEDULE_WARP or SVO_SCHEDULE_WAVEFRONT */
  int32_t mega_band_tiles; /* megakernel: pixel tiles of 32 per cone band (0: as many as 2^26 cone slots hold) */
  int32_t l2_window;    /* 1: the trace kernel reads the dense level-(B+2) nodes through an L2 persisting
                           access-policy window, -1: no window */
  int32_t pass_limit;   /* per-ray pass bound of the trace, megakernel and colour-fitting loops (0: max_steps + 2,
                           which only a fault reaches); a smaller value stops the kernels with SVO_ERR_TIMEOUT, a
                           test of that path. A stopped kernel is reported by the next call that synchronises
                           with the device (svo_synchronize included) and then cleared. */
  int32_t request_order; /* SVO_REQUESTS_ARRIVAL (default) or SVO_REQUESTS_PIXEL, see below */
  int32_t gi_stage;     /* 1: svo_trace / svo_trace_batch also run the wavefront's secondary-cone stage as the
                           reference wires it (MainWindow.cs:390-402, disabled there): evaluateMaterial's cone fan
                           of every primary hit (wavefront.cl:1568-1739), each cone of weighting > 5 put straight
                           on the background queue by saveAccumulator (:338-355) and lit by evaluateBackground
                           (:1741-1797), the hit's own colour never added. The views of a call must share their
                           cone parameters and AmbientLightLevel. -1 or 0: off */
} svo_trace_config;

/* Child requests of svo_trace / svo_trace_batch past the queue's cap
 * (max_child_request_id). ARRIVAL: the queue keeps the first requests to
 * arrive, in arrival order, as the reference's requestChild does
 * (wavefront.cl:362-375); which requests those are depends on the timing of
 * the device's atomics. PIXEL: the queue holds the requests of the lowest
 * pixel indices (views in call order, pixels row-major) in that order, so the
 * queue, and every graft decision taken from it, is the same on every run.
 * Below the cap both hold the same requests. A ray raises at most one request,
 * when it stops. */
enum { SVO_REQUESTS_ARRIVAL = 1, SVO_REQUESTS_PIXEL = 2 };

/* Ray scheduling of the persistent trace kernel. LANE: each thread claims rays
 * on its own and finished rays are replaced every `cadence` steps. WARP: each
 * warp claims 32 consecutive rays, runs them to the end and regroups before the
 * next claim (ray_chunk and cadence unused). WAVEFRONT: the reference's queue
 * compaction between passes (wavefront.cl:249-336, MainWindow.cs:452-481) inside
 * each CTA: every pass, each thread takes one step of its ray, and the rays
 * whose octant was empty are compacted into a shared-memory queue whose moves
 * the CTA's first threads run in full warps. Results are identical. */
enum { SVO_SCHEDULE_LANE = 1, SVO_SCHEDULE_WARP = 2, SVO_SCHEDULE_WAVEFRONT = 3 };

/* Counters of the last svo_mega_trace. */
typedef struct svo_mega_stats {
  uint64_t pixels;     /* primary cones */
  uint64_t surfaces;   /* primary cones that ended at a surface */
  uint64_t cones;      /* secondary cones traced (spawnRays's fans) */
  uint64_t cone_slots; /* cone slots laid out: tiles x cones of each tile's fullest pixel x 32 */
} svo_mega_stats;

/* Cones per pixel the megakernel accepts in one fan (spawnRays's loops end
 * after at most this many cones, or the call is refused). */
#define SVO_MEGA_MAX_CONES 4096

/* ---- context ------------------------------------------------------------ */

SVO_API const char *svo_last_error_string(void);
SVO_API const char *svo_version(void);

/* Replaces ComputeManagerFactory.Build (SvoTracer.Kernel/ComputeManagerFactory.cs:12-89). */
SVO_API svo_status svo_create(int32_t device, void **ctx);
/* Replaces ComputeManager.Dispose (ComputeManager.cs:357-367). */
SVO_API svo_status svo_destroy(void *ctx);
/* Runs the context's work on a caller stream (cudaStream_t); NULL = own stream. */
SVO_API svo_status svo_set_stream(void *ctx, void *stream);
SVO_API svo_status svo_synchronize(void *ctx);
SVO_API svo_status svo_set_trace_config(void *ctx, const svo_trace_config *cfg);
SVO_API svo_status svo_get_trace_config(void *ctx, svo_trace_config *cfg);

/* ---- octree residency ---------------------------------------------------- */

/* Replaces InitReadBuffer(Bases/Blocks) of MainWindow.SetupWavefrontKernels
 * (SvoTracer.Window/MainWindow.cs:143-147). block_budget is the number of
 * nodes the device arrays can hold (>= n_blocks, rounded up to whole groups);
 * 0 = n_blocks. */
SVO_API svo_status svo_upload_octree(void *ctx, uint8_t base_depth, const uint16_t *bases, size_t n_bases,
                                     const svo_block *blocks, size_t n_blocks, uint32_t block_budget);
/* Usage initialisation of MainWindow.cs:129-145. */
SVO_API svo_status svo_init_usage(void *ctx);
SVO_API svo_status svo_read_usage(void *ctx, svo_usage *out, size_t n_groups);
SVO_API svo_status svo_write_usage(void *ctx, const svo_usage *in, size_t n_groups);
SVO_API svo_status svo_read_blocks(void *ctx, svo_block *out, size_t first, size_t n);
SVO_API svo_status svo_read_bases(void *ctx, uint16_t *out, size_t n);
SVO_API svo_status svo_tree_size(void *ctx, uint8_t *base_depth, size_t *n_bases, size_t *n_blocks, size_t *block_budget);

/* ---- trace ----------------------------------------------------------------- */

/* One view: init -> runBaseTrace/runBlockTrace passes -> evaluateBackground ->
 * resolveRemainders -> drawTrace (wavefront.cl:1352-1850, driven by
 * MainWindow.RunWavefront, MainWindow.cs:356-426). Stamps usage ticks and
 * queues child requests (capped at max_child_request_id). */
SVO_API svo_status svo_trace(void *ctx, const svo_trace_input *input, const svo_trace_output *out);
/* n_views (<= 512) views in one persistent launch. out[i] receives view i. */
SVO_API svo_status svo_trace_batch(void *ctx, const svo_trace_input *inputs, int32_t n_views, const svo_trace_output *out);
/* Same, replayed from a CUDA graph captured on first use for this view set. */
SVO_API svo_status svo_trace_batch_graph(void *ctx, const svo_trace_input *inputs, int32_t n_views,
                                         const svo_trace_output *out);
SVO_API svo_status svo_last_trace_stats(void *ctx, svo_trace_stats *stats);
/* Autotuner for a view set (no reference counterpart): times svo_trace_batch
 * with warp batches and the CTA wavefront at block sizes {64,128,256}, and lane
 * refills at those sizes x ray chunks {1,2,4,8} x cadences {4,8,16,32}
 * (best of `repeats` runs each; outputs must be device pointers), keeps the
 * fastest configuration in the context and returns it. Results are identical
 * for every configuration. */
SVO_API svo_status svo_autotune(void *ctx, const svo_trace_input *inputs, int32_t n_views,
                                const svo_trace_output *out, int32_t repeats, svo_trace_config *best,
                                float *best_ms);
/* Per-ray V_block / V_base of the last trace run with collect_stats = 2,
 * in batch ray order (view 0's pixels first). */
SVO_API svo_status svo_read_ray_counts(void *ctx, uint32_t *v_block, uint32_t *v_base, size_t n);
/* Child requests of the last trace. *n = requests raised (may exceed cap). */
SVO_API svo_status svo_read_child_requests(void *ctx, svo_child_request *out, uint32_t cap, uint32_t *n);

/* ---- megakernel ------------------------------------------------------------ */

/* Replaces an Enqueue of kernel.cl's `trace` over ScreenSize (kernel.cl:1531-1558,
 * the kernel.cl build of MainWindow.cs:45): per pixel the primary cone, the
 * spawnRays fan of secondary cones from where it ends (kernel.cl:1115-1253), and
 * draw's colour (kernel.cl:1264-1275) into out->rgba. Reads the first 96 bytes of
 * `input` (kernel.cl's TraceInput, which has no AmbientLightLevel).
 * out->hit_index / hit_depth / t describe the primary cone's surface block
 * (SVO_MISS / 0 / +inf in the sky). Usage ticks are stamped and child requests
 * (Tick = input->tick, TreeSize 1) queued as by svo_trace. FovConstant <= 0 or
 * |FovMultiplier| >= 1 draws nothing, as the kernel returns; a cone schedule
 * whose loops would run past SVO_MEGA_MAX_CONES cones per pixel (the kernel's
 * would not end) returns SVO_ERR_INVALID_ARGUMENT. */
SVO_API svo_status svo_mega_trace(void *ctx, const svo_trace_input *input, const svo_trace_output *out);
SVO_API svo_status svo_last_mega_stats(void *ctx, svo_mega_stats *stats);

/* ---- tree updates: usage, block GC, grafting, pruning --------------------- */

/* Groups are the 8-node block groups (one svo_usage each). Dense-real groups
 * (the level-B+2 nodes under air+geometry level-(B+1) cells) are never
 * allocated or freed; every other group below the budget is allocatable. */
typedef struct svo_gc_report {
  uint64_t pruned; /* stale groups detached from their parent this call */
  uint64_t freed;  /* groups that became free (unreachable) this call */
  uint64_t free;   /* allocatable groups free after the call (the free list) */
} svo_gc_report;

typedef struct svo_graft_report {
  uint32_t applied;  /* records grafted */
  uint32_t skipped;  /* records skipped: bad payload range, missing target, or not enough free groups */
  uint64_t claimed;  /* groups claimed from the free list */
  uint64_t free_left;
} svo_graft_report;

typedef struct svo_prune_report {
  uint64_t freed;    /* groups freed because CullChild orphaned them */
  uint32_t requests; /* child requests raised by Location walks that met a missing child */
  uint32_t _pad;
} svo_prune_report;

/* Streaming usage initialisation (no reference counterpart; the reference's
 * rule is svo_init_usage): dense-real groups become inviolate, every group
 * reachable through Child pointers gets {tick, parent node}, all others are
 * free. */
SVO_API svo_status svo_init_usage_tree(void *ctx, uint16_t tick);
/* Block GC (the claim loop of graft, wavefront.cl:1279-1305): groups whose
 * tick is older than in->offset ticks (wrapping tick space 1..65533, now =
 * in->tick) are detached from their parent; every allocated group that is no
 * longer reachable is freed; the free groups form an ascending free list that
 * svo_graft consumes. */
SVO_API svo_status svo_gc(void *ctx, const svo_update_input *in, svo_gc_report *report);
/* The pruned, freed and free-list group indices of the last svo_gc (or of the
 * sweep of the last svo_prune / svo_graft). */
SVO_API svo_status svo_read_gc_lists(void *ctx, uint32_t *pruned, size_t cap_pruned, uint32_t *freed,
                                     size_t cap_freed, uint32_t *free_list, size_t cap_free);
/* Grafting (wavefront.cl:1306-1350, Grafting :38-43): records in order claim
 * graft_total_size groups from the free list; payload group k (blocks
 * graft_data_address + 8k .. +7, children given as payload block indices)
 * becomes claimed group k; the target node (graft_address, or the Location
 * graft_address of `locations` walked to `depth` when depth != 255) points at
 * the first claimed group. Targets must be distinct. */
SVO_API svo_status svo_graft(void *ctx, const svo_update_input *in, const svo_grafting *records, uint32_t n_records,
                             const svo_block *payload, size_t n_payload, const uint64_t *locations,
                             size_t n_locations, svo_graft_report *report);
SVO_API svo_status svo_read_graft_claims(void *ctx, uint32_t *claimed, size_t cap);
/* The child requests of the last trace answered on the device: the payload
 * svo_scene_graft_payload builds for them from `scene` (a terrain scene;
 * WorldManager.UpdateGrafting's generator, SvoTracer.Window/WorldManager.cs:
 * 84-103), grafted with svo_graft's rules and the same result node for node,
 * without reading the requests back or sending a payload. The scene's column
 * height pyramids are copied to the device on the first call with a scene. */
SVO_API svo_status svo_graft_generate(void *ctx, void *scene, const svo_update_input *in, svo_graft_report *report);
/* Pruning records (wavefront.cl:1215-1266, Pruning :24-36) applied in order;
 * groups orphaned by CullChild are freed afterwards. Child requests of
 * Location walks that meet a missing child go to the context's request queue. */
SVO_API svo_status svo_prune(void *ctx, const svo_update_input *in, const svo_pruning *records, uint32_t n_records,
                             const svo_block *surface, size_t n_surface, const uint64_t *locations,
                             size_t n_locations, svo_prune_report *report);

/* ---- differentiable colour fitting (no reference counterpart) ------------ */

/* Per-node RGBA parameters (4 floats per node, nodes 0..n_nodes-1 of the
 * resident tree; n_nodes <= the block budget, missing nodes are zero). A ray
 * composites the parameters of its LOD hits front to back (C += T a rgb,
 * T *= 1 - a), continuing past each hit, up to max_hits hits, then the sky
 * colour times the remaining transmittance. The geometry (and so the hit
 * sequence) is fixed. Pointers are device memory when on_device != 0. */
SVO_API svo_status svo_diff_set_params(void *ctx, const float *rgba, size_t n_nodes, int32_t on_device);
/* Gradients of the last svo_diff_backward, 4 floats per node. */
SVO_API svo_status svo_diff_get_grads(void *ctx, float *grad_rgba, size_t n_nodes, int32_t on_device);
/* Composited colour, 3 floats per ray, views concatenated in order (a pinned
 * host buffer is written by the kernel directly). */
SVO_API svo_status svo_diff_forward(void *ctx, const svo_trace_input *views, int32_t n_views, float *rgb,
                                    int32_t on_device);
/* L = sum over rays and channels of (C - target)^2 / rays; recomputes the
 * traversal (no per-ray hit lists are stored) and writes dL/d(params) into the
 * gradient buffer. use_saved != 0 takes C from the last svo_diff_forward
 * (which must have run on the same views, parameters and max_hits, else
 * SVO_ERR_INVALID_ARGUMENT): one traversal per ray instead of two. *loss (may
 * be NULL: no synchronisation) receives L. */
SVO_API svo_status svo_diff_backward(void *ctx, const svo_trace_input *views, int32_t n_views, const float *target,
                                     int32_t use_saved, int32_t on_device, double *loss);

/* ---- tracing without allocation ------------------------------------------ */

/* No counterpart in the reference. For callers that cannot allocate device
 * memory (an engine that owns every GPU allocation through its own pool, a
 * real-time host loop where cudaMalloc's synchronisation and latency are not
 * allowed): traces one view of a tree the caller keeps in device memory
 * (bases, blocks, usage) into caller-owned device outputs (out->on_device must
 * be 1) and, optionally, a caller-owned child-request array. The call makes no
 * cudaMalloc/cudaFree and needs no context: its scratch (queue counters, error
 * record, view record, ray tables) is a 132 KiB static device array inside
 * libsvo, so views are limited to width + height <= 16384. Every GPU that
 * loads the library holds that array until the process exits. All calls share
 * it: calls whose work overlaps on the GPU race and must not be issued. The
 * first call on a device looks up the array's device address; make it before
 * any stream capture. max_node_depth = deepest node level (0 = 24). The call
 * returns after the trace completed on `stream`; *requests_raised (if not
 * NULL) receives the number of child requests raised. */
SVO_API svo_status svo_trace_noalloc(int32_t device, void *stream, uint8_t base_depth, const uint16_t *bases,
                                     size_t n_bases, const svo_block *blocks, size_t n_blocks, svo_usage *usage,
                                     size_t n_groups, int32_t max_node_depth, const svo_trace_input *input,
                                     const svo_trace_output *out, svo_child_request *requests, uint32_t request_cap,
                                     uint32_t *requests_raised);

/* ---- procedural scenes and the tree builder (host) ----------------------- */

enum { SVO_SCENE_SPHERE = 0, SVO_SCENE_TERRAIN = 1 };

typedef struct svo_scene_params {
  int32_t kind;
  uint32_t seed;
  uint8_t base_depth;
  uint8_t max_depth;  /* deepest node level */
  uint8_t _pad[2];
  int32_t threads;    /* 0 = all cores */
  uint64_t max_size;  /* node capacity (TreeBuilder maxSize); 0 = UINT32_MAX/64 */
} svo_scene_params;

/* Replaces ITreeBuilder.BuildTree (SvoTracer.Domain/TreeBuilder.cs:102-150). */
SVO_API svo_status svo_tree_build(const svo_scene_params *params, void **tree);
SVO_API svo_status svo_tree_info(void *tree, uint8_t *base_depth, size_t *n_bases, size_t *n_blocks,
                                 uint32_t *block_count);
SVO_API svo_status svo_tree_data(void *tree, const uint16_t **bases, const svo_block **blocks);
SVO_API svo_status svo_tree_free(void *tree);

/* The .oct tree file of OctreeSerializer (SvoTracer.Domain/Serializers/
 * OctreeSerializer.cs:13-45, BlockSerializer.cs), little-endian: BaseDepth (1
 * byte), BlockCount (uint32), powSum(BaseDepth) base chunks (uint16 each),
 * then 16-byte blocks. svo_oct_write writes every block given (the reference
 * writes its whole Blocks array); svo_oct_read reads BlockCount blocks and
 * ignores anything after them, like the reference's Deserialize, and returns a
 * tree handle for svo_tree_info / svo_tree_data / svo_tree_free (TreeManager.
 * SaveTree / LoadTree, SvoTracer.Domain/TreeManager.cs:29-58). */
SVO_API svo_status svo_oct_write(const char *path, uint8_t base_depth, uint32_t block_count, const uint16_t *bases,
                                 size_t n_bases, const svo_block *blocks, size_t n_blocks);
SVO_API svo_status svo_oct_read(const char *path, void **tree);

/* Streaming-state snapshot (checkpoint / resume). svo_state_save writes, after
 * the context's pending work, everything later frames depend on: the base
 * chunks, every block of the budget (grafted groups included), the usage
 * array, the depth the tree has grown to, and the free list of the last GC with
 * the part grafts have claimed. svo_state_load replaces the context's resident
 * tree with a saved state (its own budget); the frames that follow (the caller
 * keeps the tick) give what they would have given in the saved context.
 * SVO_ERR_IO for a file that cannot be read or written or is truncated,
 * SVO_ERR_INVALID_ARGUMENT for one that is not a consistent state file. The
 * reference persists only the octree (.oct). */
SVO_API svo_status svo_state_save(void *ctx, const char *path);
SVO_API svo_status svo_state_load(void *ctx, const char *path);

/* A persistent scene: the tree builder and the graft payload source of the
 * streaming workflow (the host-side procedural generator behind
 * WorldManager.UpdateGrafting, SvoTracer.Window/WorldManager.cs:84-103).
 * params->max_depth is the deepest node level the scene can produce. */
SVO_API svo_status svo_scene_create(const svo_scene_params *params, void **scene);
SVO_API svo_status svo_scene_build_tree(void *scene, uint8_t max_depth, void **tree);
/* One Grafting record per distinct requesting node (ascending address): its
 * children, and their children when a request asked for TreeSize 1, with
 * payload-relative child indices; feed the result to svo_graft. */
SVO_API svo_status svo_scene_graft_payload(void *scene, const svo_child_request *requests, size_t n, void **graft);
SVO_API svo_status svo_graft_payload_data(void *graft, const svo_grafting **records, size_t *n_records,
                                          const svo_block **payload, size_t *n_payload);
SVO_API svo_status svo_graft_payload_free(void *graft);
SVO_API svo_status svo_scene_free(void *scene);

#ifdef __cplusplus
} /* extern "C" */
#endif

#ifdef __cplusplus
static_assert(sizeof(svo_block) == 16, "Block is 16 bytes");
static_assert(sizeof(svo_usage) == 8, "Usage is 8 bytes");
static_assert(sizeof(svo_trace_input) == 104, "TraceInput is 104 bytes");
static_assert(sizeof(svo_update_input) == 20, "UpdateInputData is 20 bytes");
static_assert(sizeof(svo_pruning) == 20, "Pruning is 20 bytes");
static_assert(sizeof(svo_grafting) == 16, "Grafting is 16 bytes");
static_assert(sizeof(svo_child_request) == 40, "ChildRequest is 40 bytes");
#else
_Static_assert(sizeof(svo_block) == 16, "Block is 16 bytes");
_Static_assert(sizeof(svo_usage) == 8, "Usage is 8 bytes");
_Static_assert(sizeof(svo_trace_input) == 104, "TraceInput is 104 bytes");
_Static_assert(sizeof(svo_update_input) == 20, "UpdateInputData is 20 bytes");
_Static_assert(sizeof(svo_pruning) == 20, "Pruning is 20 bytes");
_Static_assert(sizeof(svo_grafting) == 16, "Grafting is 16 bytes");
_Static_assert(sizeof(svo_child_request) == 40, "ChildRequest is 40 bytes");
#endif

#endif /* SVO_H */
