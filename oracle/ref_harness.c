/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's own wavefront kernels (oracle/_ref/wavefront_ref.c,
 * generated from SvoTracer/SvoTracer.Kernel/wavefront.cl by build_ref.py) on
 * the CPU, driven the way SvoTracer.Window/MainWindow.cs:356-622 drives them:
 * zero the queue counters, init over W x H, alternate runBaseTrace and
 * runBlockTrace passes over double-buffered queues until both are empty, then
 * evaluateBackground, resolveRemainders and drawTrace (into a float buffer in
 * place of the GL renderbuffer). Each pass runs its work-items in parallel
 * (work-groups of one item, real atomics on the shared counters).
 */
#include "_ref/wavefront_ref.c"

#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

_Static_assert(sizeof(TraceInput) == 104, "TraceInput layout");
_Static_assert(sizeof(Block) == 16, "Block layout");
_Static_assert(sizeof(Usage) == 8, "Usage layout");
_Static_assert(sizeof(ChildRequest) == 40, "ChildRequest layout");

_Thread_local size_t ref_gid[2];
size_t ref_gsize[2];
uint ref_image_width;

static void *zalloc(size_t n) { return calloc(n ? n : 1, 1); }

/* Returns the number of traversal passes, or -1 if max_passes ran out.
 * Only rows [row_begin, row_end) get an init work-item (a bounded sample of the
 * view); per-pixel outputs still cover the whole W x H image. */
long ref_trace_rows(const ushort *bases, uchar base_depth, const Block *blocks_in, size_t n_blocks, Usage *usage,
                    size_t n_groups, const TraceInput *in, uint *hit_index, uchar *hit_depth, float *t, float *rgba,
                    uint *acc, ChildRequest *req_out, uint req_cap, uint *n_req, int threads, long max_passes,
                    uint row_begin, uint row_end) {
  (void)n_groups;
  TraceInput input = *in;
  input.BaseDepth = base_depth;
  size_t W = input.ScreenSize[0], H = input.ScreenSize[1], N = W * H;
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
#endif
  /* Kernels take non-const pointers; the tree is not modified by a trace. */
  Block *Blocks = (Block *)blocks_in;
  ushort *Bases = (ushort *)bases;
  Usage *Usages = usage ? usage : (Usage *)zalloc(sizeof(Usage) * (n_blocks / 8 + 1));
  float3 *Origins = zalloc(sizeof(float3) * N), *Directions = zalloc(sizeof(float3) * N);
  float *FoVs = zalloc(sizeof(float) * N);
  ulong3 *Locations = zalloc(sizeof(ulong3) * N);
  uchar *Depths = zalloc(N), *Weightings = zalloc(N), *ColourRs = zalloc(N), *ColourGs = zalloc(N),
        *ColourBs = zalloc(N);
  uint *ParentTraces = zalloc(4 * N), *BaseTraces = zalloc(4 * N), *BaseTraceQueue = zalloc(4 * N),
       *BlockTraces = zalloc(4 * N), *BlockTraceQueue = zalloc(4 * N), *BackgroundQueue = zalloc(4 * N),
       *MaterialQueue = zalloc(4 * N);
  uint *FinalColourRs = zalloc(4 * N), *FinalColourGs = zalloc(4 * N), *FinalColourBs = zalloc(4 * N),
       *FinalWeightings = zalloc(4 * N);
  ChildRequest *ChildRequests = zalloc(sizeof(ChildRequest) * N);
  uint BaseTraceQueueID = 0, BlockTraceQueueID = 0, BackgroundQueueID = 0, MaterialQueueID = 0, ChildRequestID = 0;
  float *image = rgba ? rgba : zalloc(sizeof(float) * 4 * N);
  ref_image_width = (uint)W;
  long passes = 0;

  ref_gsize[0] = W;
  ref_gsize[1] = H;
  if (row_end > H) row_end = (uint)H;
  if (row_begin > row_end) row_begin = row_end;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
  for (size_t id = (size_t)row_begin * W; id < (size_t)row_end * W; id++) {
    ref_gid[0] = id % W;
    ref_gid[1] = id / W;
    init(Origins, Directions, FoVs, Locations, Depths, BaseTraceQueue, &BaseTraceQueueID, BackgroundQueue,
         &BackgroundQueueID, ParentTraces, ColourRs, ColourGs, ColourBs, Weightings, FinalColourRs, FinalColourGs,
         FinalColourBs, FinalWeightings, input);
  }

  for (;;) { /* MainWindow.RunTraces, MainWindow.cs:452-481 */
    uint nb = BaseTraceQueueID;
    BaseTraceQueueID = 0;
    if (nb) {
      uint *tmp = BaseTraces;
      BaseTraces = BaseTraceQueue;
      BaseTraceQueue = tmp;
      ref_gsize[0] = nb;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
      for (size_t i = 0; i < nb; i++) {
        ref_gid[0] = i;
        ref_gid[1] = 0;
        runBaseTrace(Bases, Origins, Directions, FoVs, Locations, Weightings, Depths, BaseTraces, BlockTraceQueue,
                     &BlockTraceQueueID, BaseTraceQueue, &BaseTraceQueueID, BackgroundQueue, &BackgroundQueueID, input);
      }
    }
    uint nk = BlockTraceQueueID;
    BlockTraceQueueID = 0;
    if (nk) {
      uint *tmp = BlockTraces;
      BlockTraces = BlockTraceQueue;
      BlockTraceQueue = tmp;
      ref_gsize[0] = nk;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
      for (size_t i = 0; i < nk; i++) {
        ref_gid[0] = i;
        ref_gid[1] = 0;
        runBlockTrace(Blocks, Usages, &ChildRequestID, ChildRequests, Origins, Directions, FoVs, Locations,
                      Weightings, Depths, BlockTraces, BlockTraceQueue, &BlockTraceQueueID, BaseTraceQueue,
                      &BaseTraceQueueID, BackgroundQueue, &BackgroundQueueID, MaterialQueue, &MaterialQueueID,
                      ParentTraces, input);
      }
    }
    if (!nb && !nk) break;
    if (++passes > max_passes) {
      passes = -1;
      break;
    }
  }

  TraceInput flat = input; /* MainWindow.cs:384-385: DoF zeroed after the traces */
  flat.DoF[0] = 0;
  flat.DoF[1] = 0;
  uint nbg = BackgroundQueueID;
  ref_gsize[0] = nbg;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
  for (size_t i = 0; i < nbg; i++) {
    ref_gid[0] = i;
    evaluateBackground(BackgroundQueue, Directions, ParentTraces, ColourRs, ColourGs, ColourBs, Weightings,
                       FinalColourRs, FinalColourGs, FinalColourBs, FinalWeightings, flat);
  }
  uint nm = MaterialQueueID;
  ref_gsize[0] = nm;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
  for (size_t i = 0; i < nm; i++) {
    ref_gid[0] = i;
    resolveRemainders(Blocks, Usages, Locations, Depths, MaterialQueue, FinalColourRs, FinalColourGs, FinalColourBs,
                      FinalWeightings, Weightings, ParentTraces, flat);
  }
  ref_gsize[0] = W;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
  for (size_t id = 0; id < N; id++) {
    ref_gid[0] = id % W;
    ref_gid[1] = id / W;
    drawTrace(FinalColourRs, FinalColourGs, FinalColourBs, FinalWeightings, image, flat);
  }

  /* Per-pixel hit node and distance, from the material rays' final state. */
  for (size_t id = 0; id < N; id++) {
    if (hit_index) hit_index[id] = 0xFFFFFFFFu;
    if (hit_depth) hit_depth[id] = 0;
    if (t) t[id] = INFINITY;
  }
  Buffers walk = {.Blocks = Blocks, .BaseDepth = base_depth};
  for (size_t i = 0; i < nm; i++) {
    uint id = MaterialQueue[i];
    uint px = ParentTraces[id];
    if (hit_index) hit_index[px] = getBlockAddress(walk, Depths[id], Locations[id]);
    if (hit_depth) hit_depth[px] = Depths[id];
    if (t) {
      float x = ulongToFloat(Locations[id][0]) - Origins[id][0];
      float y = ulongToFloat(Locations[id][1]) - Origins[id][1];
      float z = ulongToFloat(Locations[id][2]) - Origins[id][2];
      t[px] = sqrtf(x * x + y * y + z * z);
    }
  }
  if (acc)
    for (size_t id = 0; id < N; id++) {
      acc[4 * id + 0] = FinalWeightings[id];
      acc[4 * id + 1] = FinalColourRs[id];
      acc[4 * id + 2] = FinalColourGs[id];
      acc[4 * id + 3] = FinalColourBs[id];
    }
  if (n_req) *n_req = ChildRequestID;
  if (req_out) memcpy(req_out, ChildRequests, sizeof(ChildRequest) * (ChildRequestID < req_cap ? ChildRequestID : req_cap));

  if (!usage) free(Usages);
  if (!rgba) free(image);
  free(Origins); free(Directions); free(FoVs); free(Locations); free(Depths); free(Weightings);
  free(ColourRs); free(ColourGs); free(ColourBs); free(ParentTraces); free(BaseTraces); free(BaseTraceQueue);
  free(BlockTraces); free(BlockTraceQueue); free(BackgroundQueue); free(MaterialQueue); free(FinalColourRs);
  free(FinalColourGs); free(FinalColourBs); free(FinalWeightings); free(ChildRequests);
  return passes;
}

long ref_trace_view(const ushort *bases, uchar base_depth, const Block *blocks_in, size_t n_blocks, Usage *usage,
                    size_t n_groups, const TraceInput *in, uint *hit_index, uchar *hit_depth, float *t, float *rgba,
                    uint *acc, ChildRequest *req_out, uint req_cap, uint *n_req, int threads, long max_passes) {
  return ref_trace_rows(bases, base_depth, blocks_in, n_blocks, usage, n_groups, in, hit_index, hit_depth, t, rgba, acc,
                        req_out, req_cap, n_req, threads, max_passes, 0, in->ScreenSize[1]);
}
