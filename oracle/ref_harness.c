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
_Static_assert(sizeof(Pruning) == 20, "Pruning layout");
_Static_assert(sizeof(UpdateInputData) == 20, "UpdateInputData layout");

_Thread_local size_t ref_gid[2];
size_t ref_gsize[2];
uint ref_image_width;

static void *zalloc(size_t n) { return calloc(n ? n : 1, 1); }

/* Cones per pixel of a fan that takes no `break` (evaluateMaterial's spine
 * and ring loops, wavefront.cl:1655-1739, which depend only on the input): 0
 * when the kernel returns at once, -1 past 4096 (the loops would not end). */
static long gi_max_cones(const TraceInput *in) {
  if (in->FovConstant <= 0 || in->FovMultiplier >= 1 || in->FovMultiplier <= -1) return 0;
  float fov = in->FovConstant, oldfov = fov, spineAngle = 0;
  long cones = 1;
  while (spineAngle < M_PI_F) {
    fov = (in->FovMultiplier * (spineAngle + fov) + in->FovConstant) / (1 - in->FovMultiplier);
    spineAngle = (1 + in->FovMultiplier) * (spineAngle + oldfov) / (1 - in->FovMultiplier);
    oldfov = fov;
    cones += 1;
    for (int j = 1; j * fov < M_PI_2_F; j++)
      if ((cones += 2) > 4096) return -1;
    if (cones > 4096) return -1;
  }
  return cones;
}

static void *grow(void *p, size_t old_bytes, size_t new_bytes) {
  if (new_bytes <= old_bytes) return p;
  void *q = realloc(p, new_bytes);
  memset((char *)q + old_bytes, 0, new_bytes - old_bytes);
  return q;
}

/* Returns the number of traversal passes, or -1 if max_passes ran out (-2: the
 * material stage's cone loops would not end). Only rows [row_begin, row_end) get
 * an init work-item (a bounded sample of the view); per-pixel outputs still
 * cover the whole W x H image. gi = 1 also runs the secondary-cone stage that
 * MainWindow.RunWavefront has commented out (MainWindow.cs:390-402), as written
 * there: EvaulateMaterial (swap the Root buffers, reset the material queue,
 * evaluateMaterial), RunTraces, EvaulateBackground. */
long ref_trace_rows_gi(const ushort *bases, uchar base_depth, const Block *blocks_in, size_t n_blocks, Usage *usage,
                       size_t n_groups, const TraceInput *in, uint *hit_index, uchar *hit_depth, float *t, float *rgba,
                       uint *acc, ChildRequest *req_out, uint req_cap, uint *n_req, int threads, long max_passes,
                       uint row_begin, uint row_end, int gi) {
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

#define RUN_TRACES(INPUT)\
  for (;;) { /* MainWindow.RunTraces, MainWindow.cs:452-481 */ \
    uint nb = BaseTraceQueueID; \
    BaseTraceQueueID = 0; \
    if (nb) { \
      uint *tmp = BaseTraces; \
      BaseTraces = BaseTraceQueue; \
      BaseTraceQueue = tmp; \
      ref_gsize[0] = nb; \
      _Pragma("omp parallel for schedule(dynamic, 1024) num_threads(nt)") \
      for (size_t i = 0; i < nb; i++) { \
        ref_gid[0] = i; \
        ref_gid[1] = 0; \
        runBaseTrace(Bases, Origins, Directions, FoVs, Locations, Weightings, Depths, BaseTraces, BlockTraceQueue, \
                     &BlockTraceQueueID, BaseTraceQueue, &BaseTraceQueueID, BackgroundQueue, &BackgroundQueueID, INPUT); \
      } \
    } \
    uint nk = BlockTraceQueueID; \
    BlockTraceQueueID = 0; \
    if (nk) { \
      uint *tmp = BlockTraces; \
      BlockTraces = BlockTraceQueue; \
      BlockTraceQueue = tmp; \
      ref_gsize[0] = nk; \
      _Pragma("omp parallel for schedule(dynamic, 1024) num_threads(nt)") \
      for (size_t i = 0; i < nk; i++) { \
        ref_gid[0] = i; \
        ref_gid[1] = 0; \
        runBlockTrace(Blocks, Usages, &ChildRequestID, ChildRequests, Origins, Directions, FoVs, Locations, \
                      Weightings, Depths, BlockTraces, BlockTraceQueue, &BlockTraceQueueID, BaseTraceQueue, \
                      &BaseTraceQueueID, BackgroundQueue, &BackgroundQueueID, MaterialQueue, &MaterialQueueID, \
                      ParentTraces, INPUT); \
      } \
    } \
    if (!nb && !nk) break; \
    if (++passes > max_passes) { \
      passes = -1; \
      break; \
    } \
  }
  RUN_TRACES(input);
  TraceInput flat = input; /* MainWindow.cs:384-385: DoF zeroed after the traces */
  flat.DoF[0] = 0;
  flat.DoF[1] = 0;
  uint nbg = BackgroundQueueID;
  BackgroundQueueID = 0; /* EvaulateBackground's ResetIDBuffer */
  ref_gsize[0] = nbg;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
  for (size_t i = 0; i < nbg; i++) {
    ref_gid[0] = i;
    evaluateBackground(BackgroundQueue, Directions, ParentTraces, ColourRs, ColourGs, ColourBs, Weightings,
                       FinalColourRs, FinalColourGs, FinalColourBs, FinalWeightings, flat);
  }
  /* the primary states of the material queue (hit outputs below) */
  uint n_hits = MaterialQueueID;
  ulong3 *HitLocations = Locations;
  uchar *HitDepths = Depths;
  uint *HitParents = ParentTraces;
  ulong3 *RootLocations = NULL;
  float3 *RootDirections = NULL;
  uchar *RootDepths = NULL, *RootWeightings = NULL, *Luminosities = NULL;
  uint *RootParentTraces = NULL;
  float *RayLengths = NULL;
  if (gi && passes >= 0) {
    long K = gi_max_cones(&flat);
    if (K < 0) {
      passes = -2;
    } else {
      /* EvaulateMaterial (MainWindow.cs:529-560): the Root buffers swap with the
       * traces' state buffers, then the material queue count is read and reset */
      size_t cap = (size_t)n_hits * (size_t)(K > 0 ? K : 1) + 1;
      if (cap < N) cap = N;
      RootDirections = zalloc(sizeof(float3) * cap);
      RootLocations = zalloc(sizeof(ulong3) * cap);
      RootDepths = zalloc(cap);
      RootWeightings = zalloc(cap);
      RootParentTraces = zalloc(4 * cap);
      float3 *t3 = Directions; Directions = RootDirections; RootDirections = t3;
      ulong3 *tl = Locations; Locations = RootLocations; RootLocations = tl;
      uchar *tc = Depths; Depths = RootDepths; RootDepths = tc;
      tc = Weightings; Weightings = RootWeightings; RootWeightings = tc;
      uint *tu = ParentTraces; ParentTraces = RootParentTraces; RootParentTraces = tu;
      HitLocations = RootLocations;
      HitDepths = RootDepths;
      HitParents = RootParentTraces;
      /* saveAccumulator writes these at the cone ids too */
      Origins = grow(Origins, sizeof(float3) * N, sizeof(float3) * cap);
      FoVs = grow(FoVs, sizeof(float) * N, sizeof(float) * cap);
      ColourRs = grow(ColourRs, N, cap);
      ColourGs = grow(ColourGs, N, cap);
      ColourBs = grow(ColourBs, N, cap);
      BackgroundQueue = grow(BackgroundQueue, 4 * N, 4 * cap);
      Luminosities = zalloc(cap);
      RayLengths = zalloc(sizeof(float) * cap);
      uint AccumulatorID = 0;
      uint nmat = MaterialQueueID;
      MaterialQueueID = 0;
      ref_gsize[0] = nmat;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
      for (size_t i = 0; i < nmat; i++) {
        ref_gid[0] = i;
        evaluateMaterial(Blocks, Usages, Origins, Directions, FoVs, Locations, Depths, Weightings, ColourRs, ColourGs,
                         ColourBs, RayLengths, Luminosities, MaterialQueue, ParentTraces, RootDirections,
                         RootLocations, RootDepths, RootWeightings, RootParentTraces, BaseTraceQueue,
                         &BaseTraceQueueID, FinalWeightings, &AccumulatorID, BackgroundQueue, &BackgroundQueueID,
                         flat);
      }
      RUN_TRACES(flat); /* the material rays' traces: every queue is empty */
      uint nbg2 = BackgroundQueueID;
      BackgroundQueueID = 0;
      ref_gsize[0] = nbg2;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nt)
#endif
      for (size_t i = 0; i < nbg2; i++) {
        ref_gid[0] = i;
        evaluateBackground(BackgroundQueue, Directions, ParentTraces, ColourRs, ColourGs, ColourBs, Weightings,
                           FinalColourRs, FinalColourGs, FinalColourBs, FinalWeightings, flat);
      }
    }
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
  for (size_t i = 0; i < n_hits; i++) {
    uint id = MaterialQueue[i];
    uint px = HitParents[id];
    if (hit_index) hit_index[px] = getBlockAddress(walk, HitDepths[id], HitLocations[id]);
    if (hit_depth) hit_depth[px] = HitDepths[id];
    if (t) { /* a primary ray's Origin is the camera's */
      float x = ulongToFloat(HitLocations[id][0]) - input.Origin[0];
      float y = ulongToFloat(HitLocations[id][1]) - input.Origin[1];
      float z = ulongToFloat(HitLocations[id][2]) - input.Origin[2];
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
  free(RootDirections); free(RootLocations); free(RootDepths); free(RootWeightings); free(RootParentTraces);
  free(Luminosities); free(RayLengths);
  return passes;
}
#undef RUN_TRACES

long ref_trace_rows(const ushort *bases, uchar base_depth, const Block *blocks_in, size_t n_blocks, Usage *usage,
                    size_t n_groups, const TraceInput *in, uint *hit_index, uchar *hit_depth, float *t, float *rgba,
                    uint *acc, ChildRequest *req_out, uint req_cap, uint *n_req, int threads, long max_passes,
                    uint row_begin, uint row_end) {
  return ref_trace_rows_gi(bases, base_depth, blocks_in, n_blocks, usage, n_groups, in, hit_index, hit_depth, t, rgba,
                           acc, req_out, req_cap, n_req, threads, max_passes, row_begin, row_end, 0);
}

long ref_trace_view(const ushort *bases, uchar base_depth, const Block *blocks_in, size_t n_blocks, Usage *usage,
                    size_t n_groups, const TraceInput *in, uint *hit_index, uchar *hit_depth, float *t, float *rgba,
                    uint *acc, ChildRequest *req_out, uint req_cap, uint *n_req, int threads, long max_passes) {
  return ref_trace_rows(bases, base_depth, blocks_in, n_blocks, usage, n_groups, in, hit_index, hit_depth, t, rgba, acc,
                        req_out, req_cap, n_req, threads, max_passes, 0, in->ScreenSize[1]);
}

/* ---- prune (wavefront.cl:1215-1266) ------------------------------------------
 *
 * Runs the reference's own prune kernel over n records in record order, one
 * work-item at a time (x = record index), on a single-parent tree (no usage
 * tick 65534, so the Parent list is never read; the parent arrays passed are
 * dummies).
 *
 * The kernel can only run faithfully where its dereference queue stays empty
 * and findAddress meets no missing child:
 *  - helpDereference pops with atomic_dec's old value, one slot past the last
 *    push (push writes slot n and increments; pop reads slot n and decrements),
 *    so any push is followed by a pop of an unwritten slot. With the queue count
 *    at -1 before a record (the host initialises it to 0, MainWindow.cs:86, which
 *    makes even an empty queue pop slot 0), a record that pushes nothing leaves
 *    the queue untouched. A CullChild whose grandchild groups would be queued is
 *    therefore refused here.
 *  - findAddress's requestChild writes through an uninitialised Buffers
 *    (wavefront.cl:1203-1204), so a Location record whose walk meets a missing
 *    child is refused too.
 * The producer (WorldManager.UpdatePruning, WorldManager.cs:66-82) stores
 * ColourAddress as an index into the surface blocks and Address as a Location
 * index; the kernel reads pruningSurfaceData[x] and addresses[Address + k]
 * (ulongs). Each record is run with arrays arranged so that those reads return
 * the producer's entries: a surface array whose entry x is
 * surface[ColourAddress], and a ulong array whose entries Address..Address+2 are
 * Location Address. A refused record is not run, and nothing after it.
 * Returns n, or -(x + 1) for the first refused record x. */
long ref_prune(ushort *bases, uchar base_depth, Block *blocks, size_t n_blocks, Usage *usage, size_t n_groups,
               const Pruning *records, uint n, const Block *surface, size_t n_surface, const ulong *locations,
               size_t n_locations, ushort tick) {
  uint child_request_id = 0;
  ChildRequest request_sink[4];
  uint parent_size[1] = {0};
  bool parent_residency[1] = {false};
  Parent parents[1] = {{UINT_MAX, UINT_MAX}};
  uint2 queue[8];
  int semaphor = 0;
  UpdateInputData in;
  memset(&in, 0, sizeof(in));
  in.BaseDepth = base_depth;
  in.Tick = tick;
  Block *surf_by_x = zalloc(sizeof(Block) * (n ? n : 1));
  long result = n;
  for (uint x = 0; x < n; x++) {
    const Pruning *p = &records[x];
    if (((p->Properties >> 3) & 1) && p->ColourAddress < n_surface) surf_by_x[x] = surface[p->ColourAddress];
    ulong *loc_words = NULL;
    uint target = p->Address;
    if (!((p->Properties >> 4) & 1)) {
      if (p->Depth != UCHAR_MAX) {
        if ((size_t)p->Address * 3 + 3 > n_locations) {
          result = -(long)x - 1;
          break;
        }
        loc_words = zalloc(sizeof(ulong) * ((size_t)p->Address + 3));
        for (int k = 0; k < 3; k++) loc_words[p->Address + k] = locations[3 * (size_t)p->Address + k];
        ulong3 location = {loc_words[p->Address], loc_words[p->Address + 1], loc_words[p->Address + 2], 0};
        uint a = baseLocation(base_depth + 2, location);
        int missing = 0;
        for (uchar i = base_depth + 2; i < p->Depth; i++) {
          if (a >= n_blocks || blocks[a].Child == UINT_MAX) {
            missing = 1;
            break;
          }
          a = blocks[a].Child + chunkPosition(i, location);
        }
        if (missing || a >= n_blocks) {
          free(loc_words);
          result = -(long)x - 1;
          break;
        }
        target = a;
      } else if (target >= n_blocks || (size_t)(target >> 3) >= n_groups) {
        result = -(long)x - 1;
        break;
      }
      int live = p->Depth != UCHAR_MAX || usage[target >> 3].Tick != 0;
      if (live && (p->Properties & 1) && blocks[target].Child != UINT_MAX) {
        uint c0 = blocks[target].Child;
        int pushes = 0;
        for (uint i = 0; i < 8; i++) {
          uint c = c0 + i < n_blocks ? blocks[c0 + i].Child : UINT_MAX;
          if (c != UINT_MAX && usage[c >> 3].Tick < USHRT_MAX) pushes = 1;
        }
        if (pushes) {
          free(loc_words);
          result = -(long)x - 1;
          break;
        }
      }
    }
    int remaining = -1;
    ref_gid[0] = x;
    ref_gid[1] = 0;
    prune(bases, blocks, usage, &child_request_id, request_sink, parent_size, parent_residency, parents, queue,
          &remaining, &semaphor, (Pruning *)records, surf_by_x, loc_words ? loc_words : (ulong *)locations, in);
    free(loc_words);
    if (remaining != -2 || semaphor != 0) { /* the queue was used after all */
      result = -(long)x - 1;
      break;
    }
  }
  free(surf_by_x);
  return result;
}
