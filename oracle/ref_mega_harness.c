/*
 * ref_mega_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's megakernel (oracle/_ref/kernel_ref.c, generated from
 * SvoTracer/SvoTracer.Kernel/kernel.cl by build_ref.py) on the CPU: one call of
 * its `trace` kernel per pixel, as an Enqueue of `trace` over W x H would run it
 * (the kernel.cl build of SvoTracer.Window/MainWindow.cs:45), writing a float
 * RGBA buffer in place of the GL image. Work-items run in parallel on host
 * threads; the child-request counter is a real atomic.
 */
#include "_ref/kernel_ref.c"

#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

_Static_assert(sizeof(TraceInput) == 96, "TraceInput layout (kernel.cl)");
_Static_assert(sizeof(Block) == 16, "Block layout");
_Static_assert(sizeof(Usage) == 8, "Usage layout");
_Static_assert(sizeof(ChildRequest) == 40, "ChildRequest layout");

_Thread_local size_t ref_gid[2];
size_t ref_gsize[2];
uint ref_image_width;

/* Traces one pixel can run: the primary ray plus spawnRays's cones
 * (kernel.cl:1115-1253) when no `break` is taken. Each trace pushes at most one
 * child request, which sizes the request buffer (kernel.cl's requestChild has no
 * bound). Returns 0 when the cone schedule has more than `limit` entries. */
static size_t traces_bound(const TraceInput *in, size_t limit) {
  float fov = in->FovConstant, oldfov = fov, spine = 0.0f;
  size_t n = 2; /* primary, reflection cone */
  while (spine < M_PI_F) {
    fov = (in->FovMultiplier * (spine + fov) + in->FovConstant) / (1 - in->FovMultiplier);
    spine = (1 + in->FovMultiplier) * (spine + oldfov) / (1 - in->FovMultiplier);
    oldfov = fov;
    n += 1;
    for (int j = 1; j * fov < M_PI_2_F; j++) {
      n += 2;
      if (n > limit) return 0;
    }
    if (n > limit) return 0;
  }
  return n;
}

/* The megakernel over rows [row_begin, row_end) of a view (rgba covers the whole
 * image; other rows are left as they are). `in` points at the 96 bytes of
 * kernel.cl's TraceInput. Returns the number of child requests pushed, or -1
 * when the cone schedule does not end within `cone_limit` traces per pixel. */
long ref_mega_trace_rows(const ushort *bases, uchar base_depth, const Block *blocks_in, size_t n_blocks,
                         Usage *usage, const void *in, float *rgba, ChildRequest *req_out, uint req_cap, int threads,
                         uint row_begin, uint row_end, long cone_limit) {
  TraceInput input;
  memcpy(&input, in, sizeof(input));
  input.BaseDepth = base_depth;
  size_t W = input.ScreenSize[0], H = input.ScreenSize[1];
  if (row_end > H) row_end = (uint)H;
  if (row_begin > row_end) row_begin = row_end;
  size_t bound = 2;
  if (input.FovConstant > 0 && input.FovMultiplier < 1 && input.FovMultiplier > -1) {
    bound = traces_bound(&input, (size_t)cone_limit);
    if (!bound) return -1;
  }
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
#endif
  Block *Blocks = (Block *)blocks_in;
  ushort *Bases = (ushort *)bases;
  Usage *Usages = usage ? usage : (Usage *)calloc(n_blocks / 8 + 1, sizeof(Usage));
  size_t n_px = (size_t)(row_end - row_begin) * W;
  ChildRequest *ChildRequests = (ChildRequest *)calloc(n_px * bound + 1, sizeof(ChildRequest));
  uint ChildRequestID = 0;
  ref_image_width = (uint)W;
  ref_gsize[0] = W;
  ref_gsize[1] = H;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
#endif
  for (size_t id = (size_t)row_begin * W; id < (size_t)row_end * W; id++) {
    ref_gid[0] = id % W;
    ref_gid[1] = id / W;
    trace(Bases, Blocks, Usages, &ChildRequestID, ChildRequests, rgba, input);
  }
  if (req_out) memcpy(req_out, ChildRequests, sizeof(ChildRequest) * (ChildRequestID < req_cap ? ChildRequestID : req_cap));
  free(ChildRequests);
  if (!usage) free(Usages);
  return (long)ChildRequestID;
}
