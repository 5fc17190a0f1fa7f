"""Benchmark: 1080p single-view wavefront trace over the depth-11 fBm terrain octree.

One step = one full frame (1920x1080 primary rays: ray generation, base/block
traversal with the cone LOD stop, usage stamping, child requests, shading and the
final colour) over a ~48M-node tree resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is kernel-timed Mrays/s with the tree and outputs on
the device (L2 flushed between steps); `e2e` is the same metric through the public
API with host buffers (input upload and result download inside the timed region);
`roofline` uses the algorithmic bytes of the reference's walk (16 B per node read of
getBlockAddress + 2 B per base chunk read + 25 B of per-pixel output).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "svo-tracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

WIDTH, HEIGHT = 1920, 1080  # the headline view; --width/--height trace a smaller view of the same scene
BASE_DEPTH, MAX_DEPTH, SEED = 4, 11, 5
CAM_ORIGIN, CAM_TARGET, FOV = (0.08, 0.12, 0.62), (0.75, 0.8, 0.88), 60.0
METRIC = "Mrays/s 1080p"  # reported for the 1920x1080 view
OUT_BYTES = 4 + 1 + 4 + 16  # hit index, hit depth, t, float4 RGBA


def workload(st):
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=SEED).BuildTree(BASE_DEPTH, MAX_DEPTH)
    cam = st.look_at(CAM_ORIGIN, CAM_TARGET, WIDTH, HEIGHT, FOV, Tick=7, MaxChildRequestId=1 << 16)
    return tree, cam


def config_dict(tree, extra=None):
    d = {"workload": "%dx%d single view, depth-11 fBm terrain octree (seeded, 6 octaves)" % (WIDTH, HEIGHT),
         "width": WIDTH, "height": HEIGHT, "base_depth": BASE_DEPTH, "max_depth": MAX_DEPTH,
         "nodes": int(len(tree.Blocks)), "tree_bytes": int(tree.Blocks.nbytes),
         "l2": "flushed between steps (256 MiB write)"}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clock samples (every 100 ms) with the host time they arrived at.
    Started before the warm-up so that the tool is already sampling when the timed
    loops run; `summary(windows)` keeps the samples inside the timed windows."""
    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, windows, margin_s=0.05):
        rows = [r for t, r in self.rows if any(a - margin_s <= t <= b + margin_s for a, b in windows)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "timed_s": round(sum(b - a for a, b in windows), 3),
                "windows": "headline frames, e2e calls, 64-view and colour-fitting sections"}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """dram bytes per launch of the trace kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "trace_kernel_terrain1080p_traffic.json")) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_launch"])
    except (OSError, KeyError, ValueError):
        return None


def roofline(alg_bytes, ms, what):
    """HBM roofline of one timed launch (or sequence): the algorithmic bytes over the
    CUDA-event time, against the measured copy bandwidth."""
    peak, kind = measured_peak()
    achieved = alg_bytes / (ms / 1000.0) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": kind, "algorithmic_bytes": int(alg_bytes), "ms": ms, "bytes": what}


def cpu_sample(tree, cam, kind, budget_s=12.0):
    """The CPU implementation over row bands of the same frame until ~budget_s."""
    import pyoracle as po

    threads = os.cpu_count() or 1
    rows_per_band = 40 if kind == "reference" else 270
    rays = 0
    t0 = time.perf_counter()
    band = 0
    while True:
        r0 = (band * rows_per_band) % HEIGHT
        r1 = min(HEIGHT, r0 + rows_per_band)
        if kind == "reference":
            po.ref_trace_rows(tree, cam, r0, r1, threads=threads)
        else:
            po.trace_rows(tree, cam, r0, r1, threads=threads)
        rays += (r1 - r0) * WIDTH
        band += 1
        el = time.perf_counter() - t0
        if el >= budget_s or band * rows_per_band >= 4 * HEIGHT:
            break
    return {"value": rays / el / 1e6, "unit": "Mrays/s", "cores": threads, "kind": kind,
            "sample": "%d rays in %d row bands of %d rows of the 1080p frame, %.1f s" % (rays, band, rows_per_band, el)}


def reference_scene(st):
    """The benchmarked tree read from the .oct file that __graft_entry__.build()
    writes, with numpy alone: the reference arm's process never loads libsvo (a
    missing file is written by a child process)."""
    import __graft_entry__

    path = __graft_entry__.REFERENCE_SCENE
    if not os.path.exists(path):
        subprocess.run([sys.executable, "-c", "import __graft_entry__ as g; g.write_reference_scene()"], cwd=ROOT,
                       check=True)
    tree = st.map_oct(path)
    cam = st.look_at(CAM_ORIGIN, CAM_TARGET, WIDTH, HEIGHT, FOV, Tick=7, MaxChildRequestId=1 << 16)
    return tree, cam


def run_reference(args, rank, world):
    """The reference's own wavefront.cl kernels, built for the host CPU, on the same frame."""
    if rank != 0:
        return
    import pyoracle as po
    import svo_tracer as st

    if not po.ref_available():
        print(json.dumps({"impl": "reference", "unavailable": "reference kernels (oracle/_ref) not built on this host"}))
        return
    tree, cam = reference_scene(st)
    threads = os.cpu_count() or 1
    # each step: 2 bands of 20 rows; the bands of all steps spread evenly over the
    # frame (its top rows are mostly sky, its bottom rows terrain)
    rows, bands = 40, 2
    n = args.warmup + args.steps
    times = []
    for i in range(n):
        t0 = time.perf_counter()
        for j in range(bands):
            r0 = min(HEIGHT - rows // bands, int((i * bands + j + 0.5) / (n * bands) * HEIGHT))
            po.ref_trace_rows(tree, cam, r0, r0 + rows // bands, threads=threads)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    total = sum(times)
    value = rows * WIDTH * len(times) / total / 1e6
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+u64", "data": "synthetic",
            "config": config_dict(tree, {"sample_rows_per_step": rows}), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "reference",
                             "sample": "%d rows (%d rays) of the 1080p frame per step, in %d bands spread over the "
                                       "frame across the steps" % (rows, rows * WIDTH, bands)},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def multiview(tr, torch, dev, stream, flush, args, windows=None):
    """64 mixed-resolution views over the same tree: one autotuned, CUDA-graph-replayed
    persistent launch against 64 sequential plain launches, same device outputs."""
    import svo_tracer as st

    views = st.mixed_views(seed=4, Tick=7, MaxChildRequestId=1 << 16)
    sizes = [v.ScreenSize[0] * v.ScreenSize[1] for v in views]
    rays = sum(sizes)

    def alloc():
        o = [(torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
              torch.empty(n, dtype=torch.float32, device=dev), torch.empty(4 * n, dtype=torch.float32, device=dev))
             for n in sizes]
        return o, [tuple(x.data_ptr() for x in t) for t in o]

    batched_t, batched_p = alloc()
    plain_t, plain_p = alloc()
    cfg0 = {n: getattr(tr.get_config(), n) for n in ("block_size", "ray_chunk", "cadence", "ctas_per_sm")}
    # the reference walk's node and base reads of the 64 views (a counting launch, untimed)
    tr.set_config(collect_stats=1)
    tr.trace_device(views, batched_p)
    vstats = tr.stats()
    tr.set_config(collect_stats=0)
    alg = 16 * vstats["block_node_reads"] + 2 * vstats["base_steps"] + OUT_BYTES * rays
    with torch.cuda.stream(stream):
        # plain: one launch per view with the default configuration
        for _ in range(2):
            for v, p in zip(views, plain_p):
                tr.trace_device([v], [p])
        plain_ms = []
        t_win = time.perf_counter()
        for _ in range(max(3, args.steps // 4)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for v, p in zip(views, plain_p):
                tr.trace_device([v], [p])
            e1.record(stream)
            plain_ms.append((e0, e1))
        torch.cuda.synchronize(dev)
        if windows is not None:
            windows.append((t_win, time.perf_counter()))
        plain = sorted(a.elapsed_time(b) for a, b in plain_ms)[len(plain_ms) // 2]
        tuned, tune_ms = tr.autotune(views, batched_p, repeats=2)
        for _ in range(2):
            tr.trace_device(views, batched_p, graph=True)
        batch_ms = []
        t_win = time.perf_counter()
        for _ in range(max(3, args.steps // 4)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tr.trace_device(views, batched_p, graph=True)
            e1.record(stream)
            batch_ms.append((e0, e1))
        torch.cuda.synchronize(dev)
        if windows is not None:
            windows.append((t_win, time.perf_counter()))
        batched = sorted(a.elapsed_time(b) for a, b in batch_ms)[len(batch_ms) // 2]
    same = all(torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) and torch.equal(a[2], b[2])
               and torch.equal(a[3], b[3]) for a, b in zip(batched_t, plain_t))
    tr.set_config(**cfg0)
    return {"views": len(views), "rays": rays, "batched_ms": batched, "plain_ms": plain,
            "batched_mrays_s": rays / batched / 1e3, "plain_mrays_s": rays / plain / 1e3,
            "speedup": plain / batched, "identical_outputs": bool(same), "autotuned": tuned,
            "roofline": roofline(alg, batched, "16 B per node read of the reference walk + 2 B per base chunk read "
                                               "+ 25 B of output per pixel, summed over the 64 views"),
            "roofline_plain": roofline(alg, plain, "the same bytes over the 64 plain launches"),
            "batched": "one persistent launch over all views, replayed from a CUDA graph",
            "plain": "64 sequential single-view launches, same stream, default configuration"}


def sphere_workload(torch, dev, flush, args, windows=None):
    """The CPU-runnable case: one 640x480 view (FoV 60 degrees, camera at world
    distance 1.5 on a seeded direction, i.e. 0.75 in the unit cube that the [-1,1]
    world maps onto) of the depth-8 SDF sphere, traced by the plain path, with the
    reference's CPU build timed on the same whole frame."""
    import pyoracle as po
    import svo_tracer as st

    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=SEED).BuildTree(BASE_DEPTH, 8)
    cam = st.orbit_views(seed=SEED, n=1, width=640, height=480, distance=0.75, Tick=7, MaxChildRequestId=1 << 16)[0]
    n = 640 * 480
    tr = st.Tracer(dev)
    stream = torch.cuda.Stream(device=dev)
    tr.set_stream(stream.cuda_stream)
    tr.upload(tree)
    tr.init_usage()
    tr.set_config(collect_stats=1)
    tr.trace(cam)
    stats = tr.stats()
    tr.set_config(collect_stats=0)
    o = [torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
         torch.empty(n, dtype=torch.float32, device=dev), torch.empty(4 * n, dtype=torch.float32, device=dev)]
    outs = [tuple(x.data_ptr() for x in o)]
    with torch.cuda.stream(stream):
        for _ in range(3):
            tr.trace_device([cam], outs)
        ev = []
        t_win = time.perf_counter()
        for _ in range(max(5, args.steps)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tr.trace_device([cam], outs)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize(dev)
        if windows is not None:
            windows.append((t_win, time.perf_counter()))
    ms = sum(a.elapsed_time(b) for a, b in ev) / len(ev)
    tr.close()
    alg = 16 * stats["block_node_reads"] + 2 * stats["base_steps"] + OUT_BYTES * n
    out = {"workload": "640x480 view of the depth-8 SDF sphere (%d nodes)" % len(tree.Blocks), "ms": ms,
           "mrays_s": n / ms / 1e3, "algorithmic_gb_s": alg / ms / 1e6, "hits": int(stats["hits"])}
    if not args.no_cpu_baseline and po.ref_available():
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        po.ref_trace_view(tree, cam, threads=threads)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / el / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "reference",
                               "sample": "the whole 640x480 frame, %.2f s" % el}
    return out


def mega_workload(tr, torch, dev, stream, flush, args, tree, cam, windows=None):
    """The megakernel (kernel.cl's `trace`: primary cone, spawnRays's fan of
    secondary cones, draw) on the same 1080p terrain frame, with the reference's
    default cone parameters (FovMultiplier 0.2, FovConstant 0.2, WeightingMultiplier
    -0.05, WeightingConstant 0.5). Rays = primary + secondary cones."""
    import svo_tracer as st

    n = WIDTH * HEIGHT
    o = [torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
         torch.empty(n, dtype=torch.float32, device=dev), torch.empty(4 * n, dtype=torch.float32, device=dev)]
    ptrs = [x.data_ptr() for x in o]
    steps = max(3, args.steps // 4)
    with torch.cuda.stream(stream):
        # the primary and secondary cones' node and base reads (a counting launch, untimed)
        tr.set_config(collect_stats=1)
        tr.mega_trace_device(cam, *ptrs)
        mstats = tr.stats()
        tr.set_config(collect_stats=0)
        for _ in range(2):
            flush.zero_()
            tr.mega_trace_device(cam, *ptrs)
        stats = tr.mega_stats()
        ev = []
        torch.cuda.synchronize(dev)
        t_win = time.perf_counter()
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tr.mega_trace_device(cam, *ptrs)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize(dev)
        if windows is not None:
            windows.append((t_win, time.perf_counter()))
    ms = sorted(a.elapsed_time(b) for a, b in ev)
    frame_ms = sum(ms) / len(ms)
    rays = stats["pixels"] + stats["cones"]
    # end to end through the public API with pinned host outputs
    h = st.TraceResult(torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
                       torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy(),
                       torch.empty(n, dtype=torch.float32, pin_memory=True).numpy(),
                       torch.empty(n * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(n, 4))
    tr.mega_trace(cam, out=h)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(steps):
        tr.mega_trace(cam, out=h)
    e2e_s = (time.perf_counter() - t0) / steps
    if windows is not None:
        windows.append((t0, time.perf_counter()))
    return {"frame_ms": frame_ms, "frame_ms_min": ms[0], "frames_per_s": 1000.0 / frame_ms,
            "mrays_s": rays / frame_ms / 1e3, "primary_rays": stats["pixels"], "cones": stats["cones"],
            "cones_per_pixel": stats["cones"] / max(1, stats["pixels"]), "surfaces": stats["surfaces"],
            "cone_slots": stats["cone_slots"], "steps": steps,
            "roofline": roofline(16 * mstats["block_node_reads"] + 2 * mstats["base_steps"] + n * OUT_BYTES, frame_ms,
                                 "16 B per node read + 2 B per base chunk read of every primary and secondary cone "
                                 "+ 25 B of output per pixel"),
            "e2e": {"frame_ms": 1000.0 * e2e_s, "mrays_s": rays / e2e_s / 1e6,
                    "d2h_bytes_per_step": n * OUT_BYTES},
            "workload": "kernel.cl trace over the 1080p terrain frame, reference default cone parameters"}


def gi_workload(tr, torch, dev, stream, flush, args, cam, outs, windows=None):
    """The 1080p frame with the wavefront's secondary-cone stage as the reference
    wires it (svo_trace_config.gi_stage): the trace, then per hit the cone fan of
    evaluateMaterial, each cone lit by evaluateBackground (default cone
    parameters, AmbientLightLevel 100)."""
    steps = max(5, args.steps // 2)
    tr.set_config(gi_stage=1)
    with torch.cuda.stream(stream):
        for _ in range(2):
            tr.trace_device([cam], outs)
        ev = []
        t_win = time.perf_counter()
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tr.trace_device([cam], outs)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize(dev)
        if windows is not None:
            windows.append((t_win, time.perf_counter()))
    tr.set_config(gi_stage=-1)
    ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
    return {"frame_ms": ms, "mrays_s": WIDTH * HEIGHT / ms / 1e3, "steps": steps,
            "workload": "1080p terrain frame with the material stage (evaluateMaterial + saveAccumulator + "
                        "evaluateBackground of every hit's cone fan)"}


def mega_cpu_sample(tree, cam, budget_s=8.0):
    """The reference's megakernel (kernel.cl built for the host CPU) over row bands
    of the same frame until ~budget_s; rays = primary + secondary cones, the cone
    count taken from the oracle over the same rows."""
    import pyoracle as po

    if not po.ref_mega_available():
        return None
    threads = os.cpu_count() or 1
    rows, band, px, t_ref = 4, 0, 0, 0.0
    cones = 0
    while t_ref < budget_s and band * rows < HEIGHT:
        r0 = (HEIGHT // 2 + band * rows) % HEIGHT
        r1 = min(HEIGHT, r0 + rows)
        t0 = time.perf_counter()
        po.ref_mega_trace_view(tree, cam, threads=threads, rows=(r0, r1), req_cap=1 << 16)
        t_ref += time.perf_counter() - t0
        cones += int(po.mega_trace_view(tree, cam, threads=threads, rows=(r0, r1), req_cap=1)["cones"].sum())
        px += (r1 - r0) * WIDTH
        band += 1
    return {"value": (px + cones) / t_ref / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "reference",
            "frames_per_s": px / (WIDTH * HEIGHT) / t_ref,
            "sample": "%d pixels (%d cones) in %d bands of %d rows through the frame's middle, %.1f s" %
                      (px, cones, band, rows, t_ref)}


def _stream_run(st, scene, tree, cams, dev, device_generate):
    """One pass of the stream: per frame trace (usage stamps, child requests),
    graft payloads (on the device, or generated on the host and uploaded), GC of
    groups unused for more than 30 frames, grafts into the freed groups."""
    budget = 1 << 22
    import torch
    tr = st.Tracer(dev)
    stream = torch.cuda.Stream(device=dev)  # GPU time of each phase by events on the context's stream
    tr.set_stream(stream.cuda_stream)
    tr.set_config(request_order=st.REQUESTS_PIXEL)  # the kept requests do not depend on timing
    tr.upload(tree, block_budget=budget * 8)
    tr.init_usage_tree(1)
    n = WIDTH * HEIGHT
    o = [torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
         torch.empty(n, dtype=torch.float32, device=dev), torch.empty(4 * n, dtype=torch.float32, device=dev)]
    outs = [tuple(x.data_ptr() for x in o)]
    totals = {"requests": 0, "grafted_groups": 0, "graft_records": 0, "pruned_groups": 0, "freed_groups": 0}
    phase = {"trace": 0.0, "generate": 0.0, "gc": 0.0, "graft": 0.0}
    if device_generate:  # the pyramids go to the device once, before the timed loop
        tr.trace_device([cams[0]], outs)
        tr.graft_generate(1, scene)
        tr.upload(tree, block_budget=budget * 8)
        tr.init_usage_tree(1)
    ev = []
    t_loop = time.perf_counter()
    for f, cam in enumerate(cams):
        tick = f + 1
        marks = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev.append(marks)
        a = time.perf_counter()
        marks[0].record(stream)
        tr.trace_device([cam], outs)
        marks[1].record(stream)
        if device_generate:
            rec = pay = None
        else:
            req, n_req = tr.read_child_requests(cap=1 << 16)
        b = time.perf_counter()
        if not device_generate:
            rec, pay = scene.graft_payload(req)
        c = time.perf_counter()
        marks[2].record(stream)  # after the host's payload generation, if any
        rep = tr.gc(tick, 30)
        marks[3].record(stream)
        d = time.perf_counter()
        grep = tr.graft_generate(tick, scene) if device_generate else tr.graft(tick, rec, pay)
        marks[4].record(stream)
        e = time.perf_counter()
        if device_generate:
            n_req = tr.stats()["child_requests"]  # the trace's request count (kept until the next trace)
        phase["trace"] += b - a
        phase["generate"] += c - b
        phase["gc"] += d - c
        phase["graft"] += e - d
        if device_generate:
            t_loop -= time.perf_counter() - e  # the count read-back is bookkeeping, not part of the frame
        totals["requests"] += n_req
        totals["grafted_groups"] += grep["claimed"]
        totals["graft_records"] += grep["applied"]
        totals["pruned_groups"] += rep["pruned"]
        totals["freed_groups"] += rep["freed"]
    loop_s = time.perf_counter() - t_loop
    torch.cuda.synchronize(dev)
    gpu = {"trace": 0.0, "gc": 0.0, "graft": 0.0}
    for m in ev:
        gpu["trace"] += m[0].elapsed_time(m[1])
        gpu["gc"] += m[2].elapsed_time(m[3])
        gpu["graft"] += m[3].elapsed_time(m[4])
    upd_ms = gpu["gc"] + gpu["graft"]
    upd_bytes = 8 * budget * len(cams) + 16 * 8 * totals["grafted_groups"]
    usage = tr.read_usage(budget)
    resident = int(((usage["tick"] >= 1) & (usage["tick"] <= 65533)).sum())
    digest = hashlib.sha256()
    digest.update(tr.read_blocks(0, budget * 8).tobytes())
    digest.update(usage.tobytes())
    tr.close()
    frames = len(cams)
    return {"frames_per_s": frames / loop_s, "ms_per_frame": 1000 * loop_s / frames, "state_sha256": digest.hexdigest(),
            "mrays_s_with_updates": frames * n / loop_s / 1e6,
            # host wall time spent in each phase's calls: the trace returns before its
            # kernel ends and the GC's count read-back waits for it, so only the GPU
            # times below split the frame's GPU work
            "host_ms_per_frame_by_phase": {k: 1000 * v / frames for k, v in phase.items()},
            "gpu_ms_per_frame_by_phase": {k: v / frames for k, v in gpu.items()},
            "roofline_updates": roofline(upd_bytes / frames, upd_ms / frames,
                                         "per frame: 8 B per budget group of the GC's usage scan + 16 B per grafted "
                                         "node, over the GC and graft GPU time"),
            "totals": totals, "resident_groups_end": resident}


def stream_workload(torch, dev, args):
    """The pruning/grafting/GC stream: 120 frames along a Catmull-Rom camera path at
    1080p over the depth-12 terrain scene behind a budget of 2^22 block groups, with
    the graft payloads generated on the device (svo_graft_generate); the same
    frames with the payloads generated on the host cores are reported beside it.
    Wall time per frame covers the whole frame."""
    import svo_tracer as st

    frames = args.stream_frames
    t0 = time.perf_counter()
    scene = st.Scene(st.SCENE_TERRAIN, seed=SEED, base_depth=BASE_DEPTH, depth=12)
    tree = scene.build_tree(10)
    setup_s = time.perf_counter() - t0
    cams = st.camera_path(seed=3, frames=frames, width=WIDTH, height=HEIGHT, MaxChildRequestId=1 << 16)
    on_device = _stream_run(st, scene, tree, cams, dev, True)
    on_host = _stream_run(st, scene, tree, cams, dev, False)
    out = {"frames": frames, "width": WIDTH, "height": HEIGHT, "scene_depth": 12, "initial_depth": 10,
           "budget_groups": 1 << 22, "stale_frames": 30, "request_cap": 1 << 16, "setup_s": setup_s,
           "graft_generation": "device (svo_graft_generate)"}
    out.update(on_device)
    out["host_generation"] = {k: on_host[k] for k in ("ms_per_frame", "host_ms_per_frame_by_phase",
                                                       "gpu_ms_per_frame_by_phase", "totals", "state_sha256")}
    # A 1080p frame raises ~2M child requests against the 65,536-entry queue; the
    # pixel-order rule keeps those of the lowest pixels, so both generation paths
    # (and every run) reach the same tree: same totals and the same final blocks
    # and usage arrays.
    out["request_order"] = "pixel (the requests of the lowest pixel indices up to the cap)"
    out["generation_paths_agree"] = bool(on_device["state_sha256"] == on_host["state_sha256"]
                                         and on_device["totals"] == on_host["totals"])
    out["timing"] = "host wall clock per frame, synchronous pipeline"
    return out


def diff_workload(torch, dev, flush, args, windows=None):
    """Differentiable colour fitting: the depth-9 SDF sphere (512^3 leaf grid), 16
    views of 512x512 around it at the sphere case's camera distance (world 1.5, 0.75
    in the unit cube), FP32 per-node RGBA initialised uniform in [0, 1],
    targets rendered from the seeded sinusoid ground-truth field (opacity 0.9).
    One step = forward colour + backward (loss and dL/dRGBA per node, traversal
    recomputed once, the forward's colour reused), device-resident; L2 flushed
    between steps. `e2e` is one fitting
    step through the host API: parameters uploaded, forward colour read back,
    backward with the loss and the gradients read back."""
    import svo_tracer as st

    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(4, 9)
    views = st.orbit_views(seed=7, n=args.diff_views, width=args.diff_size, height=args.diff_size, distance=0.75)
    rays = sum(v.ScreenSize[0] * v.ScreenSize[1] for v in views)
    nodes = len(tree.Blocks)
    tr = st.Tracer(dev)
    stream = torch.cuda.Stream(device=dev)  # events, flush and kernels all on this stream
    tr.set_stream(stream.cuda_stream)
    tr.upload(tree)
    tr.set_config(max_hits=16)
    with torch.cuda.stream(stream):
        return _diff_timed(tr, torch, dev, stream, flush, args, tree, views, rays, nodes, windows)


def _diff_timed(tr, torch, dev, stream, flush, args, tree, views, rays, nodes, windows=None):
    import svo_tracer as st

    gt = torch.from_numpy(st.sinusoid_field(tree, seed=9)).to(dev)
    params = torch.from_numpy(np.random.default_rng(3).uniform(0.0, 1.0, (nodes, 4)).astype(np.float32)).to(dev)
    target = torch.empty(rays * 3, dtype=torch.float32, device=dev)
    rgb = torch.empty(rays * 3, dtype=torch.float32, device=dev)
    tr.diff_set_params_device(gt.data_ptr(), nodes)
    tr.diff_forward_device(views, target.data_ptr())
    tr.diff_set_params_device(params.data_ptr(), nodes)
    torch.cuda.synchronize()

    def timed(fn, steps):
        ms = []
        t_win = time.perf_counter()
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        if windows is not None:
            windows.append((t_win, time.perf_counter()))
        return float(np.median(ms))

    steps = max(5, args.steps // 2)
    # the forward walk's node and base reads and its composited hits (a counting launch, untimed)
    tr.set_config(collect_stats=1)
    tr.diff_forward_device(views, rgb.data_ptr())
    dstats = tr.stats()
    tr.set_config(collect_stats=0)
    walk = 16 * dstats["block_node_reads"] + 2 * dstats["base_steps"]
    for _ in range(3):
        tr.diff_forward_device(views, rgb.data_ptr())
        tr.diff_backward_device(views, target.data_ptr())
    fwd_ms = timed(lambda: tr.diff_forward_device(views, rgb.data_ptr()), steps)
    bwd_ms = timed(lambda: tr.diff_backward_device(views, target.data_ptr(), use_saved=True), steps)
    bwd_recompute_ms = timed(lambda: tr.diff_backward_device(views, target.data_ptr()), steps)
    step_ms = timed(lambda: (tr.diff_forward_device(views, rgb.data_ptr()),
                             tr.diff_backward_device(views, target.data_ptr(), use_saved=True)), steps)
    # host buffers in pinned memory, as a caller streaming through this API would hold them
    host_params = torch.empty((nodes, 4), dtype=torch.float32, pin_memory=True).numpy()
    host_params[:] = params.cpu().numpy()
    host_target = torch.empty(rays * 3, dtype=torch.float32, pin_memory=True).numpy()
    host_target[:] = target.cpu().numpy()
    host_rgb = torch.empty(rays * 3, dtype=torch.float32, pin_memory=True).numpy()
    host_grads = torch.empty((nodes, 4), dtype=torch.float32, pin_memory=True).numpy()
    loss0 = tr.diff_backward(views, host_target)
    t0 = time.perf_counter()
    for _ in range(steps):
        tr.diff_set_params(host_params)
        tr.diff_forward(views, out=host_rgb)
        tr.diff_backward(views, host_target, use_saved=True)
        tr.diff_grads(nodes, out=host_grads)
    e2e_s = (time.perf_counter() - t0) / steps
    tr.close()
    return {"workload": "depth-9 SDF sphere, %d views %dx%d, FP32 per-node RGBA, max 16 hits per ray"
                        % (len(views), views[0].ScreenSize[0], views[0].ScreenSize[1]),
            "nodes": nodes, "rays": rays, "fwd_ms": fwd_ms, "bwd_ms": bwd_ms, "fwd_bwd_ms": step_ms,
            "bwd_recompute_colour_ms": bwd_recompute_ms,
            "fwd_bwd_mrays_s": rays / step_ms / 1e3, "fwd_mrays_s": rays / fwd_ms / 1e3,
            "bwd_mrays_s": rays / bwd_ms / 1e3, "initial_loss": loss0,
            "hits": int(dstats["hits"]),
            "roofline": roofline(2 * (walk + 12 * rays) + 16 * dstats["hits"], step_ms,
                                 "2 x (16 B per node read + 2 B per base chunk read of the walk + 12 B of colour or "
                                 "target per ray) + 16 B of gradient per composited hit"),
            "e2e": {"value": rays / e2e_s / 1e6, "unit": "Mrays/s (fwd+bwd)",
                    "h2d_bytes_per_step": nodes * 16 + rays * 12, "d2h_bytes_per_step": rays * 12 + nodes * 16 + 8},
            "l2": "flushed between steps (256 MiB write)"}


def run_ours(args, rank, world):
    import torch

    import replicas
    import svo_tracer as st

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    tree, cam = workload(st)
    tr = st.Tracer(dev)
    stream = torch.cuda.Stream(device=dev)
    tr.set_stream(stream.cuda_stream)
    tr.upload(tree)
    tr.init_usage()
    if args.schedule:
        tr.set_config(schedule={"lane": st.SCHEDULE_LANE, "warp": st.SCHEDULE_WARP}[args.schedule])
    n = WIDTH * HEIGHT

    # algorithmic bytes of one frame (counting launch, untimed)
    tr.set_config(collect_stats=1)
    tr.trace(cam)
    stats = tr.stats()
    tr.set_config(collect_stats=0)
    alg_bytes = 16 * stats["block_node_reads"] + 2 * stats["base_steps"] + OUT_BYTES * n

    # device-resident outputs
    o_idx = torch.empty(n, dtype=torch.int32, device=dev)
    o_dep = torch.empty(n, dtype=torch.uint8, device=dev)
    o_t = torch.empty(n, dtype=torch.float32, device=dev)
    o_rgba = torch.empty(n * 4, dtype=torch.float32, device=dev)
    outs = [(o_idx.data_ptr(), o_dep.data_ptr(), o_t.data_ptr(), o_rgba.data_ptr())]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    clk = ClockSampler(dev).__enter__()  # sampling from before the warm-up
    windows = []  # host-time spans of the timed GPU work
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            tr.trace_device([cam], outs)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        t_start = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            tr.trace_device([cam], outs)
            ends[i].record(stream)
        torch.cuda.synchronize(dev)
        windows.append((t_start, time.perf_counter()))
        t_wall = windows[-1][1] - t_start
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(sum(step_ms))

    # end to end through the public API with host buffers (pinned outputs)
    h_idx = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    h_dep = torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy()
    h_t = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
    h_rgba = torch.empty(n * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(n, 4)
    res = st.TraceResult(h_idx, h_dep, h_t, h_rgba)
    for _ in range(max(1, args.warmup)):
        tr.trace(cam, out=res)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tr.trace(cam, out=res)  # uploads view + trig tables, traces, downloads all outputs, synchronises
    e2e_s = time.perf_counter() - t0
    windows.append((t0, t0 + e2e_s))

    total_ms, e2e_s = replicas.max_over_ranks([total_ms, e2e_s], dist, dev)
    if rank != 0:
        clk.__exit__(None, None, None)
        tr.close()
        if dist:
            dist.destroy_process_group()
        return

    ms_per_step = total_ms / args.steps
    value = replicas.replica_throughput(world, n, ms_per_step)
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (ms_per_step / 1000.0) / 1e9
    traffic = ncu_traffic()
    h2d = 120 + 8 * (WIDTH + HEIGHT)  # view record + sin/cos tables
    d2h = n * OUT_BYTES
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u64", "data": "synthetic",
        "config": config_dict(tree, {"parallelism": "replicas" if world > 1 else "single GPU",
                                     "step_ms_min": min(step_ms), "step_ms_max": max(step_ms),
                                     "wall_s_timed_loop": t_wall}),
        "e2e": {"value": replicas.replica_throughput(world, n, 1000.0 * e2e_s / args.steps), "unit": "Mrays/s",
                "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": int(alg_bytes),
                     "bytes_per_ray": alg_bytes / n},
        "trace_stats": {k: int(v) for k, v in stats.items()},
    }
    if not args.no_multiview:
        line["multiview"] = multiview(tr, torch, dev, stream, flush, args, windows)
    if not args.no_diff:
        line["diff"] = diff_workload(torch, dev, flush, args, windows)
    if not args.no_mega:
        line["megakernel"] = mega_workload(tr, torch, dev, stream, flush, args, tree, cam, windows)
    if not args.no_sphere:
        line["sphere_640x480"] = sphere_workload(torch, dev, flush, args, windows)
    if not args.no_gi:
        line["gi_stage"] = gi_workload(tr, torch, dev, stream, flush, args, cam, outs, windows)
    clk.__exit__(None, None, None)
    line["clocks"] = clk.summary(windows)
    if args.stream_frames > 0:
        line["stream"] = stream_workload(torch, dev, args)
    if not args.no_cpu_baseline:
        import pyoracle as po

        kind = "reference" if po.ref_available() else "port"
        line["cpu_baseline"] = cpu_sample(tree, cam, kind)
        if "megakernel" in line:
            line["megakernel"]["cpu_baseline"] = mega_cpu_sample(tree, cam)
    print(json.dumps(line))
    tr.close()
    if dist:
        dist.destroy_process_group()


def run_ncu_case(args):
    """One launch of a profiled case, for an ncu capture, then exit: `batch64` is
    the 64 mixed views over the depth-11 terrain in one batched launch (the
    multiview section's kernel, warp batches of 128 threads)."""
    import torch

    import svo_tracer as st

    tree, _ = reference_scene(st)
    views = st.mixed_views(seed=4, Tick=7, MaxChildRequestId=1 << 16)
    tr = st.Tracer(0)
    tr.upload(tree)
    tr.init_usage()
    keep, outs = [], []
    for v in views:
        n = v.ScreenSize[0] * v.ScreenSize[1]
        o = (torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.uint8, device="cuda"),
             torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(4 * n, dtype=torch.float32, device="cuda"))
        keep.append(o)
        outs.append(tuple(x.data_ptr() for x in o))
    tr.set_config(block_size=128)
    tr.trace_device(views, outs)
    torch.cuda.synchronize()
    tr.close()
    print("%s: one batched launch of %d views" % (args.ncu_case, len(views)))


def main():
    global WIDTH, HEIGHT
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-multiview", action="store_true")
    ap.add_argument("--no-diff", action="store_true")
    ap.add_argument("--no-mega", action="store_true")
    ap.add_argument("--no-sphere", action="store_true")
    ap.add_argument("--no-gi", action="store_true")
    ap.add_argument("--ncu-case", choices=["batch64"], default=None,
                    help="run one launch of a profiled case and exit (for an ncu capture)")
    ap.add_argument("--schedule", choices=["lane", "warp"], default=None)
    ap.add_argument("--diff-views", type=int, default=16)
    ap.add_argument("--diff-size", type=int, default=512)
    ap.add_argument("--stream-frames", type=int, default=120)
    ap.add_argument("--width", type=int, default=WIDTH)
    ap.add_argument("--height", type=int, default=HEIGHT)
    args = ap.parse_args()
    WIDTH, HEIGHT = args.width, args.height
    args.warmup = max(3, args.warmup)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.impl == "reference" else 1)))
    if args.ncu_case:
        import __graft_entry__

        if not os.path.exists(os.path.join(ROOT, "svo-tracer_gb300", "lib", "libsvo.so")):
            __graft_entry__.build()
        run_ncu_case(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        import __graft_entry__

        if not os.path.exists(os.path.join(ROOT, "svo-tracer_gb300", "lib", "libsvo.so")):
            __graft_entry__.build()
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
