"""ctypes bindings of the oracle libraries (TEST INFRASTRUCTURE ONLY).

``trace_view`` runs the C restatement (libsvo_oracle.so); ``ref_trace_view`` runs the
reference's own wavefront.cl kernels compiled for the CPU (oracle/_ref/libsvo_ref.so).
``mega_trace_view`` and ``ref_mega_trace_view`` are the same pair for the megakernel
(kernel.cl, oracle/_ref/libsvo_ref_mega.so). All take the same inputs as the CUDA
path and return per-pixel results.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402
import build_ref  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(HERE), "svo-tracer_gb300"))
from svo_tracer import (BLOCK_DTYPE, CHILD_REQUEST_DTYPE, GRAFTING_DTYPE, PRUNING_DTYPE, USAGE_DTYPE,  # noqa: E402
                        TraceInput)

_vp = C.c_void_p
_oracle = None
_ref = None
_ref_mega = None


class _ViewOut(C.Structure):
    _fields_ = [(n, _vp) for n in ("hit_index", "hit_depth", "t", "rgba", "acc", "v_block", "v_base", "steps",
                                   "requested", "pixel_request")]


def _p(a):
    return None if a is None else a.ctypes.data_as(_vp)


def oracle_lib() -> C.CDLL:
    global _oracle
    if _oracle is None:
        lib = C.CDLL(build_oracle.build_oracle())
        lib.oracle_trace_view.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t, _vp, C.c_size_t, C.c_char_p, C.c_int32,
                                          C.POINTER(_ViewOut), _vp, C.c_uint32, C.POINTER(C.c_uint32), C.c_int32]
        lib.oracle_trace_view.restype = C.c_int64
        lib.oracle_trace_rows.argtypes = lib.oracle_trace_view.argtypes + [C.c_uint32, C.c_uint32]
        lib.oracle_trace_rows.restype = C.c_int64
        lib.oracle_trace_rows_gi.argtypes = lib.oracle_trace_rows.argtypes + [C.c_int32]
        lib.oracle_trace_rows_gi.restype = C.c_int64
        lib.oracle_mega_trace_rows.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t, _vp, C.c_size_t, C.c_char_p,
                                               C.c_int32, C.c_int32, C.POINTER(_ViewOut), _vp, _vp, C.c_uint32,
                                               C.POINTER(C.c_uint32), C.c_int32, C.c_uint32, C.c_uint32]
        lib.oracle_mega_trace_rows.restype = C.c_int64
        lib.oracle_float_to_ulong.argtypes = [C.c_float]
        lib.oracle_float_to_ulong.restype = C.c_uint64
        lib.oracle_ulong_to_float.argtypes = [C.c_uint64]
        lib.oracle_ulong_to_float.restype = C.c_float
        lib.oracle_round_ulong.argtypes = [C.c_uint64, C.c_uint8, C.c_int]
        lib.oracle_round_ulong.restype = C.c_uint64
        lib.oracle_pow_sum.argtypes = [C.c_uint8]
        lib.oracle_pow_sum.restype = C.c_uint32
        lib.oracle_compare_positions.argtypes = [C.c_uint8, _vp, _vp, _vp]
        lib.oracle_compare_positions.restype = C.c_uint8
        lib.oracle_traverse_chunk.argtypes = [C.c_uint8, _vp, _vp, _vp, _vp]
        lib.oracle_trace_into_volume.argtypes = [_vp, _vp, _vp, C.c_float, _vp, _vp]
        lib.oracle_trace_into_volume.restype = C.c_int
        lib.oracle_init_usage.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t]
        lib.oracle_hit_lists.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t, C.c_char_p, C.c_int32, C.c_int32, _vp, _vp,
                                         _vp, _vp, C.c_int32]
        lib.oracle_diff_eval.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, C.c_int32, _vp, _vp, _vp, _vp, C.c_int32]
        lib.oracle_diff_eval.restype = C.c_double
        lib.oracle_diff_fd.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, C.c_int32, _vp, _vp, _vp, C.c_int32, C.c_double,
                                       _vp, C.c_int32]
        lib.oracle_init_usage_tree.argtypes = [_vp, C.c_int, _vp, C.c_size_t, _vp, C.c_uint16]
        lib.oracle_gc.argtypes = [_vp, C.c_int, _vp, C.c_size_t, _vp, C.c_uint16, C.c_uint32, _vp, _vp, _vp, _vp]
        lib.oracle_graft.argtypes = [C.c_int, _vp, C.c_size_t, _vp, C.c_uint16, _vp, C.c_uint32, _vp, C.c_size_t, _vp,
                                     C.c_size_t, _vp, C.c_uint64, _vp, _vp]
        lib.oracle_graft.restype = C.c_uint64
        lib.oracle_prune.argtypes = [_vp, C.c_size_t, C.c_int, _vp, C.c_size_t, _vp, C.c_uint16, _vp, C.c_uint32, _vp,
                                     C.c_size_t, _vp, C.c_size_t, _vp, C.c_uint32, C.POINTER(C.c_uint32), _vp]
        lib.oracle_prune.restype = C.c_uint64
        _oracle = lib
    return _oracle


def ref_available() -> bool:
    try:
        return build_ref.compile_ref() is not None
    except Exception:
        return False


def ref_lib() -> C.CDLL:
    global _ref
    if _ref is None:
        path = os.environ.get("SVO_REF_LIB") or build_ref.compile_ref()
        if path is None:
            raise RuntimeError("reference kernels unavailable (no wavefront.cl source)")
        lib = C.CDLL(path)
        lib.ref_trace_view.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t, _vp, C.c_size_t, C.c_char_p, _vp, _vp, _vp,
                                       _vp, _vp, _vp, C.c_uint32, C.POINTER(C.c_uint32), C.c_int, C.c_long]
        lib.ref_trace_view.restype = C.c_long
        lib.ref_trace_rows.argtypes = lib.ref_trace_view.argtypes + [C.c_uint, C.c_uint]
        lib.ref_trace_rows.restype = C.c_long
        lib.ref_trace_rows_gi.argtypes = lib.ref_trace_rows.argtypes + [C.c_int]
        lib.ref_trace_rows_gi.restype = C.c_long
        lib.ref_prune.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t, _vp, C.c_size_t, _vp, C.c_uint, _vp, C.c_size_t,
                                  _vp, C.c_size_t, C.c_uint16]
        lib.ref_prune.restype = C.c_long
        _ref = lib
    return _ref


def mega_trace_view(tree, inp: TraceInput, usage=None, max_steps: int = 1 << 16, threads: int = 0, rows=None,
                    req_cap: int = 1 << 22, cone_limit: int = 1 << 16):
    """The oracle's megakernel (kernel.cl's `trace`) on one view or rows [rows[0],
    rows[1]) of it (per-pixel outputs then cover the band). usage is stamped in
    place. Returns rgba, the primary's hit_index/hit_depth/t, per-pixel traversal
    steps and secondary cone counts, and the child requests."""
    lib = oracle_lib()
    w, h = inp.ScreenSize
    r0, r1 = (0, h) if rows is None else rows
    n = w * (r1 - r0)
    r = {"hit_index": np.empty(n, np.uint32), "hit_depth": np.empty(n, np.uint8), "t": np.empty(n, np.float32),
         "rgba": np.zeros((n, 4), np.float32), "steps": np.empty(n, np.uint32), "cones": np.zeros(n, np.uint32)}
    vo = _ViewOut(_p(r["hit_index"]), _p(r["hit_depth"]), _p(r["t"]), _p(r["rgba"]), None, None, None, _p(r["steps"]))
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    req = np.zeros(req_cap, CHILD_REQUEST_DTYPE)
    nreq = C.c_uint32(0)
    ng = 0 if usage is None else len(usage)
    rc = lib.oracle_mega_trace_rows(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), _p(usage), ng, inp.to_bytes(),
                                    max_steps, cone_limit, C.byref(vo), _p(r["cones"]), _p(req), req_cap,
                                    C.byref(nreq), threads, r0, r1)
    if rc < 0:
        raise ValueError("cone schedule does not end")
    r["requests"] = req[: min(nreq.value, req_cap)]
    r["n_requests"] = nreq.value
    return r


def ref_mega_available() -> bool:
    try:
        return build_ref.compile_ref_mega() is not None
    except Exception:
        return False


def ref_mega_lib() -> C.CDLL:
    global _ref_mega
    if _ref_mega is None:
        path = os.environ.get("SVO_REF_MEGA_LIB") or build_ref.compile_ref_mega()
        if path is None:
            raise RuntimeError("reference megakernel unavailable (no kernel.cl source)")
        lib = C.CDLL(path)
        lib.ref_mega_trace_rows.argtypes = [_vp, C.c_uint8, _vp, C.c_size_t, _vp, C.c_char_p, _vp, _vp, C.c_uint32,
                                            C.c_int, C.c_uint, C.c_uint, C.c_long]
        lib.ref_mega_trace_rows.restype = C.c_long
        _ref_mega = lib
    return _ref_mega


def _ref_usage(usage, n_blocks):
    """The usage array handed to the reference's kernels: the caller's entries plus
    room for the last, partial block group. The reference sizes its Usages buffer
    BlockCount >> 3 (MainWindow.cs:130), so when BlockCount is not a multiple of 8
    its updateUsage (wavefront.cl:377-381, kernel.cl's twin) stamps one entry past
    the buffer; here that entry exists and is dropped (_ref_usage_back)."""
    if usage is None:
        return None
    padded = np.zeros(max(len(usage), (n_blocks + 7) // 8 + 1), USAGE_DTYPE)
    padded[: len(usage)] = usage
    return padded


def _ref_usage_back(usage, padded):
    if usage is not None:
        usage[:] = padded[: len(usage)]


def ref_mega_trace_view(tree, inp: TraceInput, usage=None, threads: int = 0, rows=None, req_cap: int = 1 << 22,
                        cone_limit: int = 1 << 16):
    """Runs the reference's megakernel (CPU build of kernel.cl's `trace`) on one view,
    or on rows [rows[0], rows[1]) of it. usage is stamped in place. Returns rgba
    (rows outside the band stay zero) and the child requests."""
    lib = ref_mega_lib()
    w, h = inp.ScreenSize
    r0, r1 = (0, h) if rows is None else rows
    rgba = np.zeros((w * h, 4), np.float32)
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    req = np.zeros(req_cap, CHILD_REQUEST_DTYPE)
    u = _ref_usage(usage, len(blocks))
    n = lib.ref_mega_trace_rows(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), _p(u), inp.to_bytes()[:96],
                                _p(rgba), _p(req), req_cap, threads, r0, r1, cone_limit)
    _ref_usage_back(usage, u)
    if n < 0:
        raise ValueError("cone schedule does not end")
    return {"rgba": rgba, "requests": req[: min(n, req_cap)], "n_requests": int(n)}


def _result(n, counts=True):
    r = {
        "hit_index": np.empty(n, np.uint32), "hit_depth": np.empty(n, np.uint8), "t": np.empty(n, np.float32),
        "rgba": np.empty((n, 4), np.float32), "acc": np.empty((n, 4), np.uint32),
    }
    if counts:
        r.update(v_block=np.empty(n, np.uint32), v_base=np.empty(n, np.uint32), steps=np.empty(n, np.uint32))
    return r


def trace_view(tree, inp: TraceInput, usage=None, max_steps: int = 1 << 16, threads: int = 0, req_cap: int = 1 << 20,
               gi: bool = False):
    """Runs the oracle on one view. usage (USAGE_DTYPE array) is stamped in place.
    ``requests`` holds the queue in arrival order (capped at req_cap);
    ``pixel_requests`` every raised request in pixel order, whose first
    MaxChildRequestId entries are the queue of the pixel-order rule. gi: also the
    wavefront's secondary-cone stage as the reference wires it."""
    lib = oracle_lib()
    w, h = inp.ScreenSize
    n = w * h
    r = _result(n)
    requested = np.zeros(n, np.uint8)
    per_pixel = np.zeros(n, CHILD_REQUEST_DTYPE)
    vo = _ViewOut(*[_p(r[k]) for k in ("hit_index", "hit_depth", "t", "rgba", "acc", "v_block", "v_base", "steps")],
                  _p(requested), _p(per_pixel))
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    req = np.zeros(min(req_cap, n), CHILD_REQUEST_DTYPE)
    nreq = C.c_uint32(0)
    ng = 0 if usage is None else len(usage)
    limited = lib.oracle_trace_rows_gi(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), _p(usage), ng,
                                       inp.to_bytes(), max_steps, C.byref(vo), _p(req), len(req), C.byref(nreq),
                                       threads, 0, h, int(gi))
    if limited == -2:
        raise ValueError("cone schedule does not end")
    r["step_limited"] = int(limited)
    r["requests"] = req[: min(nreq.value, len(req))]
    r["n_requests"] = nreq.value
    r["pixel_requests"] = per_pixel[requested != 0]
    return r


def pixel_order_queue(per_view_requests, cap: int) -> np.ndarray:
    """The child-request queue of the pixel-order rule for a call over several
    views: the views' pixel-ordered requests concatenated in call order, the
    first ``cap`` kept."""
    allq = np.concatenate(per_view_requests) if per_view_requests else np.zeros(0, CHILD_REQUEST_DTYPE)
    return allq[:cap]


def ref_trace_view(tree, inp: TraceInput, usage=None, threads: int = 0, max_passes: int = 1 << 20, gi: bool = False):
    """Runs the reference's own kernels (CPU build) on one view; gi: with the
    secondary-cone stage that MainWindow.RunWavefront has commented out."""
    lib = ref_lib()
    w, h = inp.ScreenSize
    n = w * h
    r = _result(n, counts=False)
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    req = np.zeros(n, CHILD_REQUEST_DTYPE)
    nreq = C.c_uint32(0)
    u = _ref_usage(usage, len(blocks))
    ng = 0 if u is None else len(u)
    passes = lib.ref_trace_rows_gi(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), _p(u), ng, inp.to_bytes(),
                                   _p(r["hit_index"]), _p(r["hit_depth"]), _p(r["t"]), _p(r["rgba"]), _p(r["acc"]),
                                   _p(req), len(req), C.byref(nreq), threads, max_passes, 0, h, int(gi))
    _ref_usage_back(usage, u)
    if passes == -2:
        raise ValueError("cone schedule does not end")
    r["passes"] = int(passes)
    r["requests"] = req[: min(nreq.value, len(req))]
    r["n_requests"] = nreq.value
    return r


def ref_prune(bases, base_depth, blocks, usage, records, surface=None, locations=None, tick=1):
    """The reference's own prune kernel (CPU build of wavefront.cl) over the records,
    one work-item at a time in record order, editing bases, blocks and usage in
    place. Returns the number of records run; a negative value -(x + 1) names the
    first record the kernel cannot run faithfully (see ref_prune in
    ref_harness.c), which is not run, nor anything after it."""
    lib = ref_lib()
    rec = np.ascontiguousarray(records, PRUNING_DTYPE)
    sur = None if surface is None else np.ascontiguousarray(surface, BLOCK_DTYPE)
    loc = None if locations is None else np.ascontiguousarray(locations, np.uint64)
    for a in (bases, blocks, usage):
        assert a.flags.c_contiguous
    return int(lib.ref_prune(_p(bases), base_depth, _p(blocks), len(blocks), _p(usage), len(usage), _p(rec), len(rec),
                             _p(sur), 0 if sur is None else len(sur), _p(loc), 0 if loc is None else loc.size, tick))


def init_usage(tree) -> np.ndarray:
    u = np.zeros(len(tree.Blocks) // 8, USAGE_DTYPE)
    oracle_lib().oracle_init_usage(_p(np.ascontiguousarray(tree.BaseBlocks, np.uint16)), tree.BaseDepth, _p(u), len(u))
    return u


def sort_requests(req: np.ndarray) -> np.ndarray:
    """Child requests in a canonical order (queue order is not deterministic)."""
    if len(req) == 0:
        return req
    keys = (req["tree_size"], req["location"][:, 2], req["location"][:, 1], req["location"][:, 0], req["depth"],
            req["address"])
    return req[np.lexsort(keys)]


def trace_rows(tree, inp: TraceInput, row_begin: int, row_end: int, threads: int = 0, max_steps: int = 1 << 16):
    """Oracle over rows [row_begin, row_end) of a view (a bounded sample); returns the
    per-pixel hit_index of the band."""
    lib = oracle_lib()
    w = inp.ScreenSize[0]
    n = w * (row_end - row_begin)
    hit = np.empty(n, np.uint32)
    vo = _ViewOut(_p(hit), None, None, None, None, None, None, None)
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    nreq = C.c_uint32(0)
    lib.oracle_trace_rows(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), None, 0, inp.to_bytes(), max_steps,
                          C.byref(vo), None, 0, C.byref(nreq), threads, row_begin, row_end)
    return hit


def ref_trace_rows(tree, inp: TraceInput, row_begin: int, row_end: int, threads: int = 0):
    """The reference's kernels over rows [row_begin, row_end) of a view; returns the
    full-image hit_index (rows outside the band are misses)."""
    lib = ref_lib()
    w, h = inp.ScreenSize
    hit = np.empty(w * h, np.uint32)
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    nreq = C.c_uint32(0)
    passes = lib.ref_trace_rows(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), None, 0, inp.to_bytes(),
                                _p(hit), None, None, None, None, None, 0, C.byref(nreq), threads, 1 << 20,
                                row_begin, row_end)
    if passes < 0:
        raise RuntimeError("reference harness ran out of passes")
    return hit


class TreeState:
    """The oracle's copy of a resident tree padded to a block budget (whole groups),
    with its usage array: the state the tree-update oracle edits in place."""

    def __init__(self, tree, budget_groups: int):
        n = max(budget_groups, (len(tree.Blocks) + 7) // 8)
        self.B = tree.BaseDepth
        self.bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16).copy()
        self.blocks = np.zeros(n * 8, BLOCK_DTYPE)
        self.blocks[: len(tree.Blocks)] = tree.Blocks
        self.usage = np.zeros(n, USAGE_DTYPE)
        self.n_groups = n

    def init_usage_tree(self, tick):
        oracle_lib().oracle_init_usage_tree(_p(self.bases), self.B, _p(self.blocks), self.n_groups, _p(self.usage),
                                            tick)

    def gc(self, tick, threshold):
        n = self.n_groups
        pruned, freed, free = np.zeros(n, np.uint32), np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        out = (C.c_uint64 * 3)()
        oracle_lib().oracle_gc(_p(self.bases), self.B, _p(self.blocks), n, _p(self.usage), tick, threshold, _p(pruned),
                               _p(freed), _p(free), out)
        self.free_list = free[: out[2]].copy()
        self.free_used = 0
        return pruned[: out[0]], freed[: out[1]], self.free_list

    def graft(self, tick, records, payload, locations=None):
        rec = np.ascontiguousarray(records, GRAFTING_DTYPE)
        pay = np.ascontiguousarray(payload, BLOCK_DTYPE)
        loc = None if locations is None else np.ascontiguousarray(locations, np.uint64)
        free = self.free_list[self.free_used:]
        claimed = np.zeros(len(free), np.uint32)
        applied = np.zeros(len(rec), np.uint8)
        q = oracle_lib().oracle_graft(self.B, _p(self.blocks), self.n_groups, _p(self.usage), tick, _p(rec), len(rec),
                                      _p(pay), len(pay), _p(loc), 0 if loc is None else loc.size, _p(free), len(free),
                                      _p(claimed), _p(applied))
        self.free_used += int(q)
        return claimed[: int(q)], applied

    def prune(self, tick, records, surface=None, locations=None, req_cap=4096):
        rec = np.ascontiguousarray(records, PRUNING_DTYPE)
        sur = None if surface is None else np.ascontiguousarray(surface, BLOCK_DTYPE)
        loc = None if locations is None else np.ascontiguousarray(locations, np.uint64)
        req = np.zeros(req_cap, CHILD_REQUEST_DTYPE)
        nreq = C.c_uint32(0)
        freed = np.zeros(self.n_groups, np.uint32)
        nf = oracle_lib().oracle_prune(_p(self.bases), len(self.bases), self.B, _p(self.blocks), self.n_groups,
                                       _p(self.usage), tick, _p(rec), len(rec), _p(sur), 0 if sur is None else len(sur),
                                       _p(loc), 0 if loc is None else loc.size, _p(req), req_cap, C.byref(nreq),
                                       _p(freed))
        return freed[: int(nf)], req[: min(nreq.value, req_cap)]

    def as_octree(self):
        from svo_tracer import Octree
        return Octree(self.B, len(self.blocks), self.bases, self.blocks)


class HitLists:
    """FP64 reference of the differentiable forward model: the per-ray LOD hit
    lists of a set of views (fixed geometry), then compositing, loss and gradient
    in double precision over any parameter array."""

    def __init__(self, tree, views, max_hits=16, max_steps=1 << 16, threads=0):
        lib = oracle_lib()
        bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
        blocks = np.ascontiguousarray(tree.Blocks)
        parts = []
        for v in views:
            n = v.ScreenSize[0] * v.ScreenSize[1]
            hits = np.zeros((n, max_hits), np.uint32)
            nh = np.zeros(n, np.uint8)
            lv = np.zeros(n, np.uint8)
            sky = np.zeros((n, 3), np.float32)
            lib.oracle_hit_lists(_p(bases), tree.BaseDepth, _p(blocks), len(blocks), v.to_bytes(), max_steps,
                                 max_hits, _p(hits), _p(nh), _p(lv), _p(sky), threads)
            parts.append((hits, nh, lv, sky))
        self.hits = np.concatenate([p[0] for p in parts])
        self.n_hits = np.concatenate([p[1] for p in parts])
        self.leaves = np.concatenate([p[2] for p in parts])
        self.sky = np.concatenate([p[3] for p in parts])
        self.max_hits = max_hits
        self.n_rays = len(self.n_hits)
        self.threads = threads

    def eval(self, params, target=None, want_rgb=False, want_grad=False):
        params = np.ascontiguousarray(params, np.float64)
        tgt = None if target is None else np.ascontiguousarray(target, np.float64)
        rgb = np.zeros((self.n_rays, 3)) if want_rgb else None
        grad = np.zeros_like(params) if want_grad else None
        loss = oracle_lib().oracle_diff_eval(_p(self.hits), _p(self.n_hits), _p(self.leaves), _p(self.sky),
                                             self.n_rays, self.max_hits, _p(params), _p(tgt), _p(rgb), _p(grad),
                                             self.threads)
        return loss, rgb, grad

    def finite_differences(self, params, target, nodes, h=1e-4):
        """FP64 central differences of the loss with respect to the 4 parameters
        of each listed node, step h; [len(nodes), 4]."""
        params = np.ascontiguousarray(params, np.float64)
        tgt = np.ascontiguousarray(target, np.float64)
        nodes = np.asarray(nodes, np.uint32)
        order = np.argsort(nodes, kind="stable")
        srt = np.ascontiguousarray(nodes[order])
        assert len(np.unique(srt)) == len(srt), "nodes must be distinct"
        fd = np.zeros((len(nodes), 4))
        oracle_lib().oracle_diff_fd(_p(self.hits), _p(self.n_hits), _p(self.leaves), _p(self.sky), self.n_rays,
                                    self.max_hits, _p(params), _p(tgt), _p(srt), len(srt), h, _p(fd),
                                    self.threads)
        out = np.zeros_like(fd)
        out[order] = fd
        return out
