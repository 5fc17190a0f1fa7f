"""Python host binding of libsvo (ctypes over include/svo.h).

Mirrors the reference's host-side surface for the trace path:

* ``Octree`` / ``TreeBuilder``: SvoTracer.Domain/Models/Octree.cs and
  ITreeBuilder.BuildTree (SvoTracer.Domain/TreeBuilder.cs:102-150);
* ``TraceInput``: SvoTracer.Domain/Models/TraceInput.cs with the OpenCL layout of
  wavefront.cl:53-75;
* ``Tracer``: the ComputeManager + MainWindow.RunWavefront pair
  (SvoTracer.Kernel/ComputeManager.cs, SvoTracer.Window/MainWindow.cs:356-622).
  Errors raise ``SvoError("{method}: {code}")`` like ComputeManager.HandleResultCode
  (ComputeManager.cs:283-287).

There is no CPU fallback: if libsvo.so or a CUDA device is missing, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libsvo.so")

# ---- OpenCL struct layouts (include/svo.h) ---------------------------------------

BLOCK_DTYPE = np.dtype([
    ("child", "<u4"), ("chunk", "<u2"), ("normal_pitch", "<i2"), ("normal_yaw", "<i2"),
    ("colour_r", "u1"), ("colour_g", "u1"), ("colour_b", "u1"), ("opacity", "u1"),
    ("specularity", "u1"), ("gloss", "u1"),
])
USAGE_DTYPE = np.dtype([("tick", "<u2"), ("_pad", "<u2"), ("parent", "<u4")])
CHILD_REQUEST_DTYPE = np.dtype([
    ("address", "<u4"), ("tick", "<u2"), ("depth", "u1"), ("_pad0", "u1"),
    ("location", "<u8", (3,)), ("tree_size", "u1"), ("_pad1", "u1", (7,)),
])
GRAFTING_DTYPE = np.dtype([("graft_data_address", "<u4"), ("graft_total_size", "<u4"), ("depth", "u1"),
                           ("_pad", "u1", (3,)), ("graft_address", "<u4")])
PRUNING_DTYPE = np.dtype([("properties", "u1"), ("depth", "u1"), ("_pad0", "u1", (2,)), ("address", "<u4"),
                          ("chunk", "<u2"), ("_pad1", "u1", (2,)), ("colour_address", "<u4"), ("child_address", "<u4")])
assert BLOCK_DTYPE.itemsize == 16 and USAGE_DTYPE.itemsize == 8 and CHILD_REQUEST_DTYPE.itemsize == 40
assert GRAFTING_DTYPE.itemsize == 16 and PRUNING_DTYPE.itemsize == 20

NO_CHILD = 0xFFFFFFFF
MISS = 0xFFFFFFFF

STATUS_NAMES = {
    0: "Success", 1: "InvalidArgument", 2: "CudaError", 3: "OutOfMemory", 4: "QueueFull", 5: "Timeout",
    6: "NoTree", 7: "StepLimit", 8: "Budget", 9: "NoDevice", 10: "Internal",
}
SCENE_SPHERE, SCENE_TERRAIN = 0, 1
SCHEDULE_LANE, SCHEDULE_WARP, SCHEDULE_WAVEFRONT = 1, 2, 3
REQUESTS_ARRIVAL, REQUESTS_PIXEL = 1, 2


class SvoError(RuntimeError):
    def __init__(self, method: str, code: int, detail: str = ""):
        self.method, self.code, self.detail = method, code, detail
        super().__init__("%s: %s%s" % (method, STATUS_NAMES.get(code, str(code)), (" (%s)" % detail) if detail else ""))


class TraceInputC(C.Structure):
    _fields_ = [
        ("origin", C.c_float * 3), ("facing", C.c_float * 9), ("fov", C.c_float * 2), ("dof", C.c_float * 2),
        ("screen_size", C.c_uint32 * 2), ("max_opacity", C.c_uint8), ("base_depth", C.c_uint8),
        ("tick", C.c_uint16), ("max_child_request_id", C.c_uint32), ("fov_multiplier", C.c_float),
        ("fov_constant", C.c_float), ("weighting_multiplier", C.c_float), ("weighting_constant", C.c_float),
        ("ambient_light_level", C.c_uint8), ("_pad", C.c_uint8 * 7),
    ]


class TraceOutputC(C.Structure):
    _fields_ = [("hit_index", C.c_void_p), ("hit_depth", C.c_void_p), ("t", C.c_void_p), ("rgba", C.c_void_p),
                ("on_device", C.c_int32), ("_pad", C.c_int32)]


class TraceStatsC(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("rays", "hits", "base_steps", "block_node_reads", "block_steps",
                                           "child_requests", "step_limited")]


class TraceConfigC(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("block_size", "ctas_per_sm", "ray_chunk", "cadence", "max_steps",
                                          "collect_stats", "max_hits", "schedule", "mega_band_tiles", "l2_window",
                                          "pass_limit", "request_order", "gi_stage")]


class SceneParamsC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("seed", C.c_uint32), ("base_depth", C.c_uint8), ("max_depth", C.c_uint8),
                ("_pad", C.c_uint8 * 2), ("threads", C.c_int32), ("max_size", C.c_uint64)]


class UpdateInputC(C.Structure):
    _fields_ = [("base_depth", C.c_uint8), ("_pad", C.c_uint8), ("tick", C.c_uint16),
                ("max_child_request_id", C.c_uint32), ("memory_size", C.c_uint32), ("offset", C.c_uint32),
                ("graft_size", C.c_uint32)]


class GcReportC(C.Structure):
    _fields_ = [("pruned", C.c_uint64), ("freed", C.c_uint64), ("free", C.c_uint64)]


class GraftReportC(C.Structure):
    _fields_ = [("applied", C.c_uint32), ("skipped", C.c_uint32), ("claimed", C.c_uint64), ("free_left", C.c_uint64)]


class MegaStatsC(C.Structure):
    _fields_ = [("pixels", C.c_uint64), ("surfaces", C.c_uint64), ("cones", C.c_uint64), ("cone_slots", C.c_uint64)]


class PruneReportC(C.Structure):
    _fields_ = [("freed", C.c_uint64), ("requests", C.c_uint32), ("_pad", C.c_uint32)]


assert C.sizeof(TraceInputC) == 104 and C.sizeof(UpdateInputC) == 20

_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads libsvo.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise SvoError("load_library", 9, "libsvo.so not built at %s; run __graft_entry__.build()" % p)
    lib = C.CDLL(p)
    vp, sz = C.c_void_p, C.c_size_t
    sig = {
        "svo_last_error_string": ([], C.c_char_p),
        "svo_version": ([], C.c_char_p),
        "svo_create": ([C.c_int32, C.POINTER(vp)], C.c_int32),
        "svo_destroy": ([vp], C.c_int32),
        "svo_set_stream": ([vp, vp], C.c_int32),
        "svo_synchronize": ([vp], C.c_int32),
        "svo_set_trace_config": ([vp, C.POINTER(TraceConfigC)], C.c_int32),
        "svo_get_trace_config": ([vp, C.POINTER(TraceConfigC)], C.c_int32),
        "svo_upload_octree": ([vp, C.c_uint8, vp, sz, vp, sz, C.c_uint32], C.c_int32),
        "svo_init_usage": ([vp], C.c_int32),
        "svo_read_usage": ([vp, vp, sz], C.c_int32),
        "svo_write_usage": ([vp, vp, sz], C.c_int32),
        "svo_read_blocks": ([vp, vp, sz, sz], C.c_int32),
        "svo_read_bases": ([vp, vp, sz], C.c_int32),
        "svo_tree_size": ([vp, C.POINTER(C.c_uint8), C.POINTER(sz), C.POINTER(sz), C.POINTER(sz)], C.c_int32),
        "svo_trace": ([vp, C.POINTER(TraceInputC), C.POINTER(TraceOutputC)], C.c_int32),
        "svo_trace_batch": ([vp, C.POINTER(TraceInputC), C.c_int32, C.POINTER(TraceOutputC)], C.c_int32),
        "svo_trace_batch_graph": ([vp, C.POINTER(TraceInputC), C.c_int32, C.POINTER(TraceOutputC)], C.c_int32),
        "svo_last_trace_stats": ([vp, C.POINTER(TraceStatsC)], C.c_int32),
        "svo_mega_trace": ([vp, C.POINTER(TraceInputC), C.POINTER(TraceOutputC)], C.c_int32),
        "svo_last_mega_stats": ([vp, C.POINTER(MegaStatsC)], C.c_int32),
        "svo_autotune": ([vp, C.POINTER(TraceInputC), C.c_int32, C.POINTER(TraceOutputC), C.c_int32,
                          C.POINTER(TraceConfigC), C.POINTER(C.c_float)], C.c_int32),
        "svo_read_ray_counts": ([vp, vp, vp, sz], C.c_int32),
        "svo_read_child_requests": ([vp, vp, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int32),
        "svo_tree_build": ([C.POINTER(SceneParamsC), C.POINTER(vp)], C.c_int32),
        "svo_tree_info": ([vp, C.POINTER(C.c_uint8), C.POINTER(sz), C.POINTER(sz), C.POINTER(C.c_uint32)], C.c_int32),
        "svo_tree_data": ([vp, C.POINTER(vp), C.POINTER(vp)], C.c_int32),
        "svo_tree_free": ([vp], C.c_int32),
        "svo_init_usage_tree": ([vp, C.c_uint16], C.c_int32),
        "svo_graft_generate": ([vp, vp, C.POINTER(UpdateInputC), C.POINTER(GraftReportC)], C.c_int32),
        "svo_oct_write": ([C.c_char_p, C.c_uint8, C.c_uint32, vp, sz, vp, sz], C.c_int32),
        "svo_oct_read": ([C.c_char_p, C.POINTER(C.c_void_p)], C.c_int32),
        "svo_state_save": ([vp, C.c_char_p], C.c_int32),
        "svo_state_load": ([vp, C.c_char_p], C.c_int32),
        "svo_diff_set_params": ([vp, vp, sz, C.c_int32], C.c_int32),
        "svo_diff_get_grads": ([vp, vp, sz, C.c_int32], C.c_int32),
        "svo_diff_forward": ([vp, C.POINTER(TraceInputC), C.c_int32, vp, C.c_int32], C.c_int32),
        "svo_diff_backward": ([vp, C.POINTER(TraceInputC), C.c_int32, vp, C.c_int32, C.c_int32,
                               C.POINTER(C.c_double)],
                              C.c_int32),
        "svo_gc": ([vp, C.POINTER(UpdateInputC), C.POINTER(GcReportC)], C.c_int32),
        "svo_read_gc_lists": ([vp, vp, sz, vp, sz, vp, sz], C.c_int32),
        "svo_graft": ([vp, C.POINTER(UpdateInputC), vp, C.c_uint32, vp, sz, vp, sz, C.POINTER(GraftReportC)], C.c_int32),
        "svo_read_graft_claims": ([vp, vp, sz], C.c_int32),
        "svo_prune": ([vp, C.POINTER(UpdateInputC), vp, C.c_uint32, vp, sz, vp, sz, C.POINTER(PruneReportC)], C.c_int32),
        "svo_scene_create": ([C.POINTER(SceneParamsC), C.POINTER(vp)], C.c_int32),
        "svo_scene_build_tree": ([vp, C.c_uint8, C.POINTER(vp)], C.c_int32),
        "svo_scene_graft_payload": ([vp, vp, sz, C.POINTER(vp)], C.c_int32),
        "svo_graft_payload_data": ([vp, C.POINTER(vp), C.POINTER(sz), C.POINTER(vp), C.POINTER(sz)], C.c_int32),
        "svo_graft_payload_free": ([vp], C.c_int32),
        "svo_scene_free": ([vp], C.c_int32),
        "svo_trace_noalloc": ([C.c_int32, vp, C.c_uint8, vp, sz, vp, sz, vp, sz, C.c_int32, C.POINTER(TraceInputC),
                               C.POINTER(TraceOutputC), vp, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _check(method: str, status: int) -> None:
    if status != 0:
        detail = load_library().svo_last_error_string().decode(errors="replace")
        raise SvoError(method, status, detail)


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---- domain types ------------------------------------------------------------------


@dataclass
class Octree:
    """SvoTracer.Domain/Models/Octree.cs: BaseDepth, BlockCount, BaseBlocks, Blocks."""
    BaseDepth: int
    BlockCount: int
    BaseBlocks: np.ndarray  # uint16[powSum(BaseDepth)]
    Blocks: np.ndarray      # BLOCK_DTYPE[n]

    @property
    def n_groups(self) -> int:
        return len(self.Blocks) // 8


def pow_sum(depth: int) -> int:
    return sum(8 ** i for i in range(1, depth + 1))


def _tree_from_handle(lib, h) -> "Octree":
    try:
        bd, nb, nk, bc = C.c_uint8(), C.c_size_t(), C.c_size_t(), C.c_uint32()
        _check("BuildTree", lib.svo_tree_info(h, C.byref(bd), C.byref(nb), C.byref(nk), C.byref(bc)))
        pb, pk = C.c_void_p(), C.c_void_p()
        _check("BuildTree", lib.svo_tree_data(h, C.byref(pb), C.byref(pk)))
        bases = np.zeros(nb.value, np.uint16)
        raw = np.zeros(nk.value * 16, np.uint8)
        if nb.value:
            C.memmove(bases.ctypes.data, pb.value, bases.nbytes)
        if nk.value:
            C.memmove(raw.ctypes.data, pk.value, raw.nbytes)
        return Octree(bd.value, bc.value, bases, raw.view(BLOCK_DTYPE))
    finally:
        lib.svo_tree_free(h)


def write_oct(path: str, tree: Octree) -> None:
    """OctreeSerializer.Serialize (SvoTracer.Domain/Serializers/OctreeSerializer.cs:13-21)."""
    lib = load_library()
    bases = np.ascontiguousarray(tree.BaseBlocks, np.uint16)
    blocks = np.ascontiguousarray(tree.Blocks)
    assert blocks.dtype == BLOCK_DTYPE
    _check("SaveTree", lib.svo_oct_write(os.fsencode(path), tree.BaseDepth, tree.BlockCount, _ptr(bases), len(bases),
                                         _ptr(blocks), len(blocks)))


def read_oct(path: str) -> Octree:
    """OctreeSerializer.Deserialize (OctreeSerializer.cs:23-44): BlockCount blocks."""
    lib = load_library()
    h = C.c_void_p()
    _check("LoadTree", lib.svo_oct_read(os.fsencode(path), C.byref(h)))
    return _tree_from_handle(lib, h)


def map_oct(path: str) -> Octree:
    """The same file as read_oct, mapped with numpy alone (libsvo is not loaded): the
    header, the base chunks and BlockCount blocks as read-only memory maps."""
    head = np.fromfile(path, dtype=np.uint8, count=5)
    if len(head) < 5:
        raise SvoError("LoadTree", 11, "truncated header: " + path)
    base_depth = int(head[0])
    block_count = int(head[1]) | int(head[2]) << 8 | int(head[3]) << 16 | int(head[4]) << 24
    n_bases = pow_sum(base_depth)
    need = 5 + 2 * n_bases + BLOCK_DTYPE.itemsize * block_count
    if os.path.getsize(path) < need:
        raise SvoError("LoadTree", 11, "%s holds %d bytes, the header needs %d" % (path, os.path.getsize(path), need))
    bases = np.memmap(path, dtype="<u2", mode="r", offset=5, shape=(n_bases,))
    blocks = np.memmap(path, dtype=BLOCK_DTYPE, mode="r", offset=5 + 2 * n_bases, shape=(block_count,))
    return Octree(base_depth, block_count, bases, blocks)


class TreeManager:
    """ITreeManager over `{path}/{fileName}.oct` (SvoTracer.Domain/TreeManager.cs)."""

    def __init__(self, path: str):
        self._path = path

    def _file(self, fileName: str) -> str:
        return os.path.join(self._path, fileName + ".oct")

    def TreeExists(self, fileName: str) -> bool:
        return os.path.exists(self._file(fileName))

    def DeleteTree(self, fileName: str) -> None:
        os.remove(self._file(fileName))

    def LoadTree(self, fileName: str) -> Octree:
        return read_oct(self._file(fileName))

    def SaveTree(self, fileName: str, tree: Octree) -> None:
        os.makedirs(self._path, exist_ok=True)
        write_oct(self._file(fileName), tree)


class Scene:
    """A persistent procedural scene: builds the resident tree and the graft
    payloads of the streaming workflow (depth = deepest node level it produces)."""

    def __init__(self, scene: int = SCENE_TERRAIN, seed: int = 1, base_depth: int = 4, depth: int = 12,
                 threads: int = 0):
        self._lib = load_library()
        self._h = C.c_void_p()
        p = SceneParamsC(kind=scene, seed=seed, base_depth=base_depth, max_depth=depth, threads=threads, max_size=0)
        _check("SceneCreate", self._lib.svo_scene_create(C.byref(p), C.byref(self._h)))
        self.base_depth, self.depth = base_depth, depth

    def close(self):
        if self._h:
            self._lib.svo_scene_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_tree(self, max_depth: int) -> "Octree":
        h = C.c_void_p()
        _check("BuildTree", self._lib.svo_scene_build_tree(self._h, max_depth, C.byref(h)))
        return _tree_from_handle(self._lib, h)

    def graft_payload(self, requests: np.ndarray):
        req = np.ascontiguousarray(requests, dtype=CHILD_REQUEST_DTYPE)
        h = C.c_void_p()
        _check("GraftPayload", self._lib.svo_scene_graft_payload(self._h, _ptr(req), len(req), C.byref(h)))
        try:
            pr, nr, pp, npay = C.c_void_p(), C.c_size_t(), C.c_void_p(), C.c_size_t()
            _check("GraftPayload", self._lib.svo_graft_payload_data(h, C.byref(pr), C.byref(nr), C.byref(pp),
                                                                      C.byref(npay)))
            rec = np.zeros(nr.value, GRAFTING_DTYPE)
            pay = np.zeros(npay.value, BLOCK_DTYPE)
            if nr.value:
                C.memmove(rec.ctypes.data, pr.value, nr.value * 16)
            if npay.value:
                C.memmove(pay.ctypes.data, pp.value, npay.value * 16)
            return rec, pay
        finally:
            self._lib.svo_graft_payload_free(h)


class TreeBuilder:
    """ITreeBuilder over the seeded procedural scenes (sphere, terrain)."""

    def __init__(self, scene: int = SCENE_SPHERE, seed: int = 1, threads: int = 0):
        self.scene, self.seed, self.threads = scene, seed, threads

    def BuildTree(self, baseDepth: int, maxDepth: int, maxSize: int = 0) -> Octree:
        lib = load_library()
        p = SceneParamsC(kind=self.scene, seed=self.seed, base_depth=baseDepth, max_depth=maxDepth,
                         threads=self.threads, max_size=maxSize)
        h = C.c_void_p()
        _check("BuildTree", lib.svo_tree_build(C.byref(p), C.byref(h)))
        try:
            bd, nb, nk, bc = C.c_uint8(), C.c_size_t(), C.c_size_t(), C.c_uint32()
            _check("BuildTree", lib.svo_tree_info(h, C.byref(bd), C.byref(nb), C.byref(nk), C.byref(bc)))
            pb, pk = C.c_void_p(), C.c_void_p()
            _check("BuildTree", lib.svo_tree_data(h, C.byref(pb), C.byref(pk)))
            bases = np.ctypeslib.as_array(C.cast(pb, C.POINTER(C.c_uint16)), shape=(nb.value,)).copy()
            raw = np.ctypeslib.as_array(C.cast(pk, C.POINTER(C.c_uint8)), shape=(nk.value * 16,)).copy()
            blocks = raw.view(BLOCK_DTYPE)
            return Octree(bd.value, bc.value, bases, blocks)
        finally:
            lib.svo_tree_free(h)

    build_tree = BuildTree


@dataclass
class TraceInput:
    """SvoTracer.Domain/Models/TraceInput.cs. Facing is column-major (forward, right, up columns)."""
    Origin: tuple = (0.0, 0.0, 0.0)
    Facing: tuple = (1, 0, 0, 0, 1, 0, 0, 0, 1)
    FoV: tuple = (math.pi / 4, math.pi / 4)
    DoF: tuple = (0.0, 0.0)
    ScreenSize: tuple = (640, 480)
    MaxOpacity: int = 200
    BaseDepth: int = 0
    Tick: int = 1
    MaxChildRequestId: int = 6000
    FovMultiplier: float = 0.2
    FovConstant: float = 0.2
    WeightingMultiplier: float = -0.05
    WeightingConstant: float = 0.5
    AmbientLightLevel: int = 100

    def to_c(self) -> TraceInputC:
        c = TraceInputC()
        c.origin[:] = [float(v) for v in self.Origin]
        c.facing[:] = [float(v) for v in self.Facing]
        c.fov[:] = [float(v) for v in self.FoV]
        c.dof[:] = [float(v) for v in self.DoF]
        c.screen_size[:] = [int(v) for v in self.ScreenSize]
        c.max_opacity = self.MaxOpacity
        c.base_depth = self.BaseDepth
        c.tick = self.Tick
        c.max_child_request_id = self.MaxChildRequestId
        c.fov_multiplier = self.FovMultiplier
        c.fov_constant = self.FovConstant
        c.weighting_multiplier = self.WeightingMultiplier
        c.weighting_constant = self.WeightingConstant
        c.ambient_light_level = self.AmbientLightLevel
        return c

    def to_bytes(self) -> bytes:
        return bytes(self.to_c())


def look_at(origin, target, width: int, height: int, fov_deg: float, up=(0.0, 0.0, -1.0), **kw) -> TraceInput:
    """Camera at `origin` (unit-cube coordinates) looking at `target`.

    World up is -z (the reference lights its sky from -z, wavefront.cl:1756). FoV[0]
    is the horizontal angle and FoV[1] = FoV[0] * H / W (equi-angular rays)."""
    o = np.asarray(origin, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - o
    f /= np.linalg.norm(f)
    u = np.asarray(up, dtype=np.float64)
    r = np.cross(f, u)
    if np.linalg.norm(r) < 1e-9:
        r = np.cross(f, np.array([1.0, 0.0, 0.0]))
    r /= np.linalg.norm(r)
    u2 = np.cross(r, f)
    facing = tuple(float(v) for v in np.concatenate([f, r, u2]).astype(np.float32))
    fx = math.radians(fov_deg)
    return TraceInput(Origin=tuple(float(v) for v in np.float32(o)), Facing=facing,
                      FoV=(float(np.float32(fx)), float(np.float32(fx * height / width))),
                      ScreenSize=(width, height), **kw)


def mixed_views(seed: int = 4, n: int = 64, **kw):
    """The batched multi-view workload: n cameras whose pixel counts are drawn
    log-uniformly between 128x128 and 1920x1080 with aspect ratios in {1, 4/3, 16/9},
    placed uniformly on spheres of radius 1.2-2.0 (world units, [-1,1]^3 maps to the
    unit cube: radius 0.6-1.0 around its centre), looking at seeded targets within 0.2
    world units of the centre, horizontal FoV uniform in 40-90 degrees."""
    rng = np.random.default_rng(seed)
    views = []
    lo, hi = math.log(128 * 128), math.log(1920 * 1080)
    for _ in range(n):
        px = math.exp(rng.uniform(lo, hi))
        aspect = [1.0, 4.0 / 3.0, 16.0 / 9.0][int(rng.integers(0, 3))]
        h = max(1, int(round(math.sqrt(px / aspect))))
        w = max(1, int(round(h * aspect)))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        radius = rng.uniform(1.2, 2.0) * 0.5
        t = rng.normal(size=3)
        t *= rng.uniform(0.0, 0.2) * 0.5 / max(np.linalg.norm(t), 1e-12)
        target = 0.5 + t
        origin = 0.5 + radius * d
        views.append(look_at(origin, target, w, h, rng.uniform(40.0, 90.0), **kw))
    return views


def camera_path(seed: int = 3, frames: int = 120, width: int = 1920, height: int = 1080, fov: float = 60.0,
                n_points: int = 8, **kw):
    """The streaming workload's camera: a Catmull-Rom spline through n_points seeded
    control points at heights 0.35-0.6 above the terrain's base (unit-cube z = 1 - h,
    up is -z), sampled at `frames` evenly spaced parameters; each frame looks ahead
    along the path and down towards the terrain. Frame f carries Tick f + 1."""
    rng = np.random.default_rng(seed)
    pts = np.stack([rng.uniform(0.1, 0.9, n_points), rng.uniform(0.1, 0.9, n_points),
                    1.0 - rng.uniform(0.35, 0.6, n_points)], axis=1)

    def spline(u):
        seg = min(int(u), n_points - 4)
        t = u - seg
        p0, p1, p2, p3 = pts[seg], pts[seg + 1], pts[seg + 2], pts[seg + 3]
        return 0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t * t +
                      (-p0 + 3 * p1 - 3 * p2 + p3) * t * t * t)

    span = n_points - 3
    out = []
    for f in range(frames):
        u = span * f / max(frames - 1, 1)
        pos = spline(u)
        ahead = spline(min(span, u + 0.05 * span))
        if np.linalg.norm(ahead - pos) < 1e-6:
            ahead = pos + (pts[-2] - pts[1])
        target = ahead + np.array([0.0, 0.0, 0.25])
        out.append(look_at(pos, target, width, height, fov, Tick=f + 1, **kw))
    return out


def node_cells(tree: Octree):
    """Integer cell coordinates (at the node's own depth) and depth of every node
    reachable from the dense level B+2; unreachable nodes get depth 0. The dense
    level is indexed by baseLocation(B + 2) (wavefront.cl:405-411), but only the
    groups below a mixed level-(B+1) base octant hold level-(B+2) nodes
    (PopulateInitialBlocks, TreeBuilder.cs:180-227); the others are reused for
    deeper groups. Node `child + o` of a depth-d node is the octant
    o = x + 2y + 4z (chunkPosition, wavefront.cl:428-430) of its cell at depth d + 1."""
    B = tree.BaseDepth
    d0 = B + 2
    n = len(tree.Blocks)
    child = tree.Blocks["child"]
    cells = np.zeros((n, 3), np.int64)
    depth = np.zeros(n, np.uint8)
    pos = np.arange(8 ** (B + 1), dtype=np.int64)
    chunk = tree.BaseBlocks[pow_sum(B - 1) + (pos >> 3)].astype(np.int64)
    populated = pos[((chunk >> ((pos & 7) * 2)) & 3) == 3]
    front = (populated[:, None] * 8 + np.arange(8)).reshape(-1)
    front = front[front < n]
    xyz = np.zeros((len(front), 3), np.int64)
    for i in range(d0):
        dig = (front >> (3 * (d0 - 1 - i))) & 7
        xyz = xyz * 2 + np.stack([dig & 1, (dig >> 1) & 1, (dig >> 2) & 1], axis=1)
    cells[front] = xyz
    depth[front] = d0
    octs = np.array([[o & 1, (o >> 1) & 1, (o >> 2) & 1] for o in range(8)], np.int64)
    d = d0
    while len(front):
        ch = child[front]
        keep = ch != 0xFFFFFFFF
        par, first = front[keep], ch[keep].astype(np.int64)
        kids = (first[:, None] + np.arange(8)).reshape(-1)
        kc = (cells[par][:, None, :] * 2 + octs[None]).reshape(-1, 3)
        ok = (kids < n) & (depth[np.minimum(kids, n - 1)] == 0)
        kids, kc = kids[ok], kc[ok]
        cells[kids] = kc
        depth[kids] = d + 1
        front = kids
        d += 1
    return cells, depth


def sinusoid_field(tree: Octree, seed: int = 9, opacity: float = 0.9) -> np.ndarray:
    """Ground-truth per-node RGBA of the differentiable colour-fitting workload:
    channel k = 0.5 + 0.5 sin(2 pi f_k (u_k . x) + phi_k) at the node's cell
    centre x, with a seeded frequency f_k uniform in [1, 4], a seeded unit
    direction u_k and phase phi_k; alpha = `opacity`. float32 [n_nodes, 4]."""
    rng = np.random.default_rng(seed)
    cells, depth = node_cells(tree)
    centre = (cells + 0.5) / np.exp2(depth.astype(np.float64))[:, None]
    out = np.zeros((len(cells), 4), np.float32)
    for k in range(3):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        f = rng.uniform(1.0, 4.0)
        phi = rng.uniform(0.0, 2.0 * math.pi)
        out[:, k] = 0.5 + 0.5 * np.sin(2.0 * math.pi * f * (centre @ u) + phi)
    out[:, 3] = opacity
    out[depth == 0] = 0.0
    return out


def orbit_views(seed: int = 11, n: int = 16, width: int = 512, height: int = 512, distance: float = 1.5,
                fov: float = 60.0, centre=(0.5, 0.5, 0.5), **kw):
    """n pinhole views at `distance` from `centre` on seeded directions, looking
    at the centre (the colour-fitting workload's target views)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        out.append(look_at(np.asarray(centre) + distance * u, centre, width, height, fov, **kw))
    return out


@dataclass
class TraceResult:
    hit_index: np.ndarray
    hit_depth: np.ndarray
    t: np.ndarray
    rgba: np.ndarray


class Tracer:
    """Context of one GPU: octree residency, usage ticks, child requests, traces."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        self._ctx = C.c_void_p()
        self._req_cap = 0
        _check("ComputeManagerFactory.Build", self._lib.svo_create(device, C.byref(self._ctx)))

    # ComputeManager.Dispose
    def close(self) -> None:
        if self._ctx:
            self._lib.svo_destroy(self._ctx)
            self._ctx = C.c_void_p()

    Dispose = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._ctx

    def set_stream(self, stream_ptr: int | None) -> None:
        _check("SetStream", self._lib.svo_set_stream(self._ctx, C.c_void_p(stream_ptr or 0)))

    def synchronize(self) -> None:
        _check("Synchronize", self._lib.svo_synchronize(self._ctx))

    def set_config(self, **kw) -> None:
        cfg = self.get_config()
        for k, v in kw.items():
            setattr(cfg, k, int(v))
        _check("SetTraceConfig", self._lib.svo_set_trace_config(self._ctx, C.byref(cfg)))

    def get_config(self) -> TraceConfigC:
        cfg = TraceConfigC()
        _check("GetTraceConfig", self._lib.svo_get_trace_config(self._ctx, C.byref(cfg)))
        return cfg

    # MainWindow.SetupWavefrontKernels: InitReadBuffer(Bases, Blocks)
    def upload(self, tree: Octree, block_budget: int = 0) -> None:
        bases = np.ascontiguousarray(tree.BaseBlocks, dtype=np.uint16)
        blocks = np.ascontiguousarray(tree.Blocks)
        assert blocks.dtype == BLOCK_DTYPE
        _check("InitReadBuffer", self._lib.svo_upload_octree(self._ctx, tree.BaseDepth, _ptr(bases), len(bases),
                                                             _ptr(blocks), len(blocks), block_budget))

    def init_usage(self) -> None:
        _check("InitUsage", self._lib.svo_init_usage(self._ctx))

    def tree_size(self):
        bd, nb, nk, bu = C.c_uint8(), C.c_size_t(), C.c_size_t(), C.c_size_t()
        _check("TreeSize", self._lib.svo_tree_size(self._ctx, C.byref(bd), C.byref(nb), C.byref(nk), C.byref(bu)))
        return bd.value, nb.value, nk.value, bu.value

    def read_usage(self, n_groups: int | None = None) -> np.ndarray:
        if n_groups is None:
            n_groups = self.tree_size()[3] // 8
        out = np.zeros(n_groups, dtype=USAGE_DTYPE)
        _check("ReadBuffer:Usages", self._lib.svo_read_usage(self._ctx, _ptr(out), n_groups))
        return out

    def write_usage(self, usage: np.ndarray) -> None:
        u = np.ascontiguousarray(usage, dtype=USAGE_DTYPE)
        _check("WriteBuffer:Usages", self._lib.svo_write_usage(self._ctx, _ptr(u), len(u)))

    def save_state(self, path: str) -> None:
        """Checkpoint of the streaming state (tree, usage, tree depth, free list)."""
        _check("SaveState", self._lib.svo_state_save(self._ctx, os.fsencode(path)))

    def load_state(self, path: str) -> None:
        """Resume from a checkpoint: replaces the resident tree and its state."""
        _check("LoadState", self._lib.svo_state_load(self._ctx, os.fsencode(path)))

    def read_blocks(self, first: int = 0, n: int | None = None) -> np.ndarray:
        if n is None:
            n = self.tree_size()[3] - first
        out = np.zeros(n, dtype=BLOCK_DTYPE)
        _check("ReadBuffer:Blocks", self._lib.svo_read_blocks(self._ctx, _ptr(out), first, n))
        return out

    @staticmethod
    def _alloc(w: int, h: int) -> TraceResult:
        n = w * h
        return TraceResult(np.empty(n, np.uint32), np.empty(n, np.uint8), np.empty(n, np.float32),
                           np.empty((n, 4), np.float32))

    @staticmethod
    def _out(r: TraceResult) -> TraceOutputC:
        return TraceOutputC(_ptr(r.hit_index), _ptr(r.hit_depth), _ptr(r.t), _ptr(r.rgba), 0, 0)

    # MainWindow.RunWavefront for one view, results in host memory
    def trace(self, inp: TraceInput, out: TraceResult | None = None) -> TraceResult:
        r = out if out is not None else self._alloc(*inp.ScreenSize)
        c_in, c_out = inp.to_c(), self._out(r)
        self._req_cap = inp.MaxChildRequestId
        _check("RunWavefront", self._lib.svo_trace(self._ctx, C.byref(c_in), C.byref(c_out)))
        return r

    def mega_trace(self, inp: TraceInput, out: TraceResult | None = None) -> TraceResult:
        """kernel.cl's `trace` (the megakernel): the primary cone, spawnRays's cone
        fan and draw's colour. hit_index/hit_depth/t describe the primary cone."""
        r = out if out is not None else self._alloc(*inp.ScreenSize)
        c_in, c_out = inp.to_c(), self._out(r)
        self._req_cap = inp.MaxChildRequestId
        _check("RunMegakernel", self._lib.svo_mega_trace(self._ctx, C.byref(c_in), C.byref(c_out)))
        return r

    def mega_trace_device(self, inp: TraceInput, hit_index=0, hit_depth=0, t=0, rgba=0) -> None:
        """The megakernel into caller-owned device buffers (addresses, 0 = skip)."""
        c_out = TraceOutputC(hit_index or None, hit_depth or None, t or None, rgba or None, 1, 0)
        self._req_cap = inp.MaxChildRequestId
        _check("RunMegakernelDevice", self._lib.svo_mega_trace(self._ctx, C.byref(inp.to_c()), C.byref(c_out)))

    def mega_stats(self) -> dict:
        s = MegaStatsC()
        _check("MegaStats", self._lib.svo_last_mega_stats(self._ctx, C.byref(s)))
        return {n: getattr(s, n) for n, _ in MegaStatsC._fields_}

    def trace_batch(self, inputs, graph: bool = False, out=None):
        """Many views in one launch; `out`, when given, holds one TraceResult per
        view (arrays may be None to skip an output)."""
        res = list(out) if out is not None else [self._alloc(*i.ScreenSize) for i in inputs]
        c_in = (TraceInputC * len(inputs))(*[i.to_c() for i in inputs])
        c_out = (TraceOutputC * len(inputs))(*[self._out(r) for r in res])
        fn = self._lib.svo_trace_batch_graph if graph else self._lib.svo_trace_batch
        self._req_cap = max(i.MaxChildRequestId for i in inputs)
        _check("RunWavefrontBatch", fn(self._ctx, c_in, len(inputs), c_out))
        return res

    def trace_device(self, inputs, outputs, graph: bool = False) -> None:
        """Trace into caller-owned device buffers: outputs is a list of
        (hit_index_ptr, hit_depth_ptr, t_ptr, rgba_ptr) device addresses (0 = skip)."""
        c_in = (TraceInputC * len(inputs))(*[i.to_c() for i in inputs])
        c_out = (TraceOutputC * len(inputs))(*[TraceOutputC(o[0] or None, o[1] or None, o[2] or None, o[3] or None, 1, 0)
                                               for o in outputs])
        fn = self._lib.svo_trace_batch_graph if graph else self._lib.svo_trace_batch
        self._req_cap = max(i.MaxChildRequestId for i in inputs)
        _check("RunWavefrontDevice", fn(self._ctx, c_in, len(inputs), c_out))

    def autotune(self, inputs, outputs, repeats: int = 3):
        """Picks the fastest launch configuration for this view set (device outputs,
        as for trace_device); returns (config dict, milliseconds)."""
        c_in = (TraceInputC * len(inputs))(*[i.to_c() for i in inputs])
        c_out = (TraceOutputC * len(inputs))(*[TraceOutputC(o[0] or None, o[1] or None, o[2] or None, o[3] or None, 1, 0)
                                               for o in outputs])
        best = TraceConfigC()
        ms = C.c_float()
        self._req_cap = max(i.MaxChildRequestId for i in inputs)
        _check("Autotune", self._lib.svo_autotune(self._ctx, c_in, len(inputs), c_out, repeats, C.byref(best),
                                                  C.byref(ms)))
        return {n: getattr(best, n) for n, _ in TraceConfigC._fields_ if not n.startswith("_")}, ms.value

    def stats(self) -> dict:
        s = TraceStatsC()
        _check("TraceStats", self._lib.svo_last_trace_stats(self._ctx, C.byref(s)))
        return {n: getattr(s, n) for n, _ in TraceStatsC._fields_}

    def ray_counts(self, n: int):
        vb, vs = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        _check("RayCounts", self._lib.svo_read_ray_counts(self._ctx, _ptr(vb), _ptr(vs), n))
        return vb, vs

    # ---- differentiable colour fitting ----------------------------------------
    def diff_set_params(self, rgba: np.ndarray) -> None:
        p = np.ascontiguousarray(rgba, np.float32).reshape(-1, 4)
        _check("DiffSetParams", self._lib.svo_diff_set_params(self._ctx, _ptr(p), len(p), 0))

    def diff_grads(self, n_nodes: int, out: np.ndarray | None = None) -> np.ndarray:
        g = np.zeros((n_nodes, 4), np.float32) if out is None else out
        assert g.dtype == np.float32 and g.flags.c_contiguous and g.size >= 4 * n_nodes
        _check("DiffGrads", self._lib.svo_diff_get_grads(self._ctx, _ptr(g), n_nodes, 0))
        return g

    def diff_forward(self, views, out: np.ndarray | None = None) -> np.ndarray:
        """Composited colour, 3 floats per pixel; `out` (float32, C-contiguous) may
        be a caller's buffer, written in place (by the kernel when it is pinned)."""
        n = sum(v.ScreenSize[0] * v.ScreenSize[1] for v in views)
        if out is None:
            out = np.zeros((n, 3), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * n
        c_in = (TraceInputC * len(views))(*[v.to_c() for v in views])
        _check("DiffForward", self._lib.svo_diff_forward(self._ctx, c_in, len(views), _ptr(out), 0))
        return out

    def diff_backward(self, views, target: np.ndarray, use_saved: bool = False) -> float:
        """Loss and per-node gradients (read with diff_grads). use_saved: take the
        colour from the last diff_forward over the same views and parameters
        (one traversal per ray instead of two)."""
        t = np.ascontiguousarray(target, np.float32).reshape(-1, 3)
        loss = C.c_double()
        c_in = (TraceInputC * len(views))(*[v.to_c() for v in views])
        _check("DiffBackward", self._lib.svo_diff_backward(self._ctx, c_in, len(views), _ptr(t), int(use_saved), 0,
                                                           C.byref(loss)))
        return loss.value

    def diff_set_params_device(self, ptr: int, n_nodes: int) -> None:
        _check("DiffSetParams", self._lib.svo_diff_set_params(self._ctx, C.c_void_p(ptr), n_nodes, 1))

    def diff_forward_device(self, views, rgb_ptr: int) -> None:
        """Forward colour into a caller-owned device buffer (3 floats per ray)."""
        c_in = (TraceInputC * len(views))(*[v.to_c() for v in views])
        _check("DiffForward", self._lib.svo_diff_forward(self._ctx, c_in, len(views), C.c_void_p(rgb_ptr), 1))

    def diff_backward_device(self, views, target_ptr: int, use_saved: bool = False) -> None:
        """Backward against a device-resident target; the loss stays on the device
        (no synchronisation) and the gradients in the context."""
        c_in = (TraceInputC * len(views))(*[v.to_c() for v in views])
        _check("DiffBackward", self._lib.svo_diff_backward(self._ctx, c_in, len(views), C.c_void_p(target_ptr),
                                                           int(use_saved), 1, None))

    # ---- tree updates --------------------------------------------------------
    @staticmethod
    def _update(tick: int, offset: int = 0) -> UpdateInputC:
        return UpdateInputC(0, 0, tick, 0, 0, offset, 0)

    def init_usage_tree(self, tick: int) -> None:
        _check("InitUsageTree", self._lib.svo_init_usage_tree(self._ctx, tick))

    def gc(self, tick: int, threshold: int) -> dict:
        rep = GcReportC()
        _check("GC", self._lib.svo_gc(self._ctx, C.byref(self._update(tick, threshold)), C.byref(rep)))
        return {"pruned": rep.pruned, "freed": rep.freed, "free": rep.free}

    def gc_lists(self, n_pruned: int, n_freed: int, n_free: int):
        a, b, c = (np.zeros(max(n, 1), np.uint32) for n in (n_pruned, n_freed, n_free))
        _check("GcLists", self._lib.svo_read_gc_lists(self._ctx, _ptr(a), n_pruned, _ptr(b), n_freed, _ptr(c), n_free))
        return a[:n_pruned], b[:n_freed], c[:n_free]

    def graft(self, tick: int, records: np.ndarray, payload: np.ndarray, locations: np.ndarray | None = None) -> dict:
        rec = np.ascontiguousarray(records, dtype=GRAFTING_DTYPE)
        pay = np.ascontiguousarray(payload, dtype=BLOCK_DTYPE)
        loc = None if locations is None else np.ascontiguousarray(locations, dtype=np.uint64)
        rep = GraftReportC()
        _check("Graft", self._lib.svo_graft(self._ctx, C.byref(self._update(tick)), _ptr(rec), len(rec), _ptr(pay),
                                            len(pay), _ptr(loc), 0 if loc is None else loc.size, C.byref(rep)))
        return {"applied": rep.applied, "skipped": rep.skipped, "claimed": rep.claimed, "free_left": rep.free_left}

    def graft_generate(self, tick: int, scene: "Scene") -> dict:
        """Answers the last trace's child requests on the device from a terrain
        scene: what scene.graft_payload + graft do, without the host round trip."""
        rep = GraftReportC()
        _check("GraftGenerate", self._lib.svo_graft_generate(self._ctx, scene._h, C.byref(self._update(tick)),
                                                             C.byref(rep)))
        return {"applied": rep.applied, "skipped": rep.skipped, "claimed": rep.claimed, "free_left": rep.free_left}

    def graft_claims(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1), np.uint32)
        _check("GraftClaims", self._lib.svo_read_graft_claims(self._ctx, _ptr(out), n))
        return out[:n]

    def prune(self, tick: int, records: np.ndarray, surface: np.ndarray | None = None,
              locations: np.ndarray | None = None) -> dict:
        rec = np.ascontiguousarray(records, dtype=PRUNING_DTYPE)
        sur = None if surface is None else np.ascontiguousarray(surface, dtype=BLOCK_DTYPE)
        loc = None if locations is None else np.ascontiguousarray(locations, dtype=np.uint64)
        rep = PruneReportC()
        _check("Prune", self._lib.svo_prune(self._ctx, C.byref(self._update(tick)), _ptr(rec), len(rec), _ptr(sur),
                                            0 if sur is None else len(sur), _ptr(loc), 0 if loc is None else loc.size,
                                            C.byref(rep)))
        return {"freed": rep.freed, "requests": rep.requests}

    def read_bases(self) -> np.ndarray:
        n = self.tree_size()[1]
        out = np.zeros(n, np.uint16)
        _check("ReadBuffer:Bases", self._lib.svo_read_bases(self._ctx, _ptr(out), n))
        return out

    def read_child_requests(self, cap: int = 1 << 20):
        out = np.zeros(cap, dtype=CHILD_REQUEST_DTYPE)
        n = C.c_uint32()
        _check("ReadBuffer:ChildRequests", self._lib.svo_read_child_requests(self._ctx, _ptr(out), cap, C.byref(n)))
        return out[: min(n.value, cap, self._req_cap)], n.value
