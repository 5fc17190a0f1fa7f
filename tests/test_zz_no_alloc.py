"""svo_trace_noalloc: tracing for callers that cannot allocate device memory.

Such a caller (an engine that owns every GPU allocation through its own pool, a
real-time host loop that may not call cudaMalloc) keeps the octree and the output
buffers in memory it already owns and calls svo_trace_noalloc, whose only scratch is
a fixed static array inside libsvo. This test gives it buffers allocated here (the
test may allocate; the entry point does not) and checks two calls in a row against
the context-based svo_trace entry point on the same tree and view, and against the
oracle: hit indices, hit depths, usage ticks and child requests bit for bit, t and
RGBA within the tolerance the other GPU tests use (they are in fact bit-exact)."""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu

T_RTOL = 1e-5


def _entry(lib):
    return lib.svo_trace_noalloc  # bound by svo_tracer with the header's signature (checked in test_abi)


def test_noalloc_matches_trace_on_two_calls():
    torch = pytest.importorskip("torch")
    lib = st.load_library()
    trace_noalloc = _entry(lib)
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(4, 9)
    W, H, cap = 320, 180, 1 << 16
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), W, H, 60.0, Tick=9, MaxChildRequestId=cap)
    n_groups = len(tree.Blocks) // 8

    with st.Tracer(0) as tr:  # the existing entry point
        tr.upload(tree)
        tr.init_usage()
        usage0 = tr.read_usage(n_groups)
        want = tr.trace(cam)
        usage_want = tr.read_usage(n_groups)
        req_want, n_want = tr.read_child_requests()
    assert n_want > 0 and (want.hit_index != st.MISS).any()
    usage_oracle = usage0.copy()
    oracle = po.trace_view(tree, cam, usage=usage_oracle)

    dev = torch.device("cuda", 0)
    d_bases = torch.from_numpy(tree.BaseBlocks.view(np.int16).copy()).to(dev)
    d_blocks = torch.from_numpy(tree.Blocks.view(np.uint8).copy()).to(dev)
    c_in = cam.to_c()
    for call in range(2):
        d_usage = torch.from_numpy(usage0.view(np.uint8).copy()).to(dev)
        d_idx = torch.full((W * H,), -7, dtype=torch.int32, device=dev)
        d_dep = torch.full((W * H,), 99, dtype=torch.uint8, device=dev)
        d_t = torch.full((W * H,), -1.0, dtype=torch.float32, device=dev)
        d_rgba = torch.full((W * H * 4,), -1.0, dtype=torch.float32, device=dev)
        d_req = torch.zeros((cap * 40,), dtype=torch.uint8, device=dev)
        out = st.TraceOutputC(d_idx.data_ptr(), d_dep.data_ptr(), d_t.data_ptr(), d_rgba.data_ptr(), 1, 0)
        raised = C.c_uint32(0)
        torch.cuda.synchronize()
        status = trace_noalloc(0, None, tree.BaseDepth, d_bases.data_ptr(), len(tree.BaseBlocks), d_blocks.data_ptr(),
                               len(tree.Blocks), d_usage.data_ptr(), n_groups, 9, C.byref(c_in), C.byref(out),
                               d_req.data_ptr(), cap, C.byref(raised))
        assert status == 0, lib.svo_last_error_string()
        torch.cuda.synchronize()
        idx = d_idx.cpu().numpy().view(np.uint32)
        dep = d_dep.cpu().numpy()
        t = d_t.cpu().numpy()
        rgba = d_rgba.cpu().numpy().reshape(-1, 4)
        usage = d_usage.cpu().numpy().view(st.USAGE_DTYPE)
        req = d_req.cpu().numpy().view(st.CHILD_REQUEST_DTYPE)[: min(raised.value, cap)]
        # against the existing entry point, then against the oracle
        for label, ref_idx, ref_dep, ref_t, ref_rgba, ref_ticks, ref_n, ref_req in (
                ("svo_trace", want.hit_index, want.hit_depth, want.t, want.rgba, usage_want["tick"], n_want, req_want),
                ("oracle", oracle["hit_index"], oracle["hit_depth"], oracle["t"], oracle["rgba"],
                 usage_oracle["tick"], oracle["n_requests"], oracle["requests"])):
            assert np.array_equal(idx, ref_idx), "call %d vs %s: hit_index" % (call, label)
            assert np.array_equal(dep, ref_dep), "call %d vs %s: hit_depth" % (call, label)
            np.testing.assert_allclose(t, ref_t, rtol=T_RTOL, atol=0)
            np.testing.assert_allclose(rgba, ref_rgba, rtol=T_RTOL, atol=0)
            assert np.array_equal(usage["tick"], ref_ticks), "call %d vs %s: usage ticks" % (call, label)
            assert raised.value == ref_n, "call %d vs %s: requests raised" % (call, label)
            same = po.sort_requests(req).tobytes() == po.sort_requests(ref_req).tobytes()
            assert same, "call %d vs %s: child requests differ" % (call, label)


def test_noalloc_random_cameras():
    """30 seeded random cameras over two trees (origins in and around the cube,
    1-96 pixels each way, fields of view 5-350 degrees, depth of field on a third)
    through svo_trace_noalloc: every output, the usage ticks and the child
    requests equal the oracle's (the CPU tests pin the oracle to the reference on
    the same cameras)."""
    torch = pytest.importorskip("torch")
    from test_oracle_vs_reference import random_cameras
    lib = st.load_library()
    trace_noalloc = _entry(lib)
    dev = torch.device("cuda", 0)
    cap = 1 << 16
    resident = {}
    for name, tree, cam in random_cameras(seed=21, n=30, cap=cap):
        if id(tree) not in resident:
            resident[id(tree)] = (torch.from_numpy(tree.BaseBlocks.view(np.int16).copy()).to(dev),
                                  torch.from_numpy(tree.Blocks.view(np.uint8).copy()).to(dev))
        d_bases, d_blocks = resident[id(tree)]
        W, H = cam.ScreenSize
        n_groups = len(tree.Blocks) // 8
        usage0 = po.init_usage(tree)
        want_usage = usage0.copy()
        want = po.trace_view(tree, cam, usage=want_usage)
        d_usage = torch.from_numpy(usage0.view(np.uint8).copy()).to(dev)
        d_idx = torch.full((W * H,), -7, dtype=torch.int32, device=dev)
        d_dep = torch.full((W * H,), 99, dtype=torch.uint8, device=dev)
        d_t = torch.full((W * H,), -1.0, dtype=torch.float32, device=dev)
        d_rgba = torch.full((W * H * 4,), -1.0, dtype=torch.float32, device=dev)
        d_req = torch.zeros((cap * 40,), dtype=torch.uint8, device=dev)
        out = st.TraceOutputC(d_idx.data_ptr(), d_dep.data_ptr(), d_t.data_ptr(), d_rgba.data_ptr(), 1, 0)
        raised = C.c_uint32(0)
        c_in = cam.to_c()
        torch.cuda.synchronize()
        status = trace_noalloc(0, None, tree.BaseDepth, d_bases.data_ptr(), len(tree.BaseBlocks), d_blocks.data_ptr(),
                               len(tree.Blocks), d_usage.data_ptr(), n_groups, 0, C.byref(c_in), C.byref(out),
                               d_req.data_ptr(), cap, C.byref(raised))
        assert status == 0, (name, lib.svo_last_error_string())
        torch.cuda.synchronize()
        assert np.array_equal(d_idx.cpu().numpy().view(np.uint32), want["hit_index"]), name
        assert np.array_equal(d_dep.cpu().numpy(), want["hit_depth"]), name
        assert np.array_equal(d_t.cpu().numpy().view(np.uint32), want["t"].view(np.uint32)), name
        assert np.array_equal(d_rgba.cpu().numpy().reshape(-1, 4).view(np.uint32), want["rgba"].view(np.uint32)), name
        assert np.array_equal(d_usage.cpu().numpy().view(st.USAGE_DTYPE)["tick"], want_usage["tick"]), name
        assert raised.value == want["n_requests"], name
        req = d_req.cpu().numpy().view(st.CHILD_REQUEST_DTYPE)[: raised.value]
        assert po.sort_requests(req).tobytes() == po.sort_requests(want["requests"]).tobytes(), name


def test_noalloc_rejects_oversized_views_and_host_outputs():
    lib = st.load_library()
    trace_noalloc = _entry(lib)
    bases = np.zeros(st.pow_sum(2), np.uint16)
    blocks = np.zeros(8 ** 4, st.BLOCK_DTYPE)
    out = st.TraceOutputC(1, None, None, None, 1, 0)  # never dereferenced: the call must refuse first
    too_big = st.TraceInput(ScreenSize=(16000, 400)).to_c()
    status = trace_noalloc(0, None, 2, bases.ctypes.data, len(bases), blocks.ctypes.data, len(blocks), None, 0, 0,
                           C.byref(too_big), C.byref(out), None, 0, None)
    assert status == 1
    assert b"16384" in lib.svo_last_error_string()
    host_out = st.TraceOutputC(1, None, None, None, 0, 0)
    ok_size = st.TraceInput(ScreenSize=(64, 48)).to_c()
    status = trace_noalloc(0, None, 2, bases.ctypes.data, len(bases), blocks.ctypes.data, len(blocks), None, 0, 0,
                           C.byref(ok_size), C.byref(host_out), None, 0, None)
    assert status == 1
    assert b"device pointers" in lib.svo_last_error_string()
