"""The CUDA path against the reference's own kernels (wavefront.cl and the
megakernel kernel.cl, built for the CPU by oracle/build_ref.py) directly, on
the same inputs: bit-exact images, hit outputs, child requests and usage. The
oracle tests check the same through the restatement; these skip where the
rewritten reference sources are not present."""
import dataclasses

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tracer():
    t = st.Tracer(0)
    yield t
    t.close()


@pytest.fixture(scope="module")
def scenes():
    return {"sphere": st.TreeBuilder(st.SCENE_SPHERE, seed=4).BuildTree(3, 8),
            "terrain": st.TreeBuilder(st.SCENE_TERRAIN, seed=6).BuildTree(3, 8)}


def same_requests(a, b):
    a, b = po.sort_requests(a), po.sort_requests(b)
    assert len(a) == len(b)
    for f in ("address", "tick", "depth", "location", "tree_size"):
        assert np.array_equal(a[f], b[f]), f


VIEWS = [("sphere", dict(seed=2, distance=1.4)), ("terrain", dict(seed=8, distance=1.2)),
         ("terrain", dict(seed=9, distance=0.6))]


@pytest.mark.skipif(not po.ref_available(), reason="wavefront.cl reference build not available")
@pytest.mark.parametrize("scene,kw", VIEWS)
def test_wavefront_trace_equals_reference(tracer, scenes, scene, kw):
    tree = scenes[scene]
    v = dataclasses.replace(st.orbit_views(n=1, width=72, height=40, **kw)[0], Tick=5, MaxChildRequestId=1 << 20)
    tracer.upload(tree)
    tracer.init_usage()
    got = tracer.trace(v)
    req, n = tracer.read_child_requests()
    usage = tracer.read_usage(len(tree.Blocks) // 8)
    u_ref = po.init_usage(tree)
    ref = po.ref_trace_view(tree, v, usage=u_ref)
    for k in ("hit_index", "hit_depth"):
        assert np.array_equal(getattr(got, k).reshape(-1), ref[k]), k
    assert np.array_equal(got.t.reshape(-1).view(np.uint32), ref["t"].view(np.uint32))
    assert np.array_equal(got.rgba.reshape(-1, 4).view(np.uint32), ref["rgba"].view(np.uint32))
    assert n == ref["n_requests"]
    same_requests(req, ref["requests"])
    assert np.array_equal(usage["tick"], u_ref["tick"])


@pytest.mark.skipif(not po.ref_mega_available(), reason="kernel.cl reference build not available")
@pytest.mark.parametrize("scene,kw", VIEWS)
def test_megakernel_equals_reference(tracer, scenes, scene, kw):
    tree = scenes[scene]
    v = dataclasses.replace(st.orbit_views(n=1, width=72, height=40, **kw)[0], Tick=5, MaxChildRequestId=1 << 20)
    tracer.upload(tree)
    tracer.init_usage()
    got = tracer.mega_trace(v)
    req, n = tracer.read_child_requests()
    usage = tracer.read_usage(len(tree.Blocks) // 8)
    u_ref = po.init_usage(tree)
    ref = po.ref_mega_trace_view(tree, v, usage=u_ref)
    assert np.array_equal(got.rgba.reshape(-1, 4).view(np.uint32), ref["rgba"].view(np.uint32))
    assert n == ref["n_requests"]
    same_requests(req, ref["requests"])
    assert np.array_equal(usage["tick"], u_ref["tick"])
