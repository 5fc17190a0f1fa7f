"""The child-request queue past its cap (requestChild, wavefront.cl:362-375).

The reference appends requests in the order its work-items' atomics arrive, so once
a frame raises more requests than MaxChildRequestId the stored set depends on
timing. With svo_trace_config.request_order = SVO_REQUESTS_PIXEL the queue holds
the requests of the lowest pixel indices in pixel order (views in call order): the
oracle restates that rule on its own per-pixel requests, and the queue must equal
it record for record, under every schedule, in batches and graph replays, on every
run."""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu


@pytest.fixture()
def terrain(tracer):
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=10)
    tree = scene.build_tree(7)  # three levels short of the scene: most rays ask for children
    tracer.upload(tree)
    tracer.init_usage()
    yield tree
    tracer.set_config(request_order=st.REQUESTS_ARRIVAL, schedule=st.SCHEDULE_WARP, block_size=192, ctas_per_sm=0,
                      collect_stats=0)
    scene.close()


def _queue(tracer, cap):
    req, n = tracer.read_child_requests(cap=cap)
    return req.copy(), n


@pytest.mark.parametrize("schedule", [st.SCHEDULE_WARP, st.SCHEDULE_LANE, st.SCHEDULE_WAVEFRONT],
                         ids=["warp", "lane", "wavefront"])
def test_queue_past_the_cap_is_the_lowest_pixels_in_order(tracer, terrain, schedule):
    cap = 700
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 160, 90, 60.0, Tick=3, MaxChildRequestId=cap)
    want = po.trace_view(terrain, cam)
    assert want["n_requests"] > 4 * cap  # the queue overflows
    tracer.set_config(request_order=st.REQUESTS_PIXEL, schedule=schedule)
    for run in range(2):
        got = tracer.trace(cam)
        assert np.array_equal(got.hit_index, want["hit_index"])
        req, n = _queue(tracer, cap)
        assert n == want["n_requests"], "run %d: requests raised" % run
        assert len(req) == cap
        assert req.tobytes() == want["pixel_requests"][:cap].tobytes(), "run %d: queue differs" % run


def test_below_the_cap_both_orders_hold_the_same_requests(tracer, terrain):
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 96, 54, 60.0, Tick=3, MaxChildRequestId=1 << 16)
    want = po.trace_view(terrain, cam)
    assert 0 < want["n_requests"] < 1 << 16
    tracer.set_config(request_order=st.REQUESTS_ARRIVAL)
    tracer.trace(cam)
    arrival, n_a = _queue(tracer, 1 << 16)
    tracer.set_config(request_order=st.REQUESTS_PIXEL)
    tracer.trace(cam)
    pixel, n_p = _queue(tracer, 1 << 16)
    assert n_a == n_p == want["n_requests"]
    assert pixel.tobytes() == want["pixel_requests"].tobytes()
    assert po.sort_requests(arrival).tobytes() == po.sort_requests(pixel).tobytes()


@pytest.mark.parametrize("graph", [False, True], ids=["batch", "graph"])
def test_batch_queue_runs_over_the_views_in_call_order(tracer, terrain, graph):
    cap = 1500
    views = [st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 64, 36, 60.0, Tick=3, MaxChildRequestId=cap),
             st.look_at((0.8, 0.2, 0.5), (0.3, 0.6, 0.9), 50, 50, 70.0, Tick=3, MaxChildRequestId=cap),
             st.look_at((0.5, 0.9, 0.6), (0.5, 0.2, 0.85), 96, 54, 50.0, Tick=3, MaxChildRequestId=cap)]
    per_view = [po.trace_view(terrain, v) for v in views]
    total = sum(p["n_requests"] for p in per_view)
    assert total > cap > per_view[0]["n_requests"]  # the first view fits, the cap falls in a later one
    want = po.pixel_order_queue([p["pixel_requests"] for p in per_view], cap)
    tracer.set_config(request_order=st.REQUESTS_PIXEL)
    for run in range(2):
        res = tracer.trace_batch(views, graph=graph)
        for r, p in zip(res, per_view):
            assert np.array_equal(r.hit_index, p["hit_index"])
        req, n = _queue(tracer, cap)
        assert n == total
        assert req.tobytes() == want.tobytes(), "run %d: queue differs" % run


def test_request_order_is_validated(tracer):
    with pytest.raises(st.SvoError):
        tracer.set_config(request_order=3)
