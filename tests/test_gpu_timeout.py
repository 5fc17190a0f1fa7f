"""The bounded-loop paths of the device kernels (the failure detection of this
library). The reference's own loops have no bound: its host loop re-enqueues
passes until the queues drain (MainWindow.cs:452-481) and its tree kernels spin
on a global flag (wavefront.cl:226-231). Here every device loop has a pass bound;
past it a kernel records the stopped thread in an error record, returns, and
the call reports SVO_ERR_TIMEOUT. The tests lower the bound to one pass
(svo_trace_config.pass_limit), so the bound runs out on the first ray that
needs a second pass: nothing faults or hangs, the kernels only return. They then
check that each entry point reports it, and that the next call with the
default bound is bit-exact again."""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # SVO_ERR_TIMEOUT


@pytest.fixture()
def sphere(tracer):
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=3).BuildTree(3, 7)
    cam = st.orbit_views(seed=2, n=1, width=64, height=48, distance=0.75, Tick=4, MaxChildRequestId=4096)[0]
    tracer.upload(tree)
    tracer.init_usage()
    yield tree, cam
    tracer.set_config(pass_limit=0, schedule=st.SCHEDULE_WARP, block_size=192, ctas_per_sm=0, collect_stats=0)


def _stopped(call):
    with pytest.raises(st.SvoError) as e:
        call()
    assert e.value.code == TIMEOUT, str(e.value)
    assert "pass bound on ray" in e.value.detail, e.value.detail
    return e.value


def test_trace_reports_a_stopped_kernel_under_both_schedules(tracer, sphere):
    tree, cam = sphere
    for schedule in (st.SCHEDULE_WARP, st.SCHEDULE_LANE, st.SCHEDULE_WAVEFRONT):
        tracer.set_config(pass_limit=1, schedule=schedule)
        _stopped(lambda: tracer.trace(cam))  # host outputs: the call synchronises and reports
    tracer.set_config(pass_limit=0, schedule=st.SCHEDULE_WARP)
    tracer.synchronize()  # reported once, then cleared: nothing pending
    usage = po.init_usage(tree)
    tracer.init_usage()
    got = tracer.trace(cam)
    want = po.trace_view(tree, cam, usage=usage)
    for k in ("hit_index", "hit_depth", "t", "rgba"):
        assert np.array_equal(getattr(got, k), want[k]), k
    assert np.array_equal(tracer.read_usage(len(usage))["tick"], usage["tick"])


def test_device_output_trace_reports_at_synchronize(tracer, sphere):
    torch = pytest.importorskip("torch")
    tree, cam = sphere
    n = cam.ScreenSize[0] * cam.ScreenSize[1]
    dev = torch.device("cuda", 0)
    o = [torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
         torch.empty(n, dtype=torch.float32, device=dev), torch.empty(4 * n, dtype=torch.float32, device=dev)]
    outs = [tuple(x.data_ptr() for x in o)]
    tracer.set_config(pass_limit=1)
    tracer.trace_device([cam], outs)  # device outputs: no synchronisation, the error stays recorded
    err = _stopped(tracer.synchronize)
    assert err.method == "Synchronize"
    tracer.set_config(pass_limit=0)
    tracer.trace_device([cam], outs)
    tracer.synchronize()
    want = po.trace_view(tree, cam)
    assert np.array_equal(o[0].cpu().numpy().view(np.uint32), want["hit_index"])
    assert np.array_equal(o[3].cpu().numpy().reshape(-1, 4), want["rgba"])


def test_megakernel_reports_a_stopped_kernel(tracer, sphere):
    tree, cam = sphere  # the reference's default cone parameters: every pixel spawns a fan
    tracer.set_config(pass_limit=1)
    _stopped(lambda: tracer.mega_trace(cam))
    tracer.set_config(pass_limit=0)
    usage = po.init_usage(tree)
    tracer.init_usage()
    got = tracer.mega_trace(cam)
    want = po.mega_trace_view(tree, cam, usage=usage)
    assert np.array_equal(got.rgba, want["rgba"])
    assert np.array_equal(got.hit_index, want["hit_index"])


def test_colour_fitting_reports_a_stopped_kernel(tracer, sphere):
    tree, cam = sphere
    views = [cam]
    nodes = len(tree.Blocks)
    params = np.random.default_rng(5).uniform(0.0, 1.0, (nodes, 4)).astype(np.float32)
    tracer.diff_set_params(params)
    want_rgb = tracer.diff_forward(views).copy()
    target = np.random.default_rng(6).uniform(0.0, 1.0, want_rgb.shape).astype(np.float32)
    want_loss = tracer.diff_backward(views, target)
    want_grad = tracer.diff_grads(nodes).copy()
    tracer.set_config(pass_limit=1)
    _stopped(lambda: tracer.diff_forward(views))
    _stopped(lambda: tracer.diff_backward(views, target))
    tracer.set_config(pass_limit=0)
    assert np.array_equal(tracer.diff_forward(views), want_rgb)
    # the loss and the gradients are sums of atomics: equal up to the order of the additions
    assert tracer.diff_backward(views, target) == pytest.approx(want_loss, rel=1e-12)
    np.testing.assert_allclose(tracer.diff_grads(nodes), want_grad, rtol=1e-5, atol=1e-9)


def test_pass_limit_must_not_be_negative(tracer):
    with pytest.raises(st.SvoError):
        tracer.set_config(pass_limit=-1)
