"""Differentiable colour fitting through the C ABI against the FP64 oracle:
forward colour, loss, the per-node RGBA gradient against the FP64 analytic
gradient and FP64 central finite differences (h = 1e-4, 256 random hit nodes),
and a descent step that lowers the loss."""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(tracer):
    tracer.set_config(block_size=192, ctas_per_sm=0, ray_chunk=1, cadence=16, max_steps=1 << 16, collect_stats=0,
                      max_hits=16)
    yield
    tracer.set_config(max_hits=16)


@pytest.fixture(scope="module")
def fitting():
    """The colour-fitting workload at test size: the depth-9 SDF sphere, 4 views of
    128x96 around it, FP32 parameters uniform in [0, 1], targets rendered in FP64
    from the sinusoid ground-truth field (opacity 0.9)."""
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(4, 9)
    views = st.orbit_views(seed=7, n=4, width=128, height=96)
    hl = po.HitLists(tree, views, max_hits=16)
    rng = np.random.default_rng(3)
    params = rng.uniform(0.0, 1.0, size=(len(tree.Blocks), 4)).astype(np.float32)
    _, target, _ = hl.eval(st.sinusoid_field(tree).astype(np.float64), want_rgb=True)
    return tree, views, hl, params, target.astype(np.float32)


def test_forward_matches_fp64(tracer, fitting):
    tree, views, hl, params, _ = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    rgb = tracer.diff_forward(views)
    _, want, _ = hl.eval(params.astype(np.float64), want_rgb=True)
    err = np.abs(rgb - want)
    assert err.max() <= 1e-5, "max |C - C64| = %g" % err.max()
    assert (hl.n_hits > 1).sum() > 1000  # the rays composite several hits


def test_alpha_one_forward_is_the_trace_image(tracer, fitting):
    """With alpha = 1 compositing stops at the first hit, so the forward colour is
    the trace's shaded RGBA (node colour, sky where the ray misses)."""
    tree, views, _, _, _ = fitting
    tracer.upload(tree)
    p = np.zeros((len(tree.Blocks), 4), np.float32)
    p[:, 0] = tree.Blocks["colour_r"] / np.float32(255)
    p[:, 1] = tree.Blocks["colour_g"] / np.float32(255)
    p[:, 2] = tree.Blocks["colour_b"] / np.float32(255)
    p[:, 3] = 1.0
    tracer.diff_set_params(p)
    rgb = tracer.diff_forward(views)
    off = 0
    for v in views:
        n = v.ScreenSize[0] * v.ScreenSize[1]
        img = tracer.trace(v).rgba.reshape(n, 4)[:, :3]
        err = np.abs(rgb[off:off + n] - img).max()
        assert err <= 1e-6, "max |C - trace rgba| = %g" % err
        off += n


def test_backward_matches_fp64_gradient(tracer, fitting):
    tree, views, hl, params, target = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    loss = tracer.diff_backward(views, target)
    grad = tracer.diff_grads(len(tree.Blocks))
    want_loss, _, want = hl.eval(params.astype(np.float64), target.astype(np.float64), want_grad=True)
    assert abs(loss - want_loss) <= 1e-9 * want_loss, (loss, want_loss)
    scale = np.abs(want).max()
    err = np.abs(grad - want)
    ok = err <= 1e-4 * np.abs(want) + 1e-6 * scale
    assert ok.all(), "%d of %d entries off, max err %g (scale %g)" % ((~ok).sum(), ok.size, err.max(), scale)
    assert not grad[np.abs(want).sum(1) == 0].any()


def test_base_chunks_in_global_memory(tracer):
    """Base depth 6: the 299,592 base chunks (585 KB) do not fit shared memory and
    the colour-fitting kernels read them from global memory; forward colour,
    loss and gradient hold the FP64 bounds of the shared-memory case."""
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(6, 9)
    views = st.orbit_views(seed=7, n=2, width=96, height=64, distance=0.75)
    hl = po.HitLists(tree, views, max_hits=16)
    params = np.random.default_rng(3).uniform(0.0, 1.0, (len(tree.Blocks), 4)).astype(np.float32)
    _, target64, _ = hl.eval(st.sinusoid_field(tree).astype(np.float64), want_rgb=True)
    target = target64.astype(np.float32)
    tracer.upload(tree)
    tracer.diff_set_params(params)
    rgb = tracer.diff_forward(views)
    want_loss, want_rgb, want = hl.eval(params.astype(np.float64), target.astype(np.float64), want_rgb=True,
                                        want_grad=True)
    err = np.abs(rgb - want_rgb)
    assert err.max() <= 1e-5, "max |C - C64| = %g" % err.max()
    assert (hl.n_hits > 1).sum() > 1000
    loss = tracer.diff_backward(views, target)
    assert abs(loss - want_loss) <= 1e-9 * want_loss, (loss, want_loss)
    grad = tracer.diff_grads(len(tree.Blocks))
    scale = np.abs(want).max()
    ok = np.abs(grad - want) <= 1e-4 * np.abs(want) + 1e-6 * scale
    assert ok.all(), "%d of %d gradient entries off the FP64 gradient" % ((~ok).sum(), ok.size)


def check_cameras(tracer, cases, seed):
    rng = np.random.default_rng(seed)
    for name, tree, cam in cases:
        hl = po.HitLists(tree, [cam], max_hits=16)
        params = rng.uniform(0.0, 1.0, (len(tree.Blocks), 4)).astype(np.float32)
        target = rng.uniform(0.0, 1.0, (cam.ScreenSize[0] * cam.ScreenSize[1], 3)).astype(np.float32)
        tracer.upload(tree)
        tracer.diff_set_params(params)
        rgb = tracer.diff_forward([cam])
        want_loss, want_rgb, want = hl.eval(params.astype(np.float64), target.astype(np.float64), want_rgb=True,
                                            want_grad=True)
        err = np.abs(rgb - want_rgb)
        assert err.max() <= 1e-5, "%s: max |C - C64| = %g" % (name, err.max())
        loss = tracer.diff_backward([cam], target)
        # the loss is (1/P) sum over pixels and channels of e^2, e = C - target:
        # a colour error of at most d per channel moves it by at most
        # 2 sqrt(3 L) d + 3 d^2 (Cauchy-Schwarz), d the forward's bound above
        d = float(err.max())
        bound = 2.0 * np.sqrt(3.0 * want_loss) * d + 3.0 * d * d + 1e-12
        assert abs(loss - want_loss) <= bound, (name, loss, want_loss, bound)
        grad = tracer.diff_grads(len(tree.Blocks))
        scale = max(np.abs(want).max(), 1e-30)
        ok = np.abs(grad - want) <= 1e-4 * np.abs(want) + 1e-6 * scale
        assert ok.all(), "%s: %d gradient entries off the FP64 gradient" % (name, (~ok).sum())


def test_random_cameras(tracer):
    """30 seeded random cameras (origins in and around the cube, 1-96 pixels each
    way, fields of view 5-350 degrees, depth of field on a third): forward
    colour, loss and gradient within the FP64 bounds."""
    from test_oracle_vs_reference import random_cameras
    check_cameras(tracer, random_cameras(seed=55, n=30, cap=1 << 20), 13)


def test_edge_cameras(tracer):
    """Cameras along exact axes, on cell boundaries, on the cube's faces, edges and
    corner, and with fields of view past 180 degrees: forward colour, loss and
    gradient within the FP64 bounds of the other cases."""
    from test_oracle_vs_reference import axis_aligned_cases, extreme_camera_cases
    check_cameras(tracer, axis_aligned_cases() + extreme_camera_cases(), 12)


def test_backward_matches_fp64_finite_differences(tracer, fitting):
    """The acceptance check of the adjoint: within 1e-3 relative of FP64 central
    differences (h = 1e-4) on 256 random nodes that rays hit. Entries below
    1e-5 of the largest are held to 1e-3 of that absolute floor instead, where
    the FP32 gradient sums cancel."""
    tree, views, hl, params, target = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    tracer.diff_backward(views, target)
    grad = tracer.diff_grads(len(tree.Blocks))
    touched = np.unique(hl.hits[np.arange(hl.max_hits)[None] < hl.n_hits[:, None]])
    nodes = np.random.default_rng(11).choice(touched, 256, replace=False)
    fd = hl.finite_differences(params.astype(np.float64), target.astype(np.float64), nodes, h=1e-4)
    g = grad[nodes].astype(np.float64)
    floor = 1e-5 * np.abs(fd).max()
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), floor)
    assert rel.max() <= 1e-3, "max relative error %g" % rel.max()
    assert (np.abs(fd) > floor).mean() > 0.6  # most entries are held to the relative bound


def test_backward_with_saved_forward_colour(tracer, fitting):
    """The backward fed with the forward's saved colour (one traversal) gives the
    recomputing backward's loss and gradients; a saved colour of other views or
    other parameters is refused."""
    tree, views, hl, params, target = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    loss_r = tracer.diff_backward(views, target)
    grad_r = tracer.diff_grads(len(tree.Blocks))
    with pytest.raises(st.SvoError):
        tracer.diff_backward(views, target, use_saved=True)  # no forward yet for these parameters
    tracer.diff_forward(views)
    loss_s = tracer.diff_backward(views, target, use_saved=True)
    grad_s = tracer.diff_grads(len(tree.Blocks))
    assert abs(loss_s - loss_r) <= 1e-12 * loss_r
    scale = np.abs(grad_r).max()
    assert np.abs(grad_s - grad_r).max() <= 1e-6 * scale  # the same sums in another atomic order
    with pytest.raises(st.SvoError):
        tracer.diff_backward(views[:2], target[:2 * 128 * 96], use_saved=True)
    tracer.diff_set_params(params)
    with pytest.raises(st.SvoError):
        tracer.diff_backward(views, target, use_saved=True)


def test_descent_lowers_loss(tracer, fitting):
    tree, views, _, params, target = fitting
    tracer.upload(tree)
    p = params.copy()
    losses = []
    for _ in range(6):
        tracer.diff_set_params(p)
        losses.append(tracer.diff_backward(views, target))
        g = tracer.diff_grads(len(tree.Blocks))
        hit = np.abs(g).sum(1) > 0
        # per-node normalised step (each node's gradient scales with the pixels it covers)
        step = g / np.maximum(np.abs(g).max(1, keepdims=True), 1e-30)
        p[hit] = np.clip(p[hit] - 0.02 * step[hit], 0.0, 1.0)
    assert all(b < a for a, b in zip(losses, losses[1:])), losses
    assert losses[-1] < 0.9 * losses[0]


def test_multi_view_batch_equals_single_views(tracer, fitting):
    tree, views, _, params, target = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    both = tracer.diff_forward(views[:2])
    n0 = views[0].ScreenSize[0] * views[0].ScreenSize[1]
    assert np.array_equal(both[:n0], tracer.diff_forward(views[:1]))
    assert np.array_equal(both[n0:], tracer.diff_forward(views[1:2]))


def test_max_hits_limits_compositing(tracer, fitting):
    tree, views, _, params, _ = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    tracer.set_config(max_hits=2)
    rgb = tracer.diff_forward(views[:1])
    hl2 = po.HitLists(tree, views[:1], max_hits=2)
    _, want, _ = hl2.eval(params.astype(np.float64), want_rgb=True)
    assert np.abs(rgb - want).max() <= 1e-5
    with pytest.raises(st.SvoError):
        tracer.set_config(max_hits=2000)  # 1..1024; 0 keeps the current value


def test_diff_without_params_fails(tracer):
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=2).BuildTree(2, 5)
    tracer.upload(tree)
    with pytest.raises(st.SvoError):
        tracer.diff_forward(st.orbit_views(n=1, width=8, height=8))


def test_pinned_host_buffers_equal_pageable(tracer, fitting):
    """A pinned host colour buffer is written by the forward kernel and a pinned
    host target read by the backward kernel directly; the results are those of
    pageable buffers, which go through device copies."""
    torch = pytest.importorskip("torch")
    tree, views, _, params, target = fitting
    tracer.upload(tree)
    tracer.diff_set_params(params)
    n = sum(v.ScreenSize[0] * v.ScreenSize[1] for v in views)
    rgb_pinned = torch.empty(3 * n, dtype=torch.float32, pin_memory=True).numpy()
    tgt_pinned = torch.empty(3 * n, dtype=torch.float32, pin_memory=True).numpy()
    tgt_pinned[:] = target.reshape(-1)
    for _ in range(2):
        want_rgb = tracer.diff_forward(views)
        got_rgb = tracer.diff_forward(views, out=rgb_pinned)
        assert np.array_equal(got_rgb.reshape(-1, 3), want_rgb)
        want_loss = tracer.diff_backward(views, target)
        want_grad = tracer.diff_grads(len(tree.Blocks))
        got_loss = tracer.diff_backward(views, tgt_pinned)
        got_grad = tracer.diff_grads(len(tree.Blocks))
        assert abs(got_loss - want_loss) <= 1e-12 * want_loss
        assert np.abs(got_grad - want_grad).max() <= 1e-6 * np.abs(want_grad).max()  # atomic order only


def test_full_size_colour_fitting_matches_fp64(tracer):
    """The benchmarked colour-fitting workload at its stated size: the depth-9 SDF
    sphere, 16 views of 512x512 at world distance 1.5, FP32 parameters uniform in
    [0, 1], targets from the sinusoid ground truth (opacity 0.9). Every ray's
    forward colour is within 1e-5 of the FP64 oracle; the fwd+bwd step (backward
    fed with the forward's saved colour, as the bench runs it) gives the FP64 loss
    and, on 256 random hit nodes, gradients within 1e-3 relative of FP64 central
    differences (h = 1e-4), with the same absolute floor as the test-size check."""
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(4, 9)
    views = st.orbit_views(seed=7, n=16, width=512, height=512, distance=0.75)
    hl = po.HitLists(tree, views, max_hits=16)
    assert hl.n_rays == 16 * 512 * 512
    params = np.random.default_rng(3).uniform(0.0, 1.0, (len(tree.Blocks), 4)).astype(np.float32)
    _, target64, _ = hl.eval(st.sinusoid_field(tree, seed=9).astype(np.float64), want_rgb=True)
    target = target64.astype(np.float32)
    tracer.upload(tree)
    tracer.diff_set_params(params)
    rgb = tracer.diff_forward(views)
    want_loss, want_rgb, want_grad = hl.eval(params.astype(np.float64), target.astype(np.float64), want_rgb=True,
                                             want_grad=True)
    err = np.abs(rgb - want_rgb)
    assert err.max() <= 1e-5, "max |C - C64| = %g" % err.max()
    loss = tracer.diff_backward(views, target, use_saved=True)
    assert abs(loss - want_loss) <= 1e-9 * want_loss, (loss, want_loss)
    grad = tracer.diff_grads(len(tree.Blocks))
    scale = np.abs(want_grad).max()
    ok = np.abs(grad - want_grad) <= 1e-4 * np.abs(want_grad) + 1e-6 * scale
    assert ok.all(), "%d of %d gradient entries off the FP64 gradient" % ((~ok).sum(), ok.size)
    touched = np.unique(hl.hits[np.arange(hl.max_hits)[None] < hl.n_hits[:, None]])
    nodes = np.random.default_rng(11).choice(touched, 256, replace=False)
    fd = hl.finite_differences(params.astype(np.float64), target.astype(np.float64), nodes, h=1e-4)
    g = grad[nodes].astype(np.float64)
    floor = 1e-5 * np.abs(fd).max()
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), floor)
    assert rel.max() <= 1e-3, "max relative error %g" % rel.max()
    assert (np.abs(fd) > floor).mean() > 0.6
