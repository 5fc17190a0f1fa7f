"""The FP64 oracle of the differentiable colour-fitting model, on the CPU.

The hit lists are pinned to the trace oracle (itself pinned to the reference's
kernels): a ray's first LOD hit is the trace's hit node, and every hit node's
depth from the tree walk is the trace's hit depth. The analytic FP64 gradient is
checked against FP64 central finite differences."""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

NONE = 0xFFFFFFFF


@pytest.fixture(scope="module")
def sphere():
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(3, 8)
    views = st.orbit_views(seed=5, n=3, width=80, height=60)
    return tree, views, po.HitLists(tree, views, max_hits=16)


def test_node_cells_cover_tree(sphere):
    tree, _, _ = sphere
    cells, depth = st.node_cells(tree)
    live = depth > 0
    assert live.sum() == len(tree.Blocks)  # this builder leaves no unused slot at B=3, depth 8
    assert depth.max() == 8 and depth[live].min() == 5
    assert (cells[live] < (1 << depth[live].astype(np.int64))[:, None]).all()


def test_first_hit_is_trace_hit(sphere):
    tree, views, hl = sphere
    _, depth = st.node_cells(tree)
    off = 0
    for v in views:
        n = v.ScreenSize[0] * v.ScreenSize[1]
        out = po.trace_view(tree, v)
        hit_index = out["hit_index"].reshape(-1)
        hit_depth = out["hit_depth"].reshape(-1)
        hit = hit_index != NONE
        nh = hl.n_hits[off:off + n]
        first = hl.hits[off:off + n, 0]
        assert hit.any()
        assert (nh[hit] > 0).all() and (nh[~hit] == 0).all()
        assert np.array_equal(first[hit], hit_index[hit])
        assert np.array_equal(depth[first[hit]], hit_depth[hit])
        # a ray without hits ends in the sky, one with max_hits hits does not
        assert (hl.leaves[off:off + n][~hit] == 1).all()
        assert (hl.leaves[off:off + n][nh == hl.max_hits] == 0).all()
        off += n
    assert off == hl.n_rays


def test_hits_past_the_first_follow_the_ray(sphere):
    """Rays that cross the sphere hit nodes on both sides: later hits are
    further from the eye (the ray continues past each hit)."""
    tree, views, hl = sphere
    cells, depth = st.node_cells(tree)
    centre = (cells + 0.5) / np.exp2(depth.astype(np.float64))[:, None]
    n0 = views[0].ScreenSize[0] * views[0].ScreenSize[1]
    eye = np.asarray(views[0].Origin)
    rows = np.nonzero(hl.n_hits[:n0] >= 4)[0]
    assert len(rows) > 0
    for r in rows[:200]:
        d = np.linalg.norm(centre[hl.hits[r, :hl.n_hits[r]]] - eye, axis=1)
        assert d[-1] > d[0]


def test_fp64_gradient_matches_finite_differences(sphere):
    tree, _, hl = sphere
    rng = np.random.default_rng(0)
    params = rng.uniform(0.0, 1.0, size=(len(tree.Blocks), 4))
    params[:, 3] = rng.uniform(0.05, 0.95, len(tree.Blocks))
    _, target, _ = hl.eval(st.sinusoid_field(tree).astype(np.float64), want_rgb=True)
    loss, rgb, grad = hl.eval(params, target, want_rgb=True, want_grad=True)
    assert loss > 0
    touched = np.unique(hl.hits[np.arange(hl.max_hits)[None] < hl.n_hits[:, None]])
    nodes = rng.choice(touched, 256, replace=False)
    fd = hl.finite_differences(params, target, nodes, h=1e-4)
    g = grad[nodes]
    scale = np.abs(fd).max()
    # The loss is quadratic in each colour and in the alpha of a node hit once
    # per ray (central differences are then exact up to rounding); a node that
    # one ray hits k times through different octants enters its transmittance
    # as (1 - a)^k, which leaves an O(h^2) truncation term of ~1e-6 relative.
    ok = np.abs(fd - g) <= 1e-5 * np.abs(fd) + 1e-9 * scale
    assert ok.all(), "%d of %d gradient entries off" % ((~ok).sum(), ok.size)
    # nodes no ray hits have zero gradient
    cold = np.setdiff1d(np.arange(len(tree.Blocks)), touched)
    assert not grad[cold].any()


def test_loss_of_ground_truth_is_zero(sphere):
    tree, _, hl = sphere
    gt = st.sinusoid_field(tree).astype(np.float64)
    _, target, _ = hl.eval(gt, want_rgb=True)
    loss, _, grad = hl.eval(gt, target, want_grad=True)
    assert loss == 0.0 and not grad.any()
