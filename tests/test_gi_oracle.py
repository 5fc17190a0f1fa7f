"""The wavefront's secondary-cone stage (evaluateMaterial, saveAccumulator, the
second evaluateBackground), which MainWindow.RunWavefront has commented out, run
as written: the oracle's restatement against the reference's own wavefront.cl
compiled for the CPU and driven with that stage enabled. Bit-exact: the image,
the integer accumulators, the hit outputs, the usage ticks and the child
requests. Cones of weighting > 5 go straight to the background queue, so a hit
pixel's colour is its cones' sky light; the sphere's and terrain's own normals
and seeded random normals (every branch of the fan, edge-on hits) are both
covered, with the reference's default cone parameters and others."""
import dataclasses

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.skipif(not po.ref_available(), reason="reference kernels not available")


def with_random_normals(tree, seed):
    rng = np.random.default_rng(seed)
    blocks = tree.Blocks.copy()
    blocks["normal_pitch"] = rng.integers(-32768, 32768, len(blocks), dtype=np.int16)
    blocks["normal_yaw"] = rng.integers(-32768, 32768, len(blocks), dtype=np.int16)
    return dataclasses.replace(tree, Blocks=blocks)


@pytest.fixture(scope="module")
def sphere():
    return st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(3, 8)


@pytest.fixture(scope="module")
def terrain():
    return st.TreeBuilder(st.SCENE_TERRAIN, seed=2).BuildTree(3, 8)


def check(tree, view):
    ua, ub = po.init_usage(tree), po.init_usage(tree)
    ref = po.ref_trace_view(tree, view, usage=ua, gi=True)
    got = po.trace_view(tree, view, usage=ub, gi=True)
    for k in ("hit_index", "hit_depth", "t", "acc"):
        assert np.array_equal(ref[k], got[k]), k
    assert np.array_equal(ref["rgba"].view(np.uint32), got["rgba"].view(np.uint32))
    assert np.array_equal(ua, ub)
    assert ref["n_requests"] == got["n_requests"]
    assert po.sort_requests(ref["requests"]).tobytes() == po.sort_requests(got["requests"]).tobytes()
    return ref, got


VIEWS = [((1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 64, 48, 60.0), ((0.1, 1.3, 0.3), (0.5, 0.5, 0.5), 48, 40, 75.0)]


@pytest.mark.parametrize("k", range(len(VIEWS)))
def test_sphere_default_cones(sphere, k):
    o, t, w, h, fov = VIEWS[k]
    _, got = check(sphere, st.look_at(o, t, w, h, fov, Tick=5))
    hit = got["hit_index"] != st.MISS
    assert hit.any()
    plain = po.trace_view(sphere, st.look_at(o, t, w, h, fov, Tick=5))
    # the hits' colour changed (cone light only), the sky pixels kept theirs
    assert not np.array_equal(got["rgba"][hit], plain["rgba"][hit])
    assert np.array_equal(got["rgba"][~hit], plain["rgba"][~hit])


def test_terrain_random_normals(terrain):
    """Random normals: some hits are seen edge-on (one cone along the primary
    direction), fans break early, weightings vary."""
    tree = with_random_normals(terrain, 7)
    check(tree, st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 96, 54, 60.0, Tick=9))


@pytest.mark.parametrize("kw", [
    {"FovMultiplier": 0.1, "FovConstant": 0.08, "WeightingMultiplier": -0.2, "WeightingConstant": 1.5},
    {"AmbientLightLevel": 0},
    {"AmbientLightLevel": 255},
    {"WeightingConstant": 0.01},               # weighting * 255 < 6: the hit only sets FinalWeightings
    {"FovConstant": 0.0},                      # evaluateMaterial returns at once: hits stay unlit (red)
    {"WeightingMultiplier": -0.5, "WeightingConstant": 0.3},  # negative weightings saturate to 0
], ids=["other_schedule", "ambient0", "ambient255", "low_weighting", "no_stage", "negative_weighting"])
def test_cone_parameters(sphere, kw):
    tree = with_random_normals(sphere, 3)
    view = st.look_at((1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 48, 36, 60.0, Tick=5, **kw)
    ref, got = check(tree, view)
    hit = got["hit_index"] != st.MISS
    if kw.get("FovConstant") == 0.0:
        assert (got["rgba"][hit] == np.array([0.75, 0.0, 0.0, 1.0], np.float32)).all()
    if kw.get("WeightingConstant") == 0.01:
        assert (got["acc"][hit][:, 0] == 255).all() and (got["rgba"][hit][:, :3] == 0).all()


def test_endless_schedule_is_refused(sphere):
    view = st.look_at((1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 16, 12, 60.0, FovMultiplier=-0.9, FovConstant=0.01)
    with pytest.raises(ValueError):
        po.trace_view(sphere, view, gi=True)
    with pytest.raises(ValueError):
        po.ref_trace_view(sphere, view, gi=True)


def edge_camera_cases():
    """The trace's edge cameras (exact axes, origins on cell boundaries, the cube's
    faces, edges and corner, fields of view past 180 degrees), every second one
    with seeded normals."""
    from test_oracle_vs_reference import axis_aligned_cases, extreme_camera_cases
    out = []
    for i, (name, tree, cam) in enumerate(axis_aligned_cases() + extreme_camera_cases()):
        out.append((name, with_random_normals(tree, 20 + i) if i % 2 else tree, cam))
    return out


def test_edge_cameras(sphere):
    lit = 0
    for name, tree, cam in edge_camera_cases():
        _, got = check(tree, cam)
        lit += int((got["hit_index"] != st.MISS).sum())
    assert lit > 5000


def random_cases():
    """30 seeded random cameras (the trace's random-camera generator), every second
    tree with seeded normals."""
    from test_oracle_vs_reference import random_cameras
    return [(name, with_random_normals(tree, 60 + i) if i % 2 else tree, cam)
            for i, (name, tree, cam) in enumerate(random_cameras(seed=91, n=30, cap=1 << 20))]


def test_random_cameras():
    lit = 0
    for name, tree, cam in random_cases():
        _, got = check(tree, cam)
        lit += int((got["hit_index"] != st.MISS).sum())
    assert lit > 3000
