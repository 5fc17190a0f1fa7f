"""The wavefront's secondary-cone stage as the reference wires it
(svo_trace_config.gi_stage = 1) against the oracle, which is pinned to the
reference's own wavefront.cl run with that stage enabled (test_gi_oracle.py):
every pixel's RGBA, hit outputs, usage ticks and child requests bit for bit,
under both schedules, in a graph-replayed batch, with and without a hit-index
output, and for the cone parameters that change the stage's branches."""
import dataclasses

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu


def with_random_normals(tree, seed):
    rng = np.random.default_rng(seed)
    blocks = tree.Blocks.copy()
    blocks["normal_pitch"] = rng.integers(-32768, 32768, len(blocks), dtype=np.int16)
    blocks["normal_yaw"] = rng.integers(-32768, 32768, len(blocks), dtype=np.int16)
    return dataclasses.replace(tree, Blocks=blocks)


@pytest.fixture(scope="module")
def trees():
    return {"sphere": st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(3, 8),
            "terrain_random_normals": with_random_normals(st.TreeBuilder(st.SCENE_TERRAIN, seed=2).BuildTree(3, 8), 7)}


@pytest.fixture(autouse=True)
def gi_on(tracer):
    tracer.set_config(gi_stage=1, schedule=st.SCHEDULE_WARP, block_size=192, ctas_per_sm=0, collect_stats=0)
    yield
    tracer.set_config(gi_stage=-1, schedule=st.SCHEDULE_WARP)


def compare(tracer, tree, view):
    tracer.upload(tree)
    tracer.init_usage()
    got = tracer.trace(view)
    usage = po.init_usage(tree)
    want = po.trace_view(tree, view, usage=usage, gi=True)
    for k in ("hit_index", "hit_depth", "t"):
        assert np.array_equal(getattr(got, k), want[k]), k
    assert np.array_equal(got.rgba.view(np.uint32), want["rgba"].view(np.uint32)), "rgba"
    assert np.array_equal(tracer.read_usage(len(usage))["tick"], usage["tick"]), "usage ticks"
    req, n = tracer.read_child_requests()
    assert n == want["n_requests"]
    assert po.sort_requests(req).tobytes() == po.sort_requests(want["requests"]).tobytes()
    return got, want


@pytest.mark.parametrize("schedule", [st.SCHEDULE_WARP, st.SCHEDULE_LANE, st.SCHEDULE_WAVEFRONT],
                         ids=["warp", "lane", "wavefront"])
@pytest.mark.parametrize("scene", ["sphere", "terrain_random_normals"])
def test_gi_stage_matches_oracle(tracer, trees, scene, schedule):
    tracer.set_config(schedule=schedule)
    view = st.look_at((1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 123, 77, 60.0, Tick=5) if scene == "sphere" else \
        st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 160, 90, 60.0, Tick=9)
    got, _ = compare(tracer, trees[scene], view)
    assert (got.hit_index != st.MISS).any()


@pytest.mark.parametrize("schedule", [st.SCHEDULE_WARP, st.SCHEDULE_LANE, st.SCHEDULE_WAVEFRONT],
                         ids=["warp", "lane", "wavefront"])
def test_gi_edge_cameras(tracer, schedule):
    """Cameras along exact axes, on cell boundaries, on the cube's faces, edges and
    corner, and with fields of view past 180 degrees (the CPU tests pin the oracle
    to the reference on the same cameras)."""
    from test_gi_oracle import edge_camera_cases
    tracer.set_config(schedule=schedule)
    for name, tree, cam in edge_camera_cases():
        compare(tracer, tree, cam)


@pytest.mark.parametrize("schedule", [st.SCHEDULE_WARP, st.SCHEDULE_LANE, st.SCHEDULE_WAVEFRONT],
                         ids=["warp", "lane", "wavefront"])
def test_gi_random_cameras(tracer, schedule):
    """30 seeded random cameras (the CPU tests pin the oracle to the reference on
    them)."""
    from test_gi_oracle import random_cases
    tracer.set_config(schedule=schedule)
    for name, tree, cam in random_cases():
        compare(tracer, tree, cam)


@pytest.mark.parametrize("kw", [
    {"FovMultiplier": 0.1, "FovConstant": 0.08, "WeightingMultiplier": -0.2, "WeightingConstant": 1.5},
    {"AmbientLightLevel": 0},
    {"AmbientLightLevel": 255},
    {"WeightingConstant": 0.01},
    {"FovConstant": 0.0},
    {"WeightingMultiplier": -0.5, "WeightingConstant": 0.3},
], ids=["other_schedule", "ambient0", "ambient255", "low_weighting", "no_stage", "negative_weighting"])
def test_gi_cone_parameters(tracer, trees, kw):
    tree = with_random_normals(trees["sphere"], 3)
    compare(tracer, tree, st.look_at((1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 48, 36, 60.0, Tick=5, **kw))


def test_gi_batch_graph_and_device_outputs_without_hit_index(tracer, trees):
    """A graph-replayed batch of views sharing their cone parameters: rgba-only
    device outputs (the stage reads the hits from a library buffer) equal the
    oracle; views with different cone parameters are refused."""
    torch = pytest.importorskip("torch")
    tree = trees["terrain_random_normals"]
    tracer.upload(tree)
    views = [st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 64, 36, 60.0, Tick=3),
             st.look_at((0.8, 0.2, 0.5), (0.3, 0.6, 0.9), 50, 50, 70.0, Tick=3),
             st.look_at((0.5, 0.9, 0.6), (0.5, 0.2, 0.85), 96, 54, 50.0, Tick=3)]
    rgba = [torch.empty(4 * v.ScreenSize[0] * v.ScreenSize[1], dtype=torch.float32, device="cuda") for v in views]
    for _ in range(2):
        tracer.trace_device(views, [(0, 0, 0, x.data_ptr()) for x in rgba], graph=True)
        torch.cuda.synchronize()
        for v, x in zip(views, rgba):
            want = po.trace_view(tree, v, gi=True)
            assert np.array_equal(x.cpu().numpy().reshape(-1, 4).view(np.uint32), want["rgba"].view(np.uint32))
    odd = views[:2] + [dataclasses.replace(views[2], FovConstant=0.1)]
    with pytest.raises(st.SvoError):
        tracer.trace_batch(odd)


def test_gi_endless_schedule_is_refused(tracer, trees):
    tracer.upload(trees["sphere"])
    with pytest.raises(st.SvoError):
        tracer.trace(st.look_at((1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 16, 12, 60.0, FovMultiplier=-0.9,
                                FovConstant=0.01))


def test_gi_stage_is_validated(tracer):
    with pytest.raises(st.SvoError):
        tracer.set_config(gi_stage=2)
