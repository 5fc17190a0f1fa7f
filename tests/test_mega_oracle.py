"""The megakernel oracle (kernel.cl's `trace`: primary cone, spawnRays's fan of
secondary cones, draw) against the reference's own kernel.cl compiled for the
CPU, on the CPU. Bit-exact: the image, every child request field and the usage
ticks."""
import dataclasses

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.skipif(not po.ref_mega_available(), reason="kernel.cl source not available")


def with_random_normals(tree, seed):
    """The same tree with seeded NormalPitch/NormalYaw on every node, so that the
    cone fans take every branch of spawnRays (the builders leave them zero)."""
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


def same_requests(a, b):
    ra, rb = po.sort_requests(a), po.sort_requests(b)
    assert len(ra) == len(rb)
    for f in ("address", "tick", "depth", "location", "tree_size"):
        assert np.array_equal(ra[f], rb[f]), f


def check(tree, view, rows=None):
    ua, ub = po.init_usage(tree), po.init_usage(tree)
    ref = po.ref_mega_trace_view(tree, view, usage=ua, rows=rows)
    got = po.mega_trace_view(tree, view, usage=ub, rows=rows)
    w = view.ScreenSize[0]
    band = slice(None) if rows is None else slice(rows[0] * w, rows[1] * w)
    assert np.array_equal(ref["rgba"][band].view(np.uint32), got["rgba"].view(np.uint32))
    assert ref["n_requests"] == got["n_requests"]
    same_requests(ref["requests"], got["requests"])
    assert np.array_equal(ua, ub)
    return ref, got


@pytest.mark.parametrize("k", range(3))
def test_orbit_views_sphere(sphere, k):
    v = st.orbit_views(seed=5, n=3, width=64, height=48)[k]
    ref, got = check(sphere, v)
    assert got["cones"].max() > 10  # hits spawn cone fans
    assert (got["hit_index"] != st.MISS).any() and (got["hit_index"] == st.MISS).any()


@pytest.mark.parametrize("k", range(3))
def test_orbit_views_terrain_random_normals(terrain, k):
    tree = with_random_normals(terrain, 10 + k)
    v = st.orbit_views(seed=7, n=3, width=64, height=48, distance=1.2)[k]
    ref, got = check(tree, v)
    assert ref["n_requests"] > 0
    # cone counts vary with the normal (the fan stops at the first cone below the surface)
    assert len(np.unique(got["cones"][got["hit_index"] != st.MISS])) >= 3


def test_inside_cube_with_dof(sphere):
    tree = with_random_normals(sphere, 3)
    v = st.look_at((0.5, 0.5, 0.12), (0.5, 0.55, 0.6), 48, 40, 70.0, DoF=(0.02, 0.3), Tick=9)
    check(tree, v)


def mega_axis_aligned_cases(sphere):
    """Cameras whose Facing columns are exact unit axes (direction components
    exactly zero in the centre row and column), the second with its origin on the
    cell boundaries of every level and seeded normals (child requests, every
    spawnRays branch)."""
    kw = dict(Tick=3, MaxChildRequestId=1 << 20)
    return [("down_z", sphere, st.look_at((0.5, 0.5, 1.6), (0.5, 0.5, 0.5), 64, 48, 60.0, **kw)),
            ("origin_on_boundaries", with_random_normals(sphere, 4),
             st.look_at((0.5, 0.25, 0.5), (0.5, 0.9, 0.5), 48, 32, 70.0, **kw))]


def mega_extreme_cases(sphere):
    """A field of view past 180 degrees, an origin on a face of the cube and one on
    an edge with a depth of field, two of them with seeded normals."""
    kw = dict(Tick=3, MaxChildRequestId=1 << 20)
    return [("fov_200", with_random_normals(sphere, 5), st.look_at((0.5, 0.5, 0.1), (0.5, 0.5, 0.9), 48, 32, 200.0, **kw)),
            ("on_face", sphere, st.look_at((1.0, 0.5, 0.5), (0.0, 0.5, 0.5), 48, 32, 60.0, **kw)),
            ("on_edge_dof", with_random_normals(sphere, 6),
             st.look_at((1.0, 1.0, 0.5), (0.3, 0.3, 0.5), 48, 32, 60.0, DoF=(0.05, 0.5), **kw))]


def test_extreme_views(sphere):
    for name, tree, v in mega_extreme_cases(sphere):
        ref, got = check(tree, v)
        assert got["n_requests"] > 0 and got["cones"].sum() > 1000, name


def mega_random_cases():
    """30 seeded random cameras (the trace's random-camera generator), every second
    tree with seeded normals."""
    from test_oracle_vs_reference import random_cameras
    return [(name, with_random_normals(tree, 40 + i) if i % 2 else tree, cam)
            for i, (name, tree, cam) in enumerate(random_cameras(seed=77, n=30, cap=1 << 20))]


def test_random_views():
    cones = 0
    for name, tree, v in mega_random_cases():
        ref, got = check(tree, v)
        cones += int(got["cones"].sum())
    assert cones > 100000


def test_axis_aligned_views(sphere):
    for name, tree, v in mega_axis_aligned_cases(sphere):
        ref, got = check(tree, v)
        assert got["cones"].sum() > 1000, name
    assert got["n_requests"] > 0


def test_cone_schedule_parameters(terrain):
    tree = with_random_normals(terrain, 4)
    v = st.look_at((0.2, 0.1, 0.05), (0.5, 0.5, 0.8), 40, 32, 75.0, FovMultiplier=0.1, FovConstant=0.08,
                   WeightingMultiplier=0.1, WeightingConstant=0.3, Tick=3)
    ref, got = check(tree, v)
    assert got["cones"].max() > 40


def test_row_band(terrain):
    v = st.orbit_views(seed=9, n=1, width=64, height=48, distance=1.3)[0]
    check(with_random_normals(terrain, 5), v, rows=(17, 29))


def test_unusable_schedule_draws_nothing(sphere):
    v = st.orbit_views(seed=5, n=1, width=16, height=12)[0]
    for kw in ({"FovConstant": 0.0}, {"FovMultiplier": 1.0}, {"FovMultiplier": -1.0}):
        bad = dataclasses.replace(v, **kw)
        ref = po.ref_mega_trace_view(sphere, bad)
        got = po.mega_trace_view(sphere, bad)
        assert not ref["rgba"].any() and not got["rgba"].any()
        assert ref["n_requests"] == got["n_requests"] == 0


def test_endless_schedule_is_refused(sphere):
    # FovMultiplier -0.9 drives the spine angle negative: the reference's loop would not end
    v = dataclasses.replace(st.orbit_views(seed=5, n=1, width=8, height=8)[0], FovMultiplier=-0.9, FovConstant=0.01)
    with pytest.raises(ValueError):
        po.mega_trace_view(sphere, v, cone_limit=4096)
