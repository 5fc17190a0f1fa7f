"""svo_mega_trace (kernel.cl's `trace`: primary cone, spawnRays's cone fan, draw)
against the megakernel oracle: bit-exact image, primary hit outputs, child
requests and usage ticks."""
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
def sphere():
    return st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(3, 8)


@pytest.fixture(scope="module")
def terrain():
    return with_random_normals(st.TreeBuilder(st.SCENE_TERRAIN, seed=2).BuildTree(3, 8), 21)


@pytest.fixture(scope="module")
def terrain_global_bases():
    """Base depth 6: the base chunks (585 KB) are read from global memory, not staged in shared memory."""
    return st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(6, 10)


@pytest.fixture(scope="module")
def tracer():
    t = st.Tracer(0)
    yield t
    t.close()


def run_both(tracer, tree, view, **cfg):
    tracer.upload(tree)
    tracer.init_usage()
    if cfg:
        tracer.set_config(**cfg)
    try:
        got = tracer.mega_trace(view)
        stats = tracer.mega_stats()
        gpu_req, n_req = tracer.read_child_requests()
        gpu_usage = tracer.read_usage()
    finally:
        if cfg:
            tracer.set_config(**{k: 0 for k in cfg})
    usage = po.init_usage(tree)
    ref = po.mega_trace_view(tree, view, usage=usage)
    assert n_req == len(gpu_req)
    return got, stats, gpu_req, gpu_usage, ref, usage


def check(tracer, tree, view, **cfg):
    view = dataclasses.replace(view, MaxChildRequestId=1 << 20)
    got, stats, gpu_req, gpu_usage, ref, usage = run_both(tracer, tree, view, **cfg)
    n = view.ScreenSize[0] * view.ScreenSize[1]
    assert np.array_equal(got.rgba.reshape(n, 4).view(np.uint32), ref["rgba"].view(np.uint32))
    assert np.array_equal(got.hit_index.reshape(-1), ref["hit_index"])
    assert np.array_equal(got.hit_depth.reshape(-1), ref["hit_depth"])
    assert np.array_equal(got.t.reshape(-1).view(np.uint32), ref["t"].view(np.uint32))
    assert len(gpu_req) == ref["n_requests"]
    a, b = po.sort_requests(gpu_req), po.sort_requests(ref["requests"])
    for f in ("address", "tick", "depth", "location", "tree_size"):
        assert np.array_equal(a[f], b[f]), f
    assert np.array_equal(gpu_usage["tick"][: len(usage)], usage["tick"])
    assert stats["pixels"] == n
    assert stats["cones"] == int(ref["cones"].sum())
    assert stats["surfaces"] == int((ref["hit_index"] != st.MISS).sum())
    return got, stats, ref


@pytest.mark.parametrize("k", range(3))
def test_sphere_orbit_views(tracer, sphere, k):
    v = st.orbit_views(seed=5, n=3, width=64, height=48)[k]
    check(tracer, sphere, v)


@pytest.mark.parametrize("k", range(3))
def test_terrain_random_normals(tracer, terrain, k):
    v = st.orbit_views(seed=7, n=3, width=67, height=45, distance=1.2)[k]  # ragged tiles
    got, stats, ref = check(tracer, terrain, v)
    assert ref["n_requests"] > 0 and stats["cones"] > 0


@pytest.mark.parametrize("schedule", ["lane", "warp"])
def test_cone_schedules(tracer, terrain, schedule):
    """Both cone-kernel schedules (warp batches of 32 list entries, lanes refilled
    every `cadence` steps) give the same frame."""
    v = st.orbit_views(seed=11, n=1, width=56, height=40, distance=1.25)[0]
    sched = {"lane": st.SCHEDULE_LANE, "warp": st.SCHEDULE_WARP}[schedule]
    check(tracer, terrain, v, schedule=sched, cadence=5)


@pytest.mark.parametrize("schedule", ["lane", "warp"])
def test_base_chunks_in_global_memory(tracer, terrain_global_bases, schedule):
    sched = {"lane": st.SCHEDULE_LANE, "warp": st.SCHEDULE_WARP}[schedule]
    for v in (st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 96, 54, 60.0, Tick=3),
              st.orbit_views(seed=11, n=1, width=56, height=40, distance=1.25)[0]):
        got, stats, ref = check(tracer, terrain_global_bases, v, schedule=sched, cadence=5)
        assert ref["n_requests"] > 0 and stats["surfaces"] > 0


@pytest.mark.parametrize("schedule", ["lane", "warp"])
def test_axis_aligned_views(tracer, sphere, schedule):
    """Direction components exactly zero and an origin on the cell boundaries of
    every level; the CPU tests pin the oracle to kernel.cl on the same views."""
    from test_mega_oracle import mega_axis_aligned_cases
    sched = {"lane": st.SCHEDULE_LANE, "warp": st.SCHEDULE_WARP}[schedule]
    for name, tree, v in mega_axis_aligned_cases(sphere):
        check(tracer, tree, v, schedule=sched, cadence=5)


@pytest.mark.parametrize("schedule", ["lane", "warp"])
def test_random_views(tracer, schedule):
    """30 seeded random cameras; the CPU tests pin the oracle to kernel.cl on them."""
    from test_mega_oracle import mega_random_cases
    sched = {"lane": st.SCHEDULE_LANE, "warp": st.SCHEDULE_WARP}[schedule]
    for name, tree, v in mega_random_cases():
        check(tracer, tree, v, schedule=sched, cadence=7)


def test_extreme_views(tracer, sphere):
    """A field of view past 180 degrees and origins on a face and an edge of the
    cube (with a depth of field); the CPU tests pin the oracle to kernel.cl."""
    from test_mega_oracle import mega_extreme_cases
    for name, tree, v in mega_extreme_cases(sphere):
        check(tracer, tree, v)


@pytest.mark.parametrize("block_size", [64, 128, 256])
def test_block_sizes(tracer, terrain, block_size):
    """Launch shapes other than the default (192 threads) give the same frame."""
    v = st.orbit_views(seed=11, n=1, width=56, height=40, distance=1.25)[0]
    check(tracer, terrain, v, block_size=block_size)


def test_inside_cube_with_dof(tracer, sphere):
    v = st.look_at((0.5, 0.5, 0.12), (0.5, 0.55, 0.6), 48, 40, 70.0, DoF=(0.02, 0.3), Tick=9)
    check(tracer, with_random_normals(sphere, 3), v)


def test_other_cone_schedule_and_bands(tracer, terrain):
    v = st.look_at((0.2, 0.1, 0.05), (0.5, 0.5, 0.8), 40, 32, 75.0, FovMultiplier=0.1, FovConstant=0.08,
                   WeightingMultiplier=0.1, WeightingConstant=0.3, Tick=3)
    # 3 tiles per band: the fan, cone and resolve kernels run band after band
    got, stats, ref = check(tracer, terrain, v, mega_band_tiles=3)
    assert ref["cones"].max() > 40


def test_request_cap(tracer, terrain):
    v = dataclasses.replace(st.orbit_views(seed=7, n=1, width=64, height=48, distance=1.2)[0], MaxChildRequestId=50)
    tracer.upload(terrain)
    tracer.init_usage()
    tracer.mega_trace(v)
    req, n = tracer.read_child_requests()
    ref = po.mega_trace_view(terrain, v)
    assert ref["n_requests"] > 50 and len(req) == 50 and n == ref["n_requests"]
    assert tracer.stats()["child_requests"] == ref["n_requests"]


def test_unusable_schedule_draws_nothing(tracer, sphere):
    v = st.orbit_views(seed=5, n=1, width=16, height=12)[0]
    tracer.upload(sphere)
    for kw in ({"FovConstant": 0.0}, {"FovMultiplier": 1.0}, {"FovMultiplier": -1.0}):
        r = st.TraceResult(np.full((12, 16), 7, np.uint32), np.full((12, 16), 7, np.uint8),
                           np.full((12, 16), 7.0, np.float32), np.full((12, 16, 4), 7.0, np.float32))
        tracer.mega_trace(dataclasses.replace(v, **kw), out=r)
        assert (r.hit_index == 7).all() and (r.rgba == 7.0).all()
        assert tracer.mega_stats()["pixels"] == 0


def test_endless_schedule_is_refused(tracer, sphere):
    v = dataclasses.replace(st.orbit_views(seed=5, n=1, width=8, height=8)[0], FovMultiplier=-0.9, FovConstant=0.01)
    tracer.upload(sphere)
    with pytest.raises(st.SvoError):
        tracer.mega_trace(v)


def test_output_kinds_agree(tracer, terrain):
    """Pageable host outputs (staged through device buffers), pinned host outputs
    (written by the kernels) and device outputs give the same frame."""
    torch = pytest.importorskip("torch")
    v = dataclasses.replace(st.orbit_views(seed=12, n=1, width=61, height=37, distance=1.2)[0], Tick=4)
    tracer.upload(terrain)
    tracer.init_usage()
    want = tracer.mega_trace(v)
    n = 61 * 37
    pinned = st.TraceResult(torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
                            torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy(),
                            torch.empty(n, dtype=torch.float32, pin_memory=True).numpy(),
                            torch.empty(n * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(n, 4))
    got = tracer.mega_trace(v, out=pinned)
    dev = [torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.uint8, device="cuda"),
           torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(4 * n, dtype=torch.float32, device="cuda")]
    tracer.mega_trace_device(v, *[x.data_ptr() for x in dev])
    tracer.synchronize()
    on_dev = [x.cpu().numpy() for x in dev]
    for k, d in zip(("hit_index", "hit_depth", "t", "rgba"), on_dev):
        a = getattr(want, k).reshape(-1)
        assert np.array_equal(getattr(got, k).reshape(-1).view(np.uint8), a.view(np.uint8)), k
        assert np.array_equal(d.reshape(-1).view(np.uint8), a.view(np.uint8)), k


def test_step_limit_matches_oracle(tracer, terrain):
    """A primary cone or secondary cone stopped by max_steps ends as sky, on the GPU
    and in the oracle alike."""
    v = dataclasses.replace(st.orbit_views(seed=13, n=1, width=48, height=32, distance=1.2)[0], Tick=2,
                            MaxChildRequestId=1 << 20)
    tracer.upload(terrain)
    tracer.init_usage()
    tracer.set_config(max_steps=24)
    try:
        got = tracer.mega_trace(v)
        req, n = tracer.read_child_requests()
    finally:
        tracer.set_config(max_steps=0)
    ref = po.mega_trace_view(terrain, v, max_steps=24)
    full = po.mega_trace_view(terrain, v)
    assert not np.array_equal(ref["rgba"], full["rgba"])  # the limit changes the frame
    assert np.array_equal(got.rgba.reshape(-1, 4).view(np.uint32), ref["rgba"].view(np.uint32))
    assert np.array_equal(got.hit_index.reshape(-1), ref["hit_index"])
    assert n == ref["n_requests"]


@pytest.mark.parametrize("size", [(1, 1), (1, 37), (37, 1), (5, 3), (130, 2)])
def test_degenerate_view_sizes(tracer, terrain, size):
    """Single pixels, single rows and columns, and views narrower than one warp tile:
    the padded lanes of each tile draw nothing and the real pixels match the oracle."""
    w, h = size
    v = st.look_at((0.15, 0.2, 0.1), (0.55, 0.5, 0.8), w, h, 50.0, Tick=6)
    check(tracer, terrain, v)


def test_view_away_from_the_cube(tracer, sphere):
    """Every primary cone misses the volume: nothing is requested, no cone fan is
    spawned, and every pixel is what the oracle draws for a miss."""
    v = st.look_at((1.6, 0.5, 0.5), (3.0, 0.5, 0.5), 24, 16, 40.0, Tick=5)
    got, stats, ref = check(tracer, sphere, v)
    assert stats["surfaces"] == 0 and stats["cones"] == 0 and ref["n_requests"] == 0
