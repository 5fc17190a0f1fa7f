"""CUDA trace kernel against the oracle, through the C ABI. Integer outputs (hit node
index, hit depth, usage ticks, child requests) must be bit-exact; t and RGBA are
compared bit-exactly as well, since the kernel performs the same IEEE operations in the
same order (the stated tolerance of 1e-5 relative is therefore not needed)."""
import glob
import os

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st
from test_golden_cpu import GOLDEN, load_case
from test_oracle_vs_reference import axis_aligned_cases, extreme_camera_cases, random_cameras

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(tracer):
    tracer.set_config(block_size=192, ctas_per_sm=0, ray_chunk=1, cadence=16, max_steps=1 << 16, collect_stats=0,
                      schedule=st.SCHEDULE_LANE)
    yield

T_RTOL = 1e-5  # the required tolerance for t and RGBA (relative); the checks below are tighter (exact)


NONE_BLOCK = 0xFFFFFFFF


def assert_same(got, want, label=""):
    for k in ("hit_index", "hit_depth", "t", "rgba"):
        a = getattr(got, k)
        b = want[k]
        if k in ("t", "rgba"):
            np.testing.assert_allclose(a, b, rtol=T_RTOL, atol=0, err_msg=label + k)
        assert np.array_equal(a, b), "%s%s: %d pixels differ" % (label, k, int((a != b).sum()))


def same_requests(a, b):
    """(equal, short message) for two child-request arrays in any order."""
    a, b = po.sort_requests(a), po.sort_requests(b)
    if len(a) != len(b):
        return False, "request count %d vs %d" % (len(a), len(b))
    bad = np.nonzero((a.view(np.uint8).reshape(-1, 40) != b.view(np.uint8).reshape(-1, 40)).any(axis=1))[0]
    if len(bad):
        return False, "%d of %d requests differ, first %r vs %r" % (len(bad), len(a), a[bad[0]], b[bad[0]])
    return True, ""


def run_both(tracer, tree, cam, max_steps=1 << 16):
    tracer.set_config(max_steps=max_steps, collect_stats=2)
    tracer.upload(tree)
    tracer.init_usage()
    got = tracer.trace(cam)
    usage = tracer.read_usage(len(tree.Blocks) // 8)
    req, n = tracer.read_child_requests()
    stats = tracer.stats()
    vb, vs = tracer.ray_counts(cam.ScreenSize[0] * cam.ScreenSize[1])
    u_ref = po.init_usage(tree)
    want = po.trace_view(tree, cam, usage=u_ref, max_steps=max_steps)
    return got, usage, req, n, stats, (vb, vs), want, u_ref


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden_fixture(tracer, path):
    tree, cam, z = load_case(path)
    tracer.set_config(collect_stats=0)
    tracer.upload(tree)
    tracer.init_usage()
    got = tracer.trace(cam)
    assert_same(got, {k: z[k] for k in ("hit_index", "hit_depth", "t", "rgba")}, os.path.basename(path) + " ")
    usage = tracer.read_usage(len(tree.Blocks) // 8)
    assert np.array_equal(usage["tick"], z["usage_tick"])
    req, n = tracer.read_child_requests()
    assert n == int(z["n_requests"])
    ok, msg = same_requests(req, z["requests"].reshape(-1).view(st.CHILD_REQUEST_DTYPE))
    assert ok, msg


SCENES = [
    ("sphere_b4_d8", st.SCENE_SPHERE, 1, 4, 8, (1.2, 0.75, 0.1), (0.5, 0.5, 0.5), 160, 120, 60.0, (0.0, 0.0)),
    ("sphere_inside", st.SCENE_SPHERE, 2, 4, 8, (0.9, 0.1, 0.15), (0.4, 0.6, 0.5), 128, 96, 80.0, (0.0, 0.0)),
    ("sphere_dof", st.SCENE_SPHERE, 3, 3, 8, (0.1, 1.3, 0.3), (0.5, 0.5, 0.5), 96, 64, 60.0, (0.01, 0.7)),
    ("terrain_b4_d9", st.SCENE_TERRAIN, 5, 4, 9, (0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 320, 180, 60.0, (0.0, 0.0)),
    ("terrain_b2_d8_odd", st.SCENE_TERRAIN, 7, 2, 8, (0.93, 0.81, 0.4), (0.2, 0.3, 0.95), 77, 53, 90.0, (0.0, 0.0)),
    # base depth 6: 299,592 base chunks (585 KB) do not fit shared memory, the kernels read them from global memory
    ("terrain_b6_d10_global_bases", st.SCENE_TERRAIN, 5, 6, 10, (0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 320, 180, 60.0,
     (0.0, 0.0)),
    ("sphere_inside_b6_d9_global_bases", st.SCENE_SPHERE, 2, 6, 9, (0.9, 0.1, 0.15), (0.4, 0.6, 0.5), 256, 192, 60.0,
     (0.0, 0.0)),
]


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
@pytest.mark.parametrize("scene", SCENES, ids=[s[0] for s in SCENES])
def test_trace_matches_oracle(tracer, scene, schedule):
    _, kind, seed, b, d, o, t, w, h, fov, dof = scene
    tracer.set_config(schedule=schedule)
    tree = st.TreeBuilder(kind, seed=seed).BuildTree(b, d)
    cam = st.look_at(o, t, w, h, fov, DoF=dof, Tick=17, MaxChildRequestId=1 << 20)
    got, usage, req, n, stats, (vb, vs), want, u_ref = run_both(tracer, tree, cam)
    assert_same(got, want)
    assert np.array_equal(usage["tick"], u_ref["tick"]), "%d usage ticks differ" % int((usage["tick"] != u_ref["tick"]).sum())
    assert n == want["n_requests"]
    ok, msg = same_requests(req, want["requests"])
    assert ok, msg
    # algorithmic-byte accounting (V_block, V_base) matches the reference walk the oracle counts
    assert np.array_equal(vb, want["v_block"]), "V_block differs for %d rays" % int((vb != want["v_block"]).sum())
    assert np.array_equal(vs, want["v_base"]), "V_base differs for %d rays" % int((vs != want["v_base"]).sum())
    assert stats["rays"] == w * h
    assert stats["hits"] == int((want["hit_index"] != st.MISS).sum())
    assert stats["block_node_reads"] == int(want["v_block"].sum())
    assert stats["base_steps"] == int(want["v_base"].sum())
    assert stats["step_limited"] == 0


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_step_limit_matches_oracle(tracer, schedule):
    tracer.set_config(schedule=schedule)
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(3, 8)
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 64, 36, 60.0)
    got, usage, req, n, stats, _, want, u_ref = run_both(tracer, tree, cam, max_steps=12)
    assert want["step_limited"] > 0
    assert stats["step_limited"] == want["step_limited"]
    assert_same(got, want)
    assert np.array_equal(usage["tick"], u_ref["tick"])


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_small_step_limits_inside_base_level_runs(tracer, schedule):
    """Step limits of 1 to 8 stop rays in the middle of their first descents, which
    the kernel runs as base-level runs within one step call (B = 4, so a ray's
    first four steps are base levels): each limit must stop every ray at the same
    step as the oracle, with the same stamps, per-ray counts and outputs."""
    tracer.set_config(schedule=schedule)
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(4, 9)
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 48, 32, 60.0)
    for limit in range(1, 9):
        got, usage, req, n, stats, (vb, vs), want, u_ref = run_both(tracer, tree, cam, max_steps=limit)
        assert want["step_limited"] > 0
        assert stats["step_limited"] == want["step_limited"], limit
        assert_same(got, want, "max_steps %d" % limit)
        assert np.array_equal(usage["tick"], u_ref["tick"]), limit
        assert np.array_equal(vs, want["v_base"]), limit
        assert np.array_equal(vb, want["v_block"]), limit


def deep_needle_tree(p, depth=24):
    """A tree at the deepest level the library takes (SVO_MAX_TREE_DEPTH = 24) and the
    smallest base depth (1): air everywhere except a one-cell needle of geometry
    around the point p, one node per level from the base down to level 24."""
    P = [int(np.float64(v) * 2.0 ** 64) for v in p]

    def oc(d):  # p's octant below level d
        s = 63 - d
        return ((P[0] >> s) & 1) | (((P[1] >> s) & 1) << 1) | (((P[2] >> s) & 1) << 2)

    B = 1
    bases = np.full(st.pow_sum(B), 0x5555, np.uint16)
    bases[oc(0)] = 0x5555 | (2 << (2 * oc(1)))
    chain = depth - (B + 2)
    blocks = np.zeros(512 + 8 * chain, st.BLOCK_DTYPE)
    blocks["child"] = NONE_BLOCK
    blocks["chunk"] = 0x5555
    blocks["colour_r"], blocks["colour_g"], blocks["colour_b"] = 180, 90, 40
    dense = oc(0) * 64 + oc(1) * 8 + oc(2)
    blocks[dense]["chunk"] = 0x5555 | (2 << (2 * oc(3)))
    blocks[dense]["child"] = 512
    for k in range(chain):
        level = B + 3 + k
        node = 512 + 8 * k + oc(level - 1)
        blocks[node]["chunk"] = 0x5555 | (2 << (2 * oc(level)))
        if k + 1 < chain:
            blocks[node]["child"] = 512 + 8 * (k + 1)
    return st.Octree(B, len(blocks), bases, blocks)


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_deepest_tree(tracer, schedule):
    """Maximum sizes: a needle of geometry down to level 24 in a tree of base depth
    1, seen with cones narrow enough to reach it. The LOD stops rays at levels 20 and
    22 for wider views and lets the narrowest reach the level-24 leaf, which has no
    children and raises requests; every output, stamp and request equals the
    oracle's."""
    tracer.set_config(schedule=schedule)
    p = (0.3127, 0.4271, 0.5833)
    tree = deep_needle_tree(p)
    o = (p[0] + 0.2, p[1] + 0.15, p[2] - 0.1)
    deepest = 0
    for fov in (1e-4, 2e-5, 4e-6, 1e-6):
        cam = st.look_at(o, p, 32, 32, np.degrees(fov), Tick=2, MaxChildRequestId=4096)
        got, usage, req, n, stats, (vb, vs), want, u_ref = run_both(tracer, tree, cam)
        assert_same(got, want, "FoV %g: " % fov)
        assert np.array_equal(usage["tick"], u_ref["tick"])
        ok, msg = same_requests(req[:n], want["requests"])
        assert ok, msg
        assert np.array_equal(vb, want["v_block"]) and np.array_equal(vs, want["v_base"])
        deepest = max(deepest, int(got.hit_depth.max()))
    assert deepest == 24


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_axis_aligned_rays(tracer, schedule):
    """Rays with direction components that are exactly zero (infinite inverse
    direction), origins on the cell boundaries of every level and on the cube's
    corner, and child requests raised along an axis: equal to the oracle, which
    the CPU tests pin to the reference's kernels on the same cameras."""
    tracer.set_config(schedule=schedule)
    for name, tree, cam in axis_aligned_cases():
        got, usage, req, n, stats, (vb, vs), want, u_ref = run_both(tracer, tree, cam)
        assert_same(got, want, name + ": ")
        assert np.array_equal(usage["tick"], u_ref["tick"]), name
        assert n == want["n_requests"], name
        ok, msg = same_requests(req, want["requests"])
        assert ok, name + ": " + msg
        assert np.array_equal(vb, want["v_block"]) and np.array_equal(vs, want["v_base"]), name


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_extreme_cameras(tracer, schedule):
    """Fields of view past 180 degrees and origins on a face and an edge of the
    cube: equal to the oracle (pinned to the reference's kernels on the CPU)."""
    tracer.set_config(schedule=schedule)
    for name, tree, cam in extreme_camera_cases():
        got, usage, req, n, stats, _, want, u_ref = run_both(tracer, tree, cam)
        assert_same(got, want, name + ": ")
        assert np.array_equal(usage["tick"], u_ref["tick"]), name
        assert n == want["n_requests"], name
        ok, msg = same_requests(req, want["requests"])
        assert ok, name + ": " + msg


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_random_cameras(tracer, schedule):
    """60 seeded random cameras (origins in and around the cube, 1-96 pixels each
    way, fields of view 5-350 degrees, depth of field on a third): every output,
    the usage ticks, the child requests and the per-ray walk counts equal the
    oracle's; the CPU tests pin the oracle to the reference on the same cameras."""
    tracer.set_config(schedule=schedule)
    for name, tree, cam in random_cameras(cap=1 << 20):
        got, usage, req, n, stats, (vb, vs), want, u_ref = run_both(tracer, tree, cam)
        assert_same(got, want, name + ": ")
        assert np.array_equal(usage["tick"], u_ref["tick"]), name
        assert n == want["n_requests"], name
        ok, msg = same_requests(req, want["requests"])
        assert ok, name + ": " + msg
        assert np.array_equal(vb, want["v_block"]) and np.array_equal(vs, want["v_base"]), name


@pytest.mark.parametrize("kind", ["all_air", "solid_without_blocks"])
def test_degenerate_trees(tracer, kind):
    """Empty and degenerate inputs: a tree of air only (every ray reaches the sky
    and stamps nothing), and one that is geometry everywhere with no block level
    below the dense one (every ray that enters stops at level B+2 and asks for
    children). Equal to the oracle, from outside and from inside the cube."""
    B = 2
    bases = np.full(st.pow_sum(B), 0x5555 if kind == "all_air" else 0xAAAA, np.uint16)
    blocks = np.zeros(8 ** (B + 2), st.BLOCK_DTYPE)
    blocks["child"] = NONE_BLOCK
    blocks["chunk"] = 0x5555 if kind == "all_air" else 0xAAAA
    blocks["colour_g"] = 120
    tree = st.Octree(B, len(blocks), bases, blocks)
    for cam in (st.look_at((1.6, 1.3, -0.4), (0.5, 0.5, 0.5), 40, 24, 60.0, Tick=3, MaxChildRequestId=1 << 12),
                st.look_at((0.4, 0.5, 0.6), (0.9, 0.1, 0.3), 24, 40, 80.0, Tick=3, MaxChildRequestId=1 << 12)):
        got, usage, req, n, stats, (vb, vs), want, u_ref = run_both(tracer, tree, cam)
        assert_same(got, want, kind + ": ")
        assert np.array_equal(usage["tick"], u_ref["tick"])
        ok, msg = same_requests(req[:n], want["requests"])
        assert ok, msg
        if kind == "all_air":
            assert (got.hit_index == st.MISS).all() and n == 0
        else:
            hit = got.hit_index != st.MISS
            assert hit.any() and (got.hit_depth[hit] == B + 2).all() and n == int(hit.sum())


def test_request_cap(tracer):
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(2, 7)
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 128, 72, 60.0, MaxChildRequestId=50)
    tracer.set_config(collect_stats=0)
    tracer.upload(tree)
    tracer.trace(cam)
    req, n = tracer.read_child_requests()
    want = po.trace_view(tree, cam)
    assert n == want["n_requests"] > 50
    assert len(req) == 50
    allowed = {r.tobytes() for r in want["requests"]}
    assert all(r.tobytes() in allowed for r in req)


def test_batch_equals_single_views_and_graph(tracer):
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=3).BuildTree(4, 9)
    rng = np.random.default_rng(0)
    cams = []
    for i in range(6):
        w, h = [(64, 48), (33, 17), (128, 72), (1, 1), (200, 3), (96, 96)][i]
        o = (rng.uniform(0.05, 0.95), rng.uniform(0.05, 0.95), rng.uniform(0.3, 0.6))
        cams.append(st.look_at(o, (0.5, 0.5, 0.85), w, h, rng.uniform(40, 90), Tick=4))
    tracer.set_config(collect_stats=0)
    tracer.upload(tree)
    singles = [tracer.trace(c) for c in cams]
    batch = tracer.trace_batch(cams)
    graph1 = tracer.trace_batch(cams, graph=True)
    graph2 = tracer.trace_batch(cams, graph=True)  # replay
    for s, b, g1, g2 in zip(singles, batch, graph1, graph2):
        for k in ("hit_index", "hit_depth", "t", "rgba"):
            assert np.array_equal(getattr(s, k), getattr(b, k))
            assert np.array_equal(getattr(s, k), getattr(g1, k))
            assert np.array_equal(getattr(s, k), getattr(g2, k))
    for c, s in zip(cams, singles):  # includes the 1x1 and 200x3 views
        want = po.trace_view(tree, c)
        assert_same(s, want)


@pytest.mark.parametrize("schedule", [st.SCHEDULE_LANE, st.SCHEDULE_WARP, st.SCHEDULE_WAVEFRONT],
                         ids=["lane", "warp", "wavefront"])
def test_random_views_in_one_batch(tracer, schedule):
    """30 seeded random views of one tree (1-96 pixels each way, ragged tiles) in
    one batched launch and its graph replay: every view's outputs, the usage
    ticks stamped by all views and the union of their child requests equal the
    oracle's view by view."""
    import dataclasses
    cases = [c for i, c in enumerate(random_cameras(seed=33, n=60, cap=1 << 20)) if i % 2 == 0]
    tree = cases[0][1]
    views = [dataclasses.replace(cam, Tick=9) for _, _, cam in cases]
    tracer.set_config(schedule=schedule, collect_stats=0)
    tracer.upload(tree)
    tracer.init_usage()
    batch = tracer.trace_batch(views, graph=True)
    req, n = tracer.read_child_requests()
    tracer.init_usage()
    replay = tracer.trace_batch(views, graph=True)
    usage = tracer.read_usage(len(tree.Blocks) // 8)
    u_ref = po.init_usage(tree)
    wants = [po.trace_view(tree, v, usage=u_ref) for v in views]
    for (name, _, _), b, r, want in zip(cases, batch, replay, wants):
        assert_same(b, want, name + ": ")
        assert_same(r, want, name + " (replay): ")
    assert np.array_equal(usage["tick"], u_ref["tick"])
    want_req = np.concatenate([w["requests"] for w in wants])
    assert n == len(want_req)
    ok, msg = same_requests(req, want_req)
    assert ok, msg


def test_l2_window_in_graph_replay(tracer):
    """A graph captured with the L2 persisting window on replays the same frames."""
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=3).BuildTree(3, 8)
    cams = [st.look_at((0.2, 0.3, 0.4), (0.5, 0.5, 0.85), w, h, 60.0, Tick=2) for w, h in ((64, 48), (37, 19))]
    tracer.set_config(collect_stats=0, schedule=st.SCHEDULE_WARP)
    tracer.upload(tree)
    want = tracer.trace_batch(cams)
    tracer.set_config(l2_window=1)
    try:
        got = [tracer.trace_batch(cams, graph=True) for _ in range(2)]
    finally:
        tracer.set_config(l2_window=-1)
    for g in got:
        for a, b in zip(want, g):
            for k in ("hit_index", "hit_depth", "t", "rgba"):
                assert np.array_equal(getattr(a, k), getattr(b, k))


@pytest.mark.parametrize("cfg", [dict(block_size=128, ray_chunk=1, cadence=1),
                                 dict(block_size=256, ray_chunk=8, cadence=32),
                                 dict(block_size=64, ray_chunk=3, cadence=5, ctas_per_sm=1),
                                 dict(block_size=128, schedule=st.SCHEDULE_WARP),
                                 dict(block_size=256, schedule=st.SCHEDULE_WARP),
                                 dict(block_size=64, schedule=st.SCHEDULE_WARP, ctas_per_sm=1),
                                 dict(schedule=st.SCHEDULE_WARP, l2_window=1),
                                 dict(block_size=96, schedule=st.SCHEDULE_WAVEFRONT),
                                 dict(block_size=256, schedule=st.SCHEDULE_WAVEFRONT, ctas_per_sm=1)])
def test_launch_shapes_do_not_change_results(tracer, cfg):
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=6).BuildTree(4, 8)
    cam = st.look_at((1.1, 0.2, 0.9), (0.5, 0.5, 0.5), 120, 90, 60.0)
    tracer.set_config(collect_stats=0, **cfg)
    try:
        tracer.upload(tree)
        got = tracer.trace(cam)
    finally:
        tracer.set_config(block_size=256, ray_chunk=1, cadence=16, ctas_per_sm=0, schedule=st.SCHEDULE_LANE,
                          l2_window=-1)
    assert_same(got, po.trace_view(tree, cam))


def test_mixed_views_batched_graph_equals_plain_launches(tracer):
    """The 64 mixed-resolution views traced in one (graph-replayed, autotuned) launch
    give the same per-view results as 64 plain launches; a few views against the oracle."""
    torch = pytest.importorskip("torch")
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(4, 10)
    views = st.mixed_views(seed=4, Tick=3)
    tracer.upload(tree)
    sizes = [v.ScreenSize[0] * v.ScreenSize[1] for v in views]
    dev_outs = []
    keep = []
    for n in sizes:
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        dep = torch.empty(n, dtype=torch.uint8, device="cuda")
        tt = torch.empty(n, dtype=torch.float32, device="cuda")
        rgba = torch.empty(4 * n, dtype=torch.float32, device="cuda")
        keep.append((idx, dep, tt, rgba))
        dev_outs.append((idx.data_ptr(), dep.data_ptr(), tt.data_ptr(), rgba.data_ptr()))
    cfg, ms = tracer.autotune(views, dev_outs, repeats=1)
    assert cfg["block_size"] in (64, 128, 192, 256) and ms > 0
    tracer.trace_device(views, dev_outs, graph=True)
    tracer.trace_device(views, dev_outs, graph=True)  # replay
    torch.cuda.synchronize()
    batched = [tuple(x.cpu() for x in k) for k in keep]
    tracer.set_config(block_size=256, ray_chunk=1, cadence=16, schedule=st.SCHEDULE_LANE)
    for v, o in zip(views, dev_outs):
        tracer.trace_device([v], [o])
    torch.cuda.synchronize()
    for b, k in zip(batched, keep):
        for x, y in zip(b, k):
            assert torch.equal(x, y.cpu())
    small = sorted(range(len(views)), key=lambda i: sizes[i])[:3]
    for i in small:
        want = po.trace_view(tree, views[i])
        assert np.array_equal(batched[i][0].numpy().view(np.uint32), want["hit_index"])
        assert np.array_equal(batched[i][3].numpy().reshape(-1, 4), want["rgba"])


@pytest.fixture(scope="module")
def terrain11():
    """The benchmarked tree: the depth-11 fBm terrain (seed 5, base depth 4, ~48M nodes)."""
    return st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(4, 11)


def test_full_size_mixed_views_against_oracle(tracer, terrain11):
    """The 64 mixed-resolution views at their stated size (30.9M rays, 128x128 to
    1920x1080 in pixel count) over the benchmarked depth-11 terrain, traced in one
    graph-replayed batch: every ray of every view equals the oracle, the hit
    outputs and t and RGBA bit for bit."""
    tree = terrain11
    views = st.mixed_views(seed=4, Tick=7, MaxChildRequestId=1 << 16)
    assert sum(v.ScreenSize[0] * v.ScreenSize[1] for v in views) == 30908596
    tracer.set_config(collect_stats=0, schedule=st.SCHEDULE_WARP, block_size=128)
    tracer.upload(tree)
    tracer.trace_batch(views, graph=True)
    got = tracer.trace_batch(views, graph=True)  # a replay of the captured graph
    tracer.set_config(block_size=256)
    for i, (v, g) in enumerate(zip(views, got)):
        want = po.trace_view(tree, v)
        for k in ("hit_index", "hit_depth", "t", "rgba"):
            assert np.array_equal(getattr(g, k), want[k]), "view %d (%dx%d): %s" % (i, *v.ScreenSize, k)


def test_full_size_terrain_1080p(tracer, terrain11):
    """The headline workload: 1920x1080 over the depth-11 terrain (~48M nodes),
    compared pixel for pixel with the oracle (OpenMP over all host cores)."""
    tree = terrain11
    cam = st.look_at((0.08, 0.12, 0.62), (0.75, 0.8, 0.88), 1920, 1080, 60.0, Tick=21, MaxChildRequestId=1 << 16)
    tracer.set_config(collect_stats=0)
    tracer.upload(tree)
    tracer.init_usage()
    a = tracer.trace(cam)
    b = tracer.trace(cam)  # idempotent
    for k in ("hit_index", "hit_depth", "t", "rgba"):
        assert np.array_equal(getattr(a, k), getattr(b, k))
    hit = a.hit_index != st.MISS
    assert hit.mean() > 0.5
    assert (a.hit_index[hit] < len(tree.Blocks)).all()
    assert ((a.hit_depth[hit] >= 6) & (a.hit_depth[hit] <= 11)).all()
    assert np.isfinite(a.t[hit]).all() and np.isinf(a.t[~hit]).all()
    assert ((a.rgba >= 0) & (a.rgba <= 1)).all()
    u_ref = po.init_usage(tree)
    want = po.trace_view(tree, cam, usage=u_ref)
    assert_same(a, want)
    usage = tracer.read_usage(len(tree.Blocks) // 8)
    assert np.array_equal(usage["tick"], u_ref["tick"])


def test_errors(tracer):
    lib = st.load_library()
    with st.Tracer(0) as fresh:
        with pytest.raises(st.SvoError) as e:
            fresh.trace(st.TraceInput(ScreenSize=(8, 8)))
        assert "NoTree" in str(e.value)
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(2, 5)
    tracer.upload(tree)
    with pytest.raises(st.SvoError):
        tracer.trace(st.TraceInput(ScreenSize=(0, 8)))
    with pytest.raises(st.SvoError):
        tracer.trace(st.TraceInput(ScreenSize=(8, 8), BaseDepth=3))
    with pytest.raises(st.SvoError):
        tracer.set_config(block_size=100)
    with pytest.raises(st.SvoError):
        tracer.set_config(schedule=4)
    with pytest.raises(st.SvoError):
        tracer.set_config(l2_window=2)
    assert lib is not None


def test_random_cameras_pinned_host_outputs(tracer):
    """30 seeded random cameras traced into pinned host outputs (written by the
    kernel over 8x4 tiles, hit depth staged in device memory) and, as a graph-
    replayed batch, into pinned host outputs: equal to the oracle."""
    torch = pytest.importorskip("torch")
    import dataclasses
    cases = [c for i, c in enumerate(random_cameras(seed=44, n=60, cap=1 << 20)) if i % 2 == 1]
    tree = cases[0][1]

    def pinned(w, h):
        n = w * h
        return st.TraceResult(torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
                              torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy(),
                              torch.empty(n, dtype=torch.float32, pin_memory=True).numpy(),
                              torch.empty(n * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(n, 4))

    tracer.upload(tree)
    tracer.init_usage()
    views = [dataclasses.replace(cam, Tick=5) for _, _, cam in cases]
    wants = [po.trace_view(tree, v) for v in views]
    for (name, _, _), v, want in zip(cases, views, wants):
        assert_same(tracer.trace(v, out=pinned(*v.ScreenSize)), want, name + ": ")
    outs = tracer.trace_batch(views, graph=True, out=[pinned(*v.ScreenSize) for v in views])
    for (name, _, _), got, want in zip(cases, outs, wants):
        assert_same(got, want, name + " (batch): ")


def test_pinned_host_outputs_equal_staged_outputs(tracer):
    """Host outputs in pinned memory are written by the kernel directly; pageable
    host outputs go through device buffers. Both give the same results, on two
    calls in a row and in a batch with one view's outputs partly absent."""
    torch = pytest.importorskip("torch")
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(3, 8)
    tracer.upload(tree)
    tracer.init_usage()
    cams = [st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 123, 77, 60.0, Tick=3),
            st.look_at((0.9, 0.2, 0.6), (0.3, 0.6, 0.9), 64, 48, 70.0, Tick=3)]

    def pinned(w, h):
        n = w * h
        return st.TraceResult(torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
                              torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy(),
                              torch.empty(n, dtype=torch.float32, pin_memory=True).numpy(),
                              torch.empty(n * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(n, 4))

    for cam in cams:
        for _ in range(2):
            want = tracer.trace(cam)  # pageable numpy outputs: staged
            got = tracer.trace(cam, out=pinned(*cam.ScreenSize))
            for k in ("hit_index", "hit_depth", "t", "rgba"):
                assert np.array_equal(getattr(got, k).reshape(-1), getattr(want, k).reshape(-1)), k
    assert (want.hit_index != st.MISS).any()
    # a batch (plain and graph-replayed) of pinned outputs, one view without its
    # hit depth (the output staged in device memory) and one without t, against
    # the oracle
    wants = [po.trace_view(tree, cam) for cam in cams]
    for graph in (False, True):
        for _ in range(2):
            outs = [pinned(*cam.ScreenSize) for cam in cams]
            outs[0].hit_depth = None
            outs[1].t = None
            got = tracer.trace_batch(cams, graph=graph, out=outs)
            for g, w in zip(got, wants):
                assert np.array_equal(g.hit_index, w["hit_index"])
                assert np.array_equal(g.rgba.view(np.uint32), w["rgba"].view(np.uint32))
            assert np.array_equal(got[0].t.view(np.uint32), wants[0]["t"].view(np.uint32))
            assert np.array_equal(got[1].hit_depth, wants[1]["hit_depth"])
