"""Tree-update kernels (usage initialisation, block GC, grafting, pruning) against the
oracle, through the C ABI. Every set the specification defines (pruned, freed,
free-list and claimed groups) and the whole block and usage arrays must be bit-exact."""
import dataclasses

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu
NONE = 0xFFFFFFFF


@pytest.fixture(autouse=True)
def default_config(tracer):
    tracer.set_config(block_size=192, ctas_per_sm=0, ray_chunk=1, cadence=16, max_steps=1 << 16, collect_stats=0)
    yield


def gpu_state(tr, n_groups):
    return tr.read_blocks(0, n_groups * 8), tr.read_usage(n_groups)


def assert_state(tr, oracle, label):
    blocks, usage = gpu_state(tr, oracle.n_groups)
    bad_b = int((blocks.view(np.uint8).reshape(-1, 16) != oracle.blocks.view(np.uint8).reshape(-1, 16)).any(1).sum())
    bad_u = int((usage.view(np.uint8).reshape(-1, 8) != oracle.usage.view(np.uint8).reshape(-1, 8)).any(1).sum())
    assert bad_b == 0 and bad_u == 0, "%s: %d nodes and %d usage entries differ" % (label, bad_b, bad_u)


def test_init_usage_tree_matches_oracle(tracer):
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=9)
    tree = scene.build_tree(8)
    budget = 1 << 16
    tracer.upload(tree, block_budget=budget * 8)
    tracer.init_usage_tree(11)
    oracle = po.TreeState(tree, budget)
    oracle.init_usage_tree(11)
    assert_state(tracer, oracle, "init")


@pytest.mark.parametrize("base_depth,depth,initial,budget,threshold,scene_seed,path_seed",
                         [(3, 9, 7, 1 << 15, 3, 5, 3), (2, 8, 6, 1 << 13, 2, 5, 3),
                          (6, 10, 9, (1 << 21) + (1 << 16), 2, 5, 3),
                          (3, 9, 7, 1 << 15, 1, 11, 17), (2, 9, 6, 1 << 14, 4, 23, 29), (3, 10, 8, 1 << 17, 2, 31, 41)],
                         ids=["b3", "b2", "b6_global_bases", "seeded_a", "seeded_b", "seeded_c"])
def test_stream_matches_oracle(tracer, base_depth, depth, initial, budget, threshold, scene_seed, path_seed):
    """Frames of the streaming workflow: trace (usage stamps + child requests), graft
    payloads from the procedural scene, GC of groups unused for `threshold` frames,
    grafting into freed groups; GPU and oracle evolve their own copies of the tree.
    Base depth 6: 2.1M dense groups at level 8, base chunks in global memory. The
    seeded cases vary the scene, the camera path, the tree's initial depth and
    the staleness threshold (1 to 4 frames)."""
    scene = st.Scene(st.SCENE_TERRAIN, seed=scene_seed, base_depth=base_depth, depth=depth)
    tree = scene.build_tree(initial)
    tracer.upload(tree, block_budget=budget * 8)
    tracer.init_usage_tree(1)
    oracle = po.TreeState(tree, budget)
    oracle.init_usage_tree(1)
    cams = st.camera_path(seed=path_seed, frames=10, width=160, height=90, MaxChildRequestId=1 << 16)
    grafted_total = pruned_total = 0
    for f, cam in enumerate(cams):
        tick = f + 1
        got = tracer.trace(cam)
        want = po.trace_view(oracle.as_octree(), cam, usage=oracle.usage)
        for k in ("hit_index", "hit_depth", "t", "rgba"):
            assert np.array_equal(getattr(got, k), want[k]), "frame %d: %s" % (f, k)
        req, n = tracer.read_child_requests()
        assert n == want["n_requests"]
        same = po.sort_requests(req).tobytes() == po.sort_requests(want["requests"]).tobytes()
        assert same, "frame %d: child requests differ" % f
        rec, pay = scene.graft_payload(req)
        rep = tracer.gc(tick, threshold)
        g_pruned, g_freed, g_free = tracer.gc_lists(rep["pruned"], rep["freed"], rep["free"])
        o_pruned, o_freed, o_free = oracle.gc(tick, threshold)
        assert np.array_equal(g_pruned, o_pruned), "frame %d: pruned sets differ" % f
        assert np.array_equal(g_freed, o_freed), "frame %d: freed sets differ" % f
        assert np.array_equal(g_free, o_free), "frame %d: free lists differ" % f
        grep = tracer.graft(tick, rec, pay)
        claims = tracer.graft_claims(grep["claimed"])
        o_claims, applied = oracle.graft(tick, rec, pay)
        assert np.array_equal(claims, o_claims), "frame %d: grafted groups differ" % f
        assert grep["applied"] == int(applied.sum())
        assert_state(tracer, oracle, "frame %d" % f)
        grafted_total += len(claims)
        pruned_total += len(g_pruned)
    assert grafted_total > 0 and pruned_total > 0


def test_stream_past_the_request_cap_matches_oracle(tracer):
    """The streaming workflow with frames that raise far more child requests than
    the queue holds (the pixel-order rule decides which are kept), over enough frames
    for a 30-frame staleness threshold to prune: per frame the trace outputs, the
    request queue, the pruned, freed, free-list and claimed groups and the whole
    block and usage arrays match the oracle; a second context that answers the
    requests on the device (svo_graft_generate) reaches the same tree frame by
    frame."""
    cap, threshold, frames = 2048, 30, 40
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=10)
    tree = scene.build_tree(8)
    budget = (len(tree.Blocks) + 7) // 8 + (1 << 14)
    dev = st.Tracer(0)
    try:
        for tr in (tracer, dev):
            tr.set_config(block_size=192, ctas_per_sm=0, max_steps=1 << 16, collect_stats=0,
                          request_order=st.REQUESTS_PIXEL)
            tr.upload(tree, block_budget=budget * 8)
            tr.init_usage_tree(1)
        oracle = po.TreeState(tree, budget)
        oracle.init_usage_tree(1)
        cams = st.camera_path(seed=3, frames=frames, width=256, height=144, MaxChildRequestId=cap)
        overflowed = pruned_total = grafted_total = 0
        for f, cam in enumerate(cams):
            tick = f + 1
            got = tracer.trace(cam)
            dev.trace(cam)
            want = po.trace_view(oracle.as_octree(), cam, usage=oracle.usage)
            for k in ("hit_index", "hit_depth", "t", "rgba"):
                assert np.array_equal(getattr(got, k), want[k]), "frame %d: %s" % (f, k)
            req, n = tracer.read_child_requests(cap=cap)
            assert n == want["n_requests"], "frame %d: requests raised" % f
            assert req.tobytes() == want["pixel_requests"][:cap].tobytes(), "frame %d: request queue" % f
            overflowed += n > cap
            rec, pay = scene.graft_payload(req)
            rep = tracer.gc(tick, threshold)
            assert dev.gc(tick, threshold) == rep, "frame %d: device-generation context's GC" % f
            g_pruned, g_freed, g_free = tracer.gc_lists(rep["pruned"], rep["freed"], rep["free"])
            o_pruned, o_freed, o_free = oracle.gc(tick, threshold)
            assert np.array_equal(g_pruned, o_pruned), "frame %d: pruned sets differ" % f
            assert np.array_equal(g_freed, o_freed), "frame %d: freed sets differ" % f
            assert np.array_equal(g_free, o_free), "frame %d: free lists differ" % f
            grep = tracer.graft(tick, rec, pay)
            o_claims, applied = oracle.graft(tick, rec, pay)
            claims = tracer.graft_claims(grep["claimed"])
            assert np.array_equal(claims, o_claims), "frame %d: grafted groups differ" % f
            assert grep["applied"] == int(applied.sum())
            drep = dev.graft_generate(tick, scene)
            assert drep == grep, "frame %d: %r vs %r" % (f, drep, grep)
            assert_state(tracer, oracle, "frame %d" % f)
            hb, hu = gpu_state(tracer, budget)
            db, du = gpu_state(dev, budget)
            assert hb.tobytes() == db.tobytes() and hu.tobytes() == du.tobytes(), "frame %d: generation paths" % f
            pruned_total += len(g_pruned)
            grafted_total += len(claims)
        assert overflowed >= frames // 2, "the frames must overflow the queue"
        assert pruned_total > 0 and grafted_total > 0
    finally:
        dev.close()
        tracer.set_config(request_order=st.REQUESTS_ARRIVAL)
        scene.close()


def test_state_checkpoint_resumes_the_stream(tracer, tmp_path):
    """Checkpoint / resume: a stream (pixel-order requests past the cap, grafts
    generated on the device, GC with a staleness threshold that prunes) saved with
    svo_state_save after frame k (its free list partly claimed by that frame's
    grafts) and loaded into a fresh context with svo_state_load goes on exactly as
    the uninterrupted stream: the same trace outputs, GC reports and graft reports
    every frame, and the same blocks and usage at the end. Missing, malformed and
    truncated state files are refused."""
    cap, threshold, frames = 2048, 6, 16
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=10)
    tree = scene.build_tree(8)
    budget = (len(tree.Blocks) + 7) // 8 + (1 << 14)
    cams = st.camera_path(seed=3, frames=frames, width=160, height=90, MaxChildRequestId=cap)
    cfg = dict(block_size=192, ctas_per_sm=0, max_steps=1 << 16, collect_stats=0, request_order=st.REQUESTS_PIXEL)
    saves = {3: str(tmp_path / "frame3.svostate"), 9: str(tmp_path / "frame9.svostate")}
    resumed = []
    try:
        tracer.set_config(**cfg)
        tracer.upload(tree, block_budget=budget * 8)
        tracer.init_usage_tree(1)
        log = []
        for f, cam in enumerate(cams):
            tick = f + 1
            got = tracer.trace(cam)
            rep = tracer.gc(tick, threshold)
            grep = tracer.graft_generate(tick, scene)
            log.append((got, rep, grep))
            if f in saves:
                assert grep["claimed"] > 0  # the saved free list is partly claimed
                tracer.save_state(saves[f])
        assert sum(r[1]["pruned"] for r in log) > 0, "the stream must prune"
        want_b, want_u = gpu_state(tracer, budget)
        for f0, path in saves.items():
            tr = st.Tracer(0)
            resumed.append(tr)
            tr.set_config(**cfg)
            tr.load_state(path)
            for f in range(f0 + 1, frames):
                tick = f + 1
                got = tr.trace(cams[f])
                for k in ("hit_index", "hit_depth", "t", "rgba"):
                    assert np.array_equal(getattr(got, k), getattr(log[f][0], k)), "resume %d, frame %d: %s" % (f0, f, k)
                assert tr.gc(tick, threshold) == log[f][1], "resume %d, frame %d: GC" % (f0, f)
                assert tr.graft_generate(tick, scene) == log[f][2], "resume %d, frame %d: grafts" % (f0, f)
            got_b, got_u = gpu_state(tr, budget)
            assert got_b.tobytes() == want_b.tobytes(), "resume %d: blocks" % f0
            assert got_u.tobytes() == want_u.tobytes(), "resume %d: usage" % f0
        with pytest.raises(st.SvoError):
            resumed[0].load_state(str(tmp_path / "missing.svostate"))
        bad = tmp_path / "bad.svostate"
        bad.write_bytes(b"SVOSTAT1" + bytes(56))
        with pytest.raises(st.SvoError):
            resumed[0].load_state(str(bad))
        data = open(saves[3], "rb").read()
        (tmp_path / "short.svostate").write_bytes(data[: len(data) // 2])
        with pytest.raises(st.SvoError):
            resumed[0].load_state(str(tmp_path / "short.svostate"))
    finally:
        for tr in resumed:
            tr.close()
        tracer.set_config(request_order=st.REQUESTS_ARRIVAL)
        scene.close()


def test_prune_matches_oracle(tracer):
    scene = st.Scene(st.SCENE_TERRAIN, seed=8, base_depth=3, depth=9)
    tree = scene.build_tree(8)
    budget = 1 << 16
    tracer.upload(tree, block_budget=budget * 8)
    tracer.init_usage_tree(5)
    oracle = po.TreeState(tree, budget)
    oracle.init_usage_tree(5)
    rng = np.random.default_rng(1)
    live = np.nonzero(oracle.usage["tick"] == 5)[0]
    n = 64
    rec = np.zeros(n, st.PRUNING_DTYPE)
    locs = rng.integers(0, 2 ** 63, size=(n, 3), dtype=np.uint64) * 2
    for i in range(n):
        kind = i % 5
        rec[i]["properties"] = [1, 0b110, 0b010, 0b1000, 0b10000][kind] | (1 if i % 7 == 0 else 0)
        if i % 3 == 0:
            rec[i]["depth"] = rng.integers(3 + 2, 9)  # Location walk
            rec[i]["address"] = i
        else:
            rec[i]["depth"] = 255
            rec[i]["address"] = int(rng.choice(live)) * 8 + int(rng.integers(0, 8))
        if kind == 4:
            rec[i]["address"] = int(rng.integers(0, st.pow_sum(3)))
        rec[i]["chunk"] = int(rng.integers(0, 65536))
        rec[i]["colour_address"] = int(rng.integers(0, 4))
        rec[i]["child_address"] = NONE
    surface = np.zeros(4, st.BLOCK_DTYPE)
    surface["child"] = NONE
    surface["colour_r"] = [10, 20, 30, 40]
    rep = tracer.prune(9, rec, surface, locs.reshape(-1))
    o_freed, o_req = oracle.prune(9, rec, surface, locs.reshape(-1))
    assert rep["freed"] == len(o_freed)
    assert_state(tracer, oracle, "prune")
    assert np.array_equal(tracer.read_bases(), oracle.bases)
    _, g_freed, _ = tracer.gc_lists(0, rep["freed"], 0)
    assert np.array_equal(g_freed, o_freed)
    assert rep["requests"] == len(o_req)


def test_malformed_records_and_no_free_groups(tracer):
    """Records a host could get wrong are skipped, never applied in part and never
    read or written out of range, as the specification says: graft records with no
    groups, a misaligned or overflowing payload range, a target past the budget or
    a Location index past the locations; payload child links outside their record
    (nulled); prune records addressing past the blocks, the base chunks or the
    locations. The tree and the reports equal the oracle's. A budget with no free
    group lets a GC free nothing new and every graft be skipped."""
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=9)
    tree = scene.build_tree(7)
    budget = (len(tree.Blocks) + 7) // 8 + 64
    tracer.upload(tree, block_budget=budget * 8)
    tracer.init_usage_tree(1)
    oracle = po.TreeState(tree, budget)
    oracle.init_usage_tree(1)
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 64, 36, 60.0, Tick=1)
    tracer.trace(cam)
    req, n = tracer.read_child_requests()
    assert n > 4
    rec, pay = scene.graft_payload(req)
    rec = rec[:6].copy()
    pay = pay.copy()
    rep = tracer.gc(2, 100)
    o_pruned, o_freed, o_free = oracle.gc(2, 100)
    assert (rep["pruned"], rep["freed"], rep["free"]) == (len(o_pruned), len(o_freed), len(o_free))
    n_pay = len(pay)
    rec[0]["graft_total_size"] = 0                           # no groups
    rec[1]["graft_data_address"] += 3                         # misaligned payload range
    rec[2]["graft_data_address"] = (n_pay // 8) * 8           # the range runs past the payload
    rec[2]["graft_total_size"] = 2
    rec[3]["graft_address"] = budget * 8 + 5                  # target past the budget
    rec[4]["depth"] = 6                                       # Location walk ...
    rec[4]["graft_address"] = 1000                            # ... with an index past the locations
    first5 = int(rec[5]["graft_data_address"])
    pay[first5]["child"] = 0x7FFFFFF0                         # a payload child link outside its record
    locs = np.zeros(6, np.uint64)
    grep = tracer.graft(2, rec, pay, locs)
    o_claims, applied = oracle.graft(2, rec, pay, locs)
    assert grep["applied"] == int(applied.sum()) and grep["skipped"] >= 5
    assert np.array_equal(tracer.graft_claims(grep["claimed"]), o_claims)
    assert_state(tracer, oracle, "malformed grafts")
    prec = np.zeros(4, st.PRUNING_DTYPE)
    prec["child_address"] = NONE
    prec[0]["properties"], prec[0]["depth"], prec[0]["address"] = 0b1000, 255, budget * 8 + 1    # node past the blocks
    prec[1]["properties"], prec[1]["depth"], prec[1]["address"] = 0b10000, 255, st.pow_sum(3) + 9  # base chunk past the bases
    prec[2]["properties"], prec[2]["depth"], prec[2]["address"] = 0b0110, 6, 50                   # Location index past the locations
    prec[3]["properties"], prec[3]["depth"], prec[3]["address"] = 1, 255, budget * 8 + 64          # cull past the blocks
    surface = np.zeros(1, st.BLOCK_DTYPE)
    surface["child"] = NONE
    rep = tracer.prune(3, prec, surface, locs)
    o_freed, o_req = oracle.prune(3, prec, surface, locs)
    assert rep["freed"] == len(o_freed) == 0 and rep["requests"] == len(o_req)
    assert_state(tracer, oracle, "malformed prunes")
    assert np.array_equal(tracer.read_bases(), oracle.bases)
    # no free group at all: a budget that is the tree itself
    full = (len(tree.Blocks) + 7) // 8
    with st.Tracer(0) as tight:
        tight.upload(tree, block_budget=full * 8)
        tight.init_usage_tree(1)
        o2 = po.TreeState(tree, full)
        o2.init_usage_tree(1)
        tight.trace(cam)
        req2, _ = tight.read_child_requests()
        rec2, pay2 = scene.graft_payload(req2)
        rep2 = tight.gc(2, 100)
        o_pruned, o_freed2, o_free = o2.gc(2, 100)
        assert rep2["pruned"] == len(o_pruned) and rep2["freed"] == len(o_freed2) and rep2["free"] == len(o_free)
        g2 = tight.graft(2, rec2, pay2)
        o_claims2, applied2 = o2.graft(2, rec2, pay2)
        assert g2["applied"] == int(applied2.sum()) and g2["claimed"] == len(o_claims2)
        assert g2["skipped"] + g2["applied"] == len(rec2)
        assert_state(tight, o2, "no free groups")


def test_graft_location_targets_and_budget(tracer):
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=9)
    tree = scene.build_tree(7)
    budget = (len(tree.Blocks) + 7) // 8 + 64  # only a few free groups beyond the tree
    tracer.upload(tree, block_budget=budget * 8)
    tracer.init_usage_tree(1)
    oracle = po.TreeState(tree, budget)
    oracle.init_usage_tree(1)
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 96, 54, 60.0, Tick=1)
    tracer.trace(cam)
    req, n = tracer.read_child_requests()
    assert n > 0
    rec, pay = scene.graft_payload(req)
    # address half of the records by Location (walk to the requesting node's depth)
    uniq = {}
    for r in po.sort_requests(req):
        uniq.setdefault(int(r["address"]), r)
    locs = []
    for i, r in enumerate(rec):
        if i % 2:
            q = uniq[int(r["graft_address"])]
            r["depth"] = q["depth"]
            r["graft_address"] = len(locs) // 3
            locs.extend(int(v) for v in q["location"])
    locs = np.array(locs, np.uint64)
    rep = tracer.gc(2, 100)
    oracle.gc(2, 100)
    grep = tracer.graft(2, rec, pay, locs)
    o_claims, applied = oracle.graft(2, rec, pay, locs)
    assert grep["skipped"] > 0  # the budget runs out
    assert grep["applied"] == int(applied.sum()) > 0
    assert np.array_equal(tracer.graft_claims(grep["claimed"]), o_claims)
    assert_state(tracer, oracle, "graft")


def test_location_grafts_deepen_the_tree_for_trace_and_gc(tracer):
    """Grafts addressed only by Location: the library records the tree's new depth
    from the records' levels and payloads, and the next trace and GC reach the
    grafted levels exactly as the oracle does."""
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=9)
    tree = scene.build_tree(7)
    budget = (len(tree.Blocks) + 7) // 8 + (1 << 14)
    tracer.upload(tree, block_budget=budget * 8)
    tracer.init_usage_tree(1)
    oracle = po.TreeState(tree, budget)
    oracle.init_usage_tree(1)
    # close enough to the terrain that the cones want two levels below the tree
    cam = st.look_at((0.4, 0.4, 0.7), (0.6, 0.6, 0.9), 96, 54, 40.0, Tick=1, MaxChildRequestId=1 << 16)
    tracer.trace(cam)
    req, n = tracer.read_child_requests()
    assert 0 < n <= 1 << 16
    rec, pay = scene.graft_payload(req)
    uniq = {}
    for r in po.sort_requests(req):
        uniq.setdefault(int(r["address"]), r)
    locs = []
    for r in rec:
        q = uniq[int(r["graft_address"])]
        r["depth"] = q["depth"]
        r["graft_address"] = len(locs) // 3
        locs.extend(int(v) for v in q["location"])
    locs = np.array(locs, np.uint64)
    tracer.gc(2, 100)
    oracle.gc(2, 100)
    grep = tracer.graft(2, rec, pay, locs)
    o_claims, applied = oracle.graft(2, rec, pay, locs)
    assert grep["applied"] == int(applied.sum()) > 0
    assert np.array_equal(tracer.graft_claims(grep["claimed"]), o_claims)
    assert_state(tracer, oracle, "graft")
    cam3 = dataclasses.replace(cam, Tick=3)
    got = tracer.trace(cam3)
    want = po.trace_view(oracle.as_octree(), cam3, usage=oracle.usage)
    assert int(want["hit_depth"].max()) == 9  # the grafted grandchildren are hit
    for k in ("hit_index", "hit_depth", "t", "rgba"):
        assert np.array_equal(getattr(got, k), want[k]), k
    rep = tracer.gc(3, 100)
    g_pruned, g_freed, g_free = tracer.gc_lists(rep["pruned"], rep["freed"], rep["free"])
    o_pruned, o_freed, o_free = oracle.gc(3, 100)
    assert np.array_equal(g_freed, o_freed) and np.array_equal(g_free, o_free)
    assert_state(tracer, oracle, "gc after the grafts")


@pytest.mark.parametrize("initial,extra_groups", [(7, 1 << 14), (6, 40)], ids=["roomy", "budget_runs_out"])
def test_graft_generate_matches_host_path(tracer, initial, extra_groups):
    """Device-side generation (svo_graft_generate) against the host path of the
    streaming workflow (read the requests back, generate the payload on the
    host, svo_graft): same reports, same claimed groups, same tree, frame by
    frame; with a small budget most jobs are skipped once it runs out."""
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=9)
    tree = scene.build_tree(initial)
    budget = len(tree.Blocks) // 8 + extra_groups
    dev = st.Tracer(0)
    try:
        for tr in (tracer, dev):
            tr.set_config(block_size=192, ctas_per_sm=0, ray_chunk=1, cadence=16, max_steps=1 << 16, collect_stats=0)
            tr.upload(tree, block_budget=budget * 8)
            tr.init_usage_tree(1)
        cams = st.camera_path(seed=3, frames=8, width=160, height=90, MaxChildRequestId=1 << 16)
        applied = skipped = 0
        for f, cam in enumerate(cams):
            tick = f + 1
            tracer.trace(cam)
            dev.trace(cam)
            req, _ = tracer.read_child_requests()
            rec, pay = scene.graft_payload(req)
            assert tracer.gc(tick, 3) == dev.gc(tick, 3)
            a = tracer.graft(tick, rec, pay)
            b = dev.graft_generate(tick, scene)
            assert a == b, "frame %d: %r vs %r" % (f, a, b)
            assert np.array_equal(tracer.graft_claims(a["claimed"]), dev.graft_claims(b["claimed"]))
            hb, hu = gpu_state(tracer, budget)
            db, du = gpu_state(dev, budget)
            assert hb.tobytes() == db.tobytes(), "frame %d: blocks differ" % f
            assert hu.tobytes() == du.tobytes(), "frame %d: usage differs" % f
            applied += a["applied"]
            skipped += a["skipped"]
        assert applied > 0
        if extra_groups < 100:
            assert skipped > 0
    finally:
        dev.close()


def test_graft_generate_needs_terrain(tracer):
    scene = st.Scene(st.SCENE_SPHERE, seed=1, base_depth=2, depth=6)
    tracer.upload(scene.build_tree(5))
    with pytest.raises(st.SvoError):
        tracer.graft_generate(1, scene)


def test_graft_generate_edge_cases(tracer):
    """Without child requests there is nothing to graft; a tick outside 1..65533 is
    refused."""
    scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=2, depth=7)
    tree = scene.build_tree(5)
    with st.Tracer(0) as fresh:  # no trace yet: no request queue
        fresh.upload(tree, block_budget=(len(tree.Blocks) // 8 + 64) * 8)
        rep = fresh.graft_generate(1, scene)
        assert rep["applied"] == 0 and rep["claimed"] == 0
        with pytest.raises(st.SvoError):
            fresh.graft_generate(0, scene)
        with pytest.raises(st.SvoError):
            fresh.graft_generate(65534, scene)
        # a view of the sky only raises no requests
        fresh.trace(st.look_at((0.5, 0.5, -2.0), (0.5, 0.5, -3.0), 16, 16, 30.0, MaxChildRequestId=64))
        assert fresh.read_child_requests()[1] == 0
        rep = fresh.graft_generate(2, scene)
        assert rep["applied"] == 0 and rep["claimed"] == 0
