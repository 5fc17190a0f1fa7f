"""The tree-update oracle (oracle/svo_tree_oracle.c) against the invariants of its
specification, on CPU: usage initialisation, block GC, grafting and pruning."""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

NONE = 0xFFFFFFFF


def dense_real(state, g):
    if g >= 8 ** (state.B + 1):
        return False
    chunk = int(state.bases[st.pow_sum(state.B - 1) + (g >> 3)])
    return ((chunk >> ((g & 7) * 2)) & 3) == 3


def reachable(state):
    """Allocatable groups reachable from the dense-real groups (Python BFS)."""
    n = state.n_groups
    seen = np.zeros(n, bool)
    frontier = [g for g in range(min(n, 8 ** (state.B + 1))) if dense_real(state, g)]
    child = state.blocks["child"]
    while frontier:
        nxt = []
        for g in frontier:
            for c in child[g * 8: g * 8 + 8]:
                c = int(c)
                if c == NONE or c % 8:
                    continue
                h = c // 8
                if h < n and not dense_real(state, h) and not seen[h]:
                    seen[h] = True
                    nxt.append(h)
        frontier = nxt
    return seen


@pytest.fixture(scope="module")
def scene():
    return st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=2, depth=8)


def test_init_usage_tree(scene):
    tree = scene.build_tree(6)
    s = po.TreeState(tree, 1 << 13)
    s.init_usage_tree(7)
    reach = reachable(s)
    for g in range(s.n_groups):
        u = s.usage[g]
        if dense_real(s, g):
            assert u["tick"] == 65535
        elif reach[g]:
            assert u["tick"] == 7 and s.blocks[u["parent"]]["child"] == g * 8
        else:
            assert u["tick"] == 0 and u["parent"] == NONE


def test_gc_frees_stale_subtrees_and_lists_free_groups(scene):
    tree = scene.build_tree(7)
    s = po.TreeState(tree, 1 << 14)
    s.init_usage_tree(1)
    reach0 = reachable(s)
    # refresh all but a few subtrees: their roots and descendants keep tick 1
    alloc = np.nonzero(reach0)[0]
    rng = np.random.default_rng(0)
    stale_roots = set(rng.choice(alloc, 5, replace=False).tolist())
    s.usage["tick"][alloc] = 40
    for g in stale_roots:
        s.usage["tick"][g] = 1
    pruned, freed, free = s.gc(40, 30)
    assert set(pruned.tolist()) == stale_roots
    reach1 = reachable(s)
    assert not reach1[list(stale_roots)].any()
    assert set(freed.tolist()) == set(np.nonzero(reach0 & ~reach1)[0].tolist())
    assert np.all(np.diff(free) > 0)
    assert not reach1[free].any()
    assert (s.usage["tick"][free] == 0).all()
    for g in stale_roots:
        assert s.usage["tick"][g] == 0


def test_graft_links_payload_subtrees(scene):
    tree = scene.build_tree(6)
    s = po.TreeState(tree, 1 << 14)
    s.init_usage_tree(3)
    s.gc(3, 10)
    cam = st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 64, 36, 60.0, Tick=3)
    out = po.trace_view(s.as_octree(), cam, usage=s.usage)
    assert out["n_requests"] > 0
    rec, pay = scene.graft_payload(out["requests"])
    assert len(rec) > 0 and np.all(np.diff(rec["graft_address"].astype(np.int64)) > 0)
    claimed, applied = s.graft(4, rec, pay)
    assert applied.all() and len(claimed) == rec["graft_total_size"].sum()
    reach = reachable(s)
    assert reach[claimed].all()
    k = 0
    for r in rec:
        g0 = claimed[k]
        assert s.blocks[r["graft_address"]]["child"] == g0 * 8
        assert s.usage[g0]["parent"] == r["graft_address"] and s.usage[g0]["tick"] == 4
        p0 = r["graft_data_address"]
        for i in range(8):
            want, got = pay[p0 + i], s.blocks[g0 * 8 + i]
            assert want["chunk"] == got["chunk"] and want["colour_r"] == got["colour_r"]
        k += int(r["graft_total_size"])


def test_prune_records(scene):
    tree = scene.build_tree(7)
    s = po.TreeState(tree, 1 << 14)
    s.init_usage_tree(2)
    reach0 = reachable(s)
    parents = [int(s.usage[g]["parent"]) for g in np.nonzero(reach0)[0][:3]]
    rec = np.zeros(4, st.PRUNING_DTYPE)
    rec[0]["properties"] = 1  # CullChild
    rec[0]["depth"] = 255
    rec[0]["address"] = parents[0]
    rec[0]["child_address"] = NONE
    rec[1]["properties"] = 0b110  # make inviolate
    rec[1]["depth"] = 255
    rec[1]["address"] = parents[1]
    rec[2]["properties"] = 0b1000  # overwrite node and chunk
    rec[2]["depth"] = 255
    rec[2]["address"] = parents[2]
    rec[2]["chunk"] = 0x5555
    rec[2]["colour_address"] = 0
    rec[3]["properties"] = 0b10000  # base chunk
    rec[3]["address"] = 3
    rec[3]["chunk"] = 0x1234
    surface = np.zeros(1, st.BLOCK_DTYPE)
    surface[0]["child"] = NONE
    surface[0]["colour_r"] = 200
    freed, req = s.prune(9, rec, surface)
    assert s.blocks[parents[0]]["child"] == NONE
    assert len(freed) > 0 and not reachable(s)[freed].any()
    assert s.usage[parents[1] >> 3]["tick"] == 65535
    assert s.blocks[parents[2]]["chunk"] == 0x5555 and s.blocks[parents[2]]["colour_r"] == 200
    assert s.bases[3] == 0x1234
