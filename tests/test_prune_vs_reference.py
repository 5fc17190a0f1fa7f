"""The tree-update specification's prune (oracle/svo_tree_oracle.c, which the CUDA
prune is tested against bit for bit) against the reference's own prune kernel
(wavefront.cl:1215-1266, compiled for the CPU) on the same tree and records.

The reference kernel runs one work-item at a time in record order (ref_prune in
oracle/ref_harness.c). Every record kind it can run faithfully is covered, by
direct and by Location addressing: base chunks (bit 4), usage stamps (bits 1-2 =
01), inviolate (11), node overwrites (bit 3) and CullChild (bit 0). The bases,
every node and every usage entry must agree, except where the specification
departs from the reference on purpose; each such departure has its own test:

* CullChild frees the groups it orphans. The reference's dereference leaves the
  culled child group itself allocated (it queues only the grandchildren,
  wavefront.cl:1176-1186), and its queue pops one slot past the last push, so a
  deeper subtree cannot be freed by it at all (the harness refuses those records).
* A Location walk that meets a missing child raises a child request. The
  reference's findAddress calls requestChild through an uninitialised Buffers
  (wavefront.cl:1203-1204): the harness refuses those records.
"""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.skipif(not po.ref_available(), reason="reference kernels not available")
NONE = 0xFFFFFFFF
B = 3


@pytest.fixture(scope="module")
def tree():
    return st.TreeBuilder(st.SCENE_TERRAIN, seed=8).BuildTree(B, 8)


def _states(tree, tick=5):
    spec = po.TreeState(tree, (len(tree.Blocks) + 7) // 8 + 64)
    spec.init_usage_tree(tick)
    ref = (spec.bases.copy(), spec.blocks.copy(), spec.usage.copy())
    return spec, ref


def _octant_bits(loc, level, k):
    s = 63 - level
    for axis in range(3):
        if (k >> axis) & 1:
            loc[axis] |= 1 << s


def _random_path(rng, blocks, depth):
    """A Location whose walk from level B+2 reaches a node at `depth` (every node on
    the way has children); returns (location words, node address) or None."""
    dense = 8 ** (B + 2)
    for _ in range(200):
        a = int(rng.integers(0, dense))
        loc = [int(rng.integers(0, 2 ** 62)) & ~((2 ** 64 - 1) << (64 - depth) & (2 ** 64 - 1)) for _ in range(3)]
        for i in range(B + 2):  # the octal digits of the dense address are the octants of levels 0..B+1
            _octant_bits(loc, i, (a >> (3 * (B + 1 - i))) & 7)
        ok = True
        for level in range(B + 2, depth):
            c = int(blocks[a]["child"])
            if c == NONE:
                ok = False
                break
            k = int(rng.integers(0, 8))
            _octant_bits(loc, level, k)
            a = c + k
        if ok:
            return np.array(loc, np.uint64), a
    return None


def _leaf_group_parents(blocks, usage, live_tick):
    """Nodes of live groups whose child group has no grandchildren."""
    out = []
    for node in np.nonzero(blocks["child"] != NONE)[0]:
        c = int(blocks[node]["child"])
        if c + 8 > len(blocks) or usage[node >> 3]["tick"] != live_tick:
            continue
        if (blocks[c:c + 8]["child"] == NONE).all():
            out.append(int(node))
    return out


def _records(rng, tree, spec, n=240, tick=5):
    blocks, usage = spec.blocks, spec.usage
    live = np.nonzero(usage["tick"] == tick)[0]
    leaf_nodes = [int(g) * 8 + i for g in live[:4000] for i in range(8) if blocks[int(g) * 8 + i]["child"] == NONE]
    cullable = _leaf_group_parents(blocks, usage, tick)
    free = np.nonzero(usage["tick"] == 0)[0]
    rec = np.zeros(n, st.PRUNING_DTYPE)
    locs = []
    surface = np.zeros(16, st.BLOCK_DTYPE)
    surface["child"] = NONE
    surface["colour_r"] = np.arange(16) * 7
    surface["opacity"] = 200
    culled = set()
    for i in range(n):
        kind = i % 8
        r = rec[i]
        r["depth"] = 255
        r["child_address"] = NONE
        r["chunk"] = int(rng.integers(0, 65536))
        r["colour_address"] = int(rng.integers(0, len(surface)))
        if kind == 0:  # base chunk of levels 1..B-1 (level B decides which dense groups are real)
            r["properties"] = 0b10000
            r["address"] = int(rng.integers(0, st.pow_sum(B - 1)))
        elif kind in (1, 2):  # stamp / inviolate, direct
            r["properties"] = 0b010 if kind == 1 else 0b110
            r["address"] = int(rng.choice(live)) * 8 + int(rng.integers(0, 8))
        elif kind == 3:  # overwrite a leaf node (no child is orphaned)
            r["properties"] = 0b1000
            r["address"] = int(rng.choice(leaf_nodes))
        elif kind in (4, 5):  # by Location: stamp, or overwrite a leaf node the walk reaches
            path = None
            while path is None:
                depth = int(rng.integers(B + 3, 9))
                path = _random_path(rng, blocks, depth)
            loc, node = path
            r["properties"] = 0b010 if kind == 4 or blocks[node]["child"] != NONE else 0b1010
            r["depth"] = depth
            r["address"] = len(locs)
            locs.append(loc)
        elif kind == 6:  # CullChild of a node whose children are leaves
            cand = [c for c in cullable if c not in culled and (blocks[c]["child"] >> 3) not in culled]
            node = int(rng.choice(cand))
            culled.add(node)
            culled.add(int(blocks[node]["child"]) >> 3)
            r["properties"] = 0b1
            r["address"] = node
        else:  # a node of a free group: the kernel returns (dereferenced)
            r["properties"] = 0b010
            r["address"] = int(rng.choice(free)) * 8 if len(free) else int(rng.choice(live)) * 8
    return rec, surface, np.array(locs, np.uint64).reshape(-1)


def test_prune_spec_matches_reference_prune(tree):
    spec, (r_bases, r_blocks, r_usage) = _states(tree)
    rng = np.random.default_rng(3)
    rec, surface, locs = _records(rng, tree, spec)
    before = spec.usage.copy()
    ran = po.ref_prune(r_bases, B, r_blocks, r_usage, rec, surface, locs, tick=9)
    assert ran == len(rec), "the reference harness refused record %d" % (-ran - 1)
    freed, req = spec.prune(9, rec, surface, locs)
    assert len(req) == 0
    assert np.array_equal(spec.bases, r_bases)
    assert spec.blocks.tobytes() == r_blocks.tobytes()
    # every usage entry agrees except the culled child groups: the specification
    # frees them, the reference leaves them allocated with their old tick
    diff = np.nonzero(spec.usage.view(np.uint64) != r_usage.view(np.uint64))[0]
    assert set(diff.tolist()) == set(freed.tolist())
    n_cull = int((rec["properties"] & 1).sum())
    assert len(freed) == n_cull > 0
    assert (spec.usage[freed]["tick"] == 0).all() and (spec.usage[freed]["parent"] == NONE).all()
    assert np.array_equal(r_usage[freed], before[freed])
    # the sequence exercised every kind: stamps, inviolate groups, overwritten nodes, base chunks
    assert (r_usage["tick"] == 9).sum() > 0 and (r_usage["tick"] == 65535).sum() > (before["tick"] == 65535).sum()


@pytest.mark.parametrize("kind", ["base", "stamp", "inviolate", "overwrite", "cull", "location", "free"])
def test_each_record_kind_alone_matches(tree, kind):
    spec, (r_bases, r_blocks, r_usage) = _states(tree)
    rng = np.random.default_rng(11)
    rec, surface, locs = _records(rng, tree, spec, n=64)
    pick = {"base": 0, "stamp": 1, "inviolate": 2, "overwrite": 3, "location": 4, "cull": 6, "free": 7}[kind]
    one = rec[pick::8][:4].copy()
    ran = po.ref_prune(r_bases, B, r_blocks, r_usage, one, surface, locs, tick=9)
    assert ran == len(one)
    freed, _ = spec.prune(9, one, surface, locs)
    assert np.array_equal(spec.bases, r_bases)
    assert spec.blocks.tobytes() == r_blocks.tobytes()
    diff = np.nonzero(spec.usage.view(np.uint64) != r_usage.view(np.uint64))[0]
    assert set(diff.tolist()) == set(freed.tolist())


def test_level_b_base_chunk_decides_which_dense_groups_are_real(tree):
    """A level-B base chunk that makes a cell solid (geometry, no air) leaves its
    level-(B+2) groups out of the tree: the reference only writes the chunk, the
    specification's sweep after a CullChild in the same call also frees the
    subtrees that hung below them."""
    spec, (r_bases, r_blocks, r_usage) = _states(tree)
    first_b = st.pow_sum(B - 1)
    dense_groups = 8 ** (B + 1)
    # a level-B chunk with an air+geometry child cell whose dense group has children
    target = None
    for i in range(st.pow_sum(B) - first_b):
        chunk = int(spec.bases[first_b + i])
        for k in range(8):
            g = i * 8 + k
            if g < dense_groups and (chunk >> (2 * k)) & 3 == 3 and (spec.blocks[g * 8:g * 8 + 8]["child"] != NONE).any():
                target = (first_b + i, k, g)
                break
        if target:
            break
    assert target
    index, k, g = target
    solid = int(spec.bases[index]) & ~(1 << (2 * k))  # clear the air bit of cell k
    rec = np.zeros(2, st.PRUNING_DTYPE)
    rec[0]["properties"] = 0b10000
    rec[0]["depth"] = 255
    rec[0]["address"] = index
    rec[0]["chunk"] = solid
    cull = _leaf_group_parents(spec.blocks, spec.usage, 5)[0]  # any cull runs the sweep
    rec[1]["properties"] = 1
    rec[1]["depth"] = 255
    rec[1]["address"] = cull
    rec[1]["child_address"] = NONE
    assert po.ref_prune(r_bases, B, r_blocks, r_usage, rec, tick=9) == 2
    freed, _ = spec.prune(9, rec)
    assert np.array_equal(spec.bases, r_bases) and spec.blocks.tobytes() == r_blocks.tobytes()
    below = {int(c) >> 3 for c in spec.blocks[g * 8:g * 8 + 8]["child"] if c != NONE}
    assert below <= set(freed.tolist())  # the groups below the now-solid cell's dense group
    assert (r_usage[list(below)]["tick"] != 0).all()  # the reference keeps them


def test_cull_of_a_deeper_subtree_frees_the_whole_subtree(tree):
    """The reference cannot run this record faithfully (its dereference queue would
    pop an unwritten slot); the specification frees every group below the cut."""
    spec, (r_bases, r_blocks, r_usage) = _states(tree)
    blocks = spec.blocks
    node = None
    for g in range(8 ** (B + 1) // 8 * 8, len(spec.usage)):
        for i in range(8):
            c = int(blocks[g * 8 + i]["child"])
            if c != NONE and (blocks[c:c + 8]["child"] != NONE).any() and spec.usage[g]["tick"] == 5:
                node = g * 8 + i
                break
        if node is not None:
            break
    assert node is not None
    subtree, stack = set(), [int(blocks[node]["child"]) >> 3]
    while stack:
        g = stack.pop()
        if g in subtree:
            continue
        subtree.add(g)
        for c in blocks[g * 8:g * 8 + 8]["child"]:
            if c != NONE:
                stack.append(int(c) >> 3)
    rec = np.zeros(1, st.PRUNING_DTYPE)
    rec[0]["properties"] = 1
    rec[0]["depth"] = 255
    rec[0]["address"] = node
    rec[0]["child_address"] = NONE
    assert po.ref_prune(r_bases, B, r_blocks, r_usage, rec, tick=9) == -1
    freed, _ = spec.prune(9, rec)
    assert set(freed.tolist()) == subtree and len(subtree) > 1
    assert spec.blocks[node]["child"] == NONE


def test_location_walk_to_a_missing_child_raises_a_request(tree):
    """The reference's findAddress would write the request through an uninitialised
    buffer set (the harness refuses the record); the specification queues it with
    the walk's depth, the frame's tick and the remaining levels as TreeSize."""
    spec, (r_bases, r_blocks, r_usage) = _states(tree)
    rng = np.random.default_rng(5)
    blocks = spec.blocks
    for _ in range(500):
        loc = rng.integers(0, 2 ** 63, size=3, dtype=np.uint64) * np.uint64(2)
        a = 0
        for i in range(B + 2):
            s = 63 - i
            a = a * 8 + int(((int(loc[0]) >> s) & 1) | (((int(loc[1]) >> s) & 1) << 1) | (((int(loc[2]) >> s) & 1) << 2))
        d = B + 2
        while blocks[a]["child"] != NONE and d < 12:
            s = 63 - d
            a = int(blocks[a]["child"]) + (((int(loc[0]) >> s) & 1) | (((int(loc[1]) >> s) & 1) << 1) |
                                           (((int(loc[2]) >> s) & 1) << 2))
            d += 1
        if d < 12 and d > B + 2:
            break
    rec = np.zeros(1, st.PRUNING_DTYPE)
    rec[0]["properties"] = 0b010
    rec[0]["depth"] = d + 2
    rec[0]["address"] = 0
    assert po.ref_prune(r_bases, B, r_blocks, r_usage, rec, locations=loc, tick=9) == -1
    freed, req = spec.prune(9, rec, locations=loc)
    assert len(freed) == 0 and len(req) == 1
    q = req[0]
    assert q["address"] == a and q["depth"] == d and q["tick"] == 9 and q["tree_size"] == 2
    assert list(q["location"]) == [int(v) for v in loc]
