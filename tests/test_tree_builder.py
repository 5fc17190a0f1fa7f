"""The host tree builder against TreeBuilder's rules (SvoTracer.Domain/TreeBuilder.cs)."""
import numpy as np
import pytest

import svo_tracer as st


def morton(x, y, z, bits):
    out = 0
    for i in range(bits):
        out |= ((x >> i) & 1) << (3 * i) | ((y >> i) & 1) << (3 * i + 1) | ((z >> i) & 1) << (3 * i + 2)
    return out


def can_have_children(chunk):
    return any(((chunk >> (2 * k)) & 3) == 3 for k in range(8))


@pytest.fixture(scope="module", params=[(st.SCENE_SPHERE, 2, 7), (st.SCENE_TERRAIN, 3, 7), (st.SCENE_SPHERE, 4, 8)])
def tree(request):
    scene, b, d = request.param
    return st.TreeBuilder(scene, seed=9).BuildTree(b, d), b, d


def test_base_levels(tree):
    t, b, d = tree
    assert len(t.BaseBlocks) == st.pow_sum(b)
    # a level-(d-1) base cell with geometry must have geometry in its level-d parent cell
    for lvl in range(2, b + 1):
        start, pstart = st.pow_sum(lvl - 1), st.pow_sum(lvl - 2)
        for idx in range(8 ** lvl):
            parent = t.BaseBlocks[pstart + (idx >> 3)]
            octant = idx & 7
            geo = (t.BaseBlocks[start + idx] >> 1) & 0x5555
            if geo:
                assert (parent >> (2 * octant + 1)) & 1


def test_dense_level_and_allocation_order(tree):
    """Level B+2 nodes exist exactly under air+geometry level-(B+1) cells, and the
    groups of deeper levels are taken in TreeBuilder's order: the sorted unused
    level-(B+1) slots first, then 8^(B+1), 8^(B+1)+1, ..., visiting level-B+2 nodes
    x-major and each subtree depth-first."""
    t, b, d = tree
    bl = t.Blocks
    base_start = st.pow_sum(b - 1)
    populated = []
    for pos in range(8 ** (b + 1)):
        pair = (int(t.BaseBlocks[base_start + (pos >> 3)]) >> ((pos & 7) * 2)) & 3
        populated.append(pair == 3)
    empty = [p for p in range(8 ** (b + 1)) if not populated[p]]
    queue = empty + list(range(8 ** (b + 1), 8 ** (b + 1) + (len(bl) + 7) // 8))
    seq = []

    def visit(group):
        seq.append(group)
        for i in range(8):
            if group * 8 + i >= len(bl):
                continue  # dropped by the trim to BlockCount
            c = int(bl[group * 8 + i]["child"])
            if c != st.NO_CHILD:
                assert c % 8 == 0
                visit(c // 8)

    n2 = 1 << (b + 2)
    for x in range(n2):
        for y in range(n2):
            for z in range(n2):
                a = morton(x, y, z, b + 2)
                if not populated[a >> 3]:
                    continue
                node = bl[a]
                if d > b + 2 and can_have_children(int(node["chunk"])):
                    assert int(node["child"]) != st.NO_CHILD
                    visit(int(node["child"]) // 8)
                else:
                    assert int(node["child"]) == st.NO_CHILD
    assert seq == queue[: len(seq)]


def test_blocks_trimmed_to_block_count(tree):
    """BuildTree ends with Blocks = Blocks.Take(BlockCount) (TreeBuilder.cs:144-145)."""
    t, b, d = tree
    assert len(t.Blocks) == t.BlockCount


def test_check_tree(tree):
    """TreeBuilder.checkTree (TreeBuilder.cs:344-396): below any node, an octant that is
    not pure air must not have an all-air child."""
    t, b, d = tree
    bl = t.Blocks
    for a in np.nonzero((bl["child"] != st.NO_CHILD) & (bl["chunk"] != 0))[0][:20000]:
        c = int(bl[a]["child"])
        for k in range(8):
            if ((int(bl[a]["chunk"]) >> (2 * k)) & 3) != 1 and c + k < len(bl):
                assert int(bl[c + k]["chunk"]) != 0x5555


def test_deterministic_and_thread_independent():
    a = st.TreeBuilder(st.SCENE_TERRAIN, seed=4, threads=1).BuildTree(3, 7)
    b = st.TreeBuilder(st.SCENE_TERRAIN, seed=4, threads=8).BuildTree(3, 7)
    assert a.BlockCount == b.BlockCount
    assert np.array_equal(a.BaseBlocks, b.BaseBlocks)
    same = a.Blocks.tobytes() == b.Blocks.tobytes()
    assert same, "blocks differ"


def test_budget_and_argument_errors():
    with pytest.raises(st.SvoError):
        st.TreeBuilder(st.SCENE_SPHERE).BuildTree(4, 5)  # max_depth < base_depth + 2
    with pytest.raises(st.SvoError) as e:
        st.TreeBuilder(st.SCENE_TERRAIN, seed=1).BuildTree(2, 8, maxSize=1 << 12)
    assert "Budget" in str(e.value)
