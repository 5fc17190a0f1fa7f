"""The .oct tree file (OctreeSerializer / BlockSerializer / TreeManager of
SvoTracer.Domain) through the C ABI: byte layout, round trips, the reader's
BlockCount semantics and error reporting."""
import os
import struct

import numpy as np
import pytest

import svo_tracer as st


def handmade_tree():
    bases = np.arange(8, dtype=np.uint16) * 4097  # powSum(1) = 8 chunks
    blocks = np.zeros(3, st.BLOCK_DTYPE)
    blocks["child"] = [0xFFFFFFFF, 16, 0x01020304]
    blocks["chunk"] = [0xAAAA, 0x5555, 0x1234]
    blocks["normal_pitch"] = [-1, 300, -32768]
    blocks["normal_yaw"] = [7, -2, 32767]
    for k, name in enumerate(("colour_r", "colour_g", "colour_b", "opacity", "specularity", "gloss")):
        blocks[name] = [k + 1, 100 + k, 250 - k]
    return st.Octree(1, 3, bases, blocks)


def reference_bytes(tree, block_count=None):
    """The byte stream OctreeSerializer.Serialize writes, field by field."""
    out = struct.pack("<BI", tree.BaseDepth, tree.BlockCount if block_count is None else block_count)
    out += struct.pack("<%dH" % len(tree.BaseBlocks), *[int(b) for b in tree.BaseBlocks])
    for b in tree.Blocks:
        out += struct.pack("<IHhhBBBBBB", int(b["child"]), int(b["chunk"]), int(b["normal_pitch"]),
                           int(b["normal_yaw"]), int(b["colour_r"]), int(b["colour_g"]), int(b["colour_b"]),
                           int(b["opacity"]), int(b["specularity"]), int(b["gloss"]))
    return out


def same_tree(a, b):
    return (a.BaseDepth == b.BaseDepth and a.BlockCount == b.BlockCount and np.array_equal(a.BaseBlocks, b.BaseBlocks)
            and a.Blocks.tobytes() == b.Blocks.tobytes())


def test_byte_layout_matches_serializer(tmp_path):
    tree = handmade_tree()
    path = str(tmp_path / "t.oct")
    st.write_oct(path, tree)
    with open(path, "rb") as f:
        data = f.read()
    assert data == reference_bytes(tree)
    assert same_tree(st.read_oct(path), tree)


@pytest.mark.parametrize("scene,base,depth", [(st.SCENE_SPHERE, 2, 6), (st.SCENE_TERRAIN, 3, 7)])
def test_round_trip_of_built_trees(tmp_path, scene, base, depth):
    tree = st.TreeBuilder(scene, seed=4).BuildTree(base, depth)
    path = str(tmp_path / "t.oct")
    st.write_oct(path, tree)
    assert os.path.getsize(path) == 5 + 2 * st.pow_sum(base) + 16 * len(tree.Blocks)
    back = st.read_oct(path)
    assert back.BaseDepth == base and back.BlockCount == tree.BlockCount
    assert np.array_equal(back.BaseBlocks, tree.BaseBlocks)
    # the reader takes BlockCount blocks, like OctreeSerializer.Deserialize
    n = min(tree.BlockCount, len(tree.Blocks))
    assert back.Blocks.tobytes() == tree.Blocks[:n].tobytes()


def test_reader_takes_block_count_blocks(tmp_path):
    tree = handmade_tree()
    path = str(tmp_path / "t.oct")
    with open(path, "wb") as f:
        f.write(reference_bytes(tree, block_count=2))  # three blocks follow, the header says two
    back = st.read_oct(path)
    assert back.BlockCount == 2 and back.Blocks.tobytes() == tree.Blocks[:2].tobytes()


def test_errors(tmp_path):
    with pytest.raises(st.SvoError):
        st.read_oct(str(tmp_path / "missing.oct"))
    data = reference_bytes(handmade_tree())
    short = tmp_path / "short.oct"
    short.write_bytes(data[:-1])
    with pytest.raises(st.SvoError):
        st.read_oct(str(short))
    deep = tmp_path / "deep.oct"
    deep.write_bytes(struct.pack("<BI", 12, 0))
    with pytest.raises(st.SvoError):
        st.read_oct(str(deep))
    bad = handmade_tree()
    bad.BaseBlocks = bad.BaseBlocks[:5]
    with pytest.raises(st.SvoError):
        st.write_oct(str(tmp_path / "bad.oct"), bad)


def test_tree_manager(tmp_path):
    tm = st.TreeManager(str(tmp_path / "trees"))
    tree = st.TreeBuilder(st.SCENE_SPHERE, seed=2).BuildTree(2, 5)
    assert not tm.TreeExists("sphere")
    tm.SaveTree("sphere", tree)
    assert tm.TreeExists("sphere")
    back = tm.LoadTree("sphere")
    assert back.Blocks.tobytes() == tree.Blocks[:back.BlockCount].tobytes()
    tm.DeleteTree("sphere")
    assert not tm.TreeExists("sphere")


def test_numpy_mapping_equals_the_library_reader(tmp_path):
    """map_oct (numpy alone, as the benchmark's reference arm reads its scene) gives
    the same tree as the library's svo_oct_read."""
    tree = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(3, 7)
    path = str(tmp_path / "t.oct")
    st.write_oct(path, tree)
    a, b = st.read_oct(path), st.map_oct(path)
    assert (a.BaseDepth, a.BlockCount) == (b.BaseDepth, b.BlockCount)
    assert np.array_equal(a.BaseBlocks, b.BaseBlocks)
    assert a.Blocks.tobytes() == np.asarray(b.Blocks).tobytes()
    with open(path, "r+b") as f:
        f.truncate(100)
    with pytest.raises(st.SvoError):
        st.map_oct(path)
