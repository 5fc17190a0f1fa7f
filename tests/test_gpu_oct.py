"""A tree saved to and loaded from a .oct file traces bit-exactly like the oracle
(TreeManager.SaveTree / LoadTree, then InitReadBuffer and RunWavefront)."""
import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(tracer):
    tracer.set_config(block_size=192, ctas_per_sm=0, ray_chunk=1, cadence=16, max_steps=1 << 16, collect_stats=0)
    yield


def test_trace_of_loaded_tree_matches_oracle(tracer, tmp_path):
    tm = st.TreeManager(str(tmp_path))
    tm.SaveTree("terrain", st.TreeBuilder(st.SCENE_TERRAIN, seed=6).BuildTree(3, 8))
    tree = tm.LoadTree("terrain")
    tracer.upload(tree)
    tracer.init_usage()
    cam = st.look_at((0.1, 0.2, 0.6), (0.8, 0.7, 0.9), 200, 120, 60.0, Tick=3, MaxChildRequestId=1 << 14)
    got = tracer.trace(cam)
    usage = po.init_usage(tree)
    want = po.trace_view(tree, cam, usage=usage)
    for k in ("hit_index", "hit_depth", "t", "rgba"):
        assert np.array_equal(getattr(got, k), want[k]), k
    assert (got.hit_index != 0xFFFFFFFF).sum() > 1000
    assert np.array_equal(tracer.read_usage(len(usage))["tick"], usage["tick"])
