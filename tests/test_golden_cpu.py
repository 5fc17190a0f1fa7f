"""The oracle against the committed golden fixtures (generated from the reference's
own kernels by tests/golden/make_golden.py)."""
import glob
import os

import numpy as np
import pytest

import pyoracle as po
import svo_tracer as st

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def load_case(path):
    z = np.load(path)
    tree = st.Octree(int(z["base_depth"]), int(z["block_count"]), z["bases"], z["blocks"].view(st.BLOCK_DTYPE))
    raw = z["trace_input"].tobytes()
    c = st.TraceInputC.from_buffer_copy(raw)
    cam = st.TraceInput(Origin=tuple(c.origin), Facing=tuple(c.facing), FoV=tuple(c.fov), DoF=tuple(c.dof),
                        ScreenSize=tuple(c.screen_size), MaxOpacity=c.max_opacity, BaseDepth=c.base_depth,
                        Tick=c.tick, MaxChildRequestId=c.max_child_request_id, FovMultiplier=c.fov_multiplier,
                        FovConstant=c.fov_constant, WeightingMultiplier=c.weighting_multiplier,
                        WeightingConstant=c.weighting_constant, AmbientLightLevel=c.ambient_light_level)
    assert cam.to_bytes() == raw
    return tree, cam, z


def test_fixtures_present():
    assert len(GOLDEN) >= 4


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_golden(path):
    tree, cam, z = load_case(path)
    usage = po.init_usage(tree)
    out = po.trace_view(tree, cam, usage=usage)
    for k in ("hit_index", "hit_depth", "t", "rgba", "acc"):
        assert np.array_equal(out[k], z[k]), k
    assert np.array_equal(usage["tick"], z["usage_tick"])
    assert out["n_requests"] == int(z["n_requests"])
    same = po.sort_requests(out["requests"]).view(np.uint8).reshape(-1, 40).tobytes() == z["requests"].tobytes()
    assert same, "child requests differ"
