"""Generates the golden fixtures in tests/golden/*.npz.

The expected outputs come from the reference's own wavefront.cl kernels compiled for
the CPU (oracle/_ref, see oracle/build_ref.py), run through the harness that drives
them like MainWindow.RunWavefront. The script also runs the C restatement
(oracle/svo_oracle.c) and refuses to write a fixture unless both agree bit for bit.

Inputs are small seeded scenes built by the library's tree builder and stored in the
fixture, so the tests do not depend on the builder. Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "svo-tracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_native  # noqa: E402
import pyoracle as po  # noqa: E402
import svo_tracer as st  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, scene, seed, base_depth, max_depth, camera (origin, target), W, H, fov, dof, tick
    ("sphere_b2_d7", st.SCENE_SPHERE, 3, 2, 7, ((1.15, 0.8, 0.05), (0.5, 0.5, 0.5)), 64, 48, 60.0, (0.0, 0.0), 5),
    ("sphere_inside_b2_d7", st.SCENE_SPHERE, 4, 2, 7, ((0.88, 0.12, 0.2), (0.5, 0.5, 0.5)), 48, 32, 80.0, (0.0, 0.0), 9),
    ("terrain_b2_d7", st.SCENE_TERRAIN, 5, 2, 7, ((0.1, 0.15, 0.55), (0.7, 0.7, 0.9)), 80, 45, 60.0, (0.0, 0.0), 2),
    ("terrain_dof_b3_d7", st.SCENE_TERRAIN, 6, 3, 7, ((0.9, 0.1, 0.5), (0.3, 0.6, 0.85)), 64, 36, 70.0, (0.02, 0.5), 7),
]


def main() -> None:
    build_native.build()
    for name, scene, seed, b, d, (o, t), w, h, fov, dof, tick in CASES:
        tree = st.TreeBuilder(scene, seed=seed).BuildTree(b, d)
        cam = st.look_at(o, t, w, h, fov, DoF=dof, Tick=tick, MaxChildRequestId=65536)
        u_ref = po.init_usage(tree)
        u_orc = u_ref.copy()
        ref = po.ref_trace_view(tree, cam, usage=u_ref)
        orc = po.trace_view(tree, cam, usage=u_orc)
        for k in ("hit_index", "hit_depth", "t", "rgba", "acc"):
            assert np.array_equal(ref[k], orc[k]), (name, k)
        assert np.array_equal(u_ref["tick"], u_orc["tick"]), name
        ra, oa = po.sort_requests(ref["requests"]), po.sort_requests(orc["requests"])
        assert ra.tobytes() == oa.tobytes(), name
        np.savez_compressed(
            os.path.join(OUT, name + ".npz"),
            base_depth=np.uint8(tree.BaseDepth), block_count=np.uint32(tree.BlockCount), bases=tree.BaseBlocks,
            blocks=tree.Blocks.view(np.uint8), trace_input=np.frombuffer(cam.to_bytes(), np.uint8),
            hit_index=ref["hit_index"], hit_depth=ref["hit_depth"], t=ref["t"], rgba=ref["rgba"], acc=ref["acc"],
            usage_tick=u_ref["tick"], requests=ra.view(np.uint8).reshape(-1, 40), n_requests=np.uint32(ref["n_requests"]),
            generator=np.array("reference wavefront.cl kernels (CPU build, oracle/_ref); oracle restatement agrees"),
        )
        print("%-22s nodes %7d hits %5d/%5d requests %d" % (name, len(tree.Blocks), int((ref["hit_index"] != st.MISS).sum()),
                                                           w * h, ref["n_requests"]))


if __name__ == "__main__":
    main()
