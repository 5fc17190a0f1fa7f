"""The checked build (SVO_CHECKED: every index of the step code into the path
cache, the base chunks and the per-pixel outputs checked before use; a failed
check is reported as SVO_ERR_INTERNAL and the access skipped, so an index
error shows as an error status instead of an access out of bounds). It is
compiled here into a scratch directory, runs the trace (single view and batch),
the megakernel, colour fitting and a few frames of the prune/graft/GC stream in
a child process, reports no failed check, and gives the same results as the
normal build."""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import svo_tracer as st

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "svo-tracer_gb300")

# The workloads, run with either library: returns a dict of arrays.
WORKLOADS = textwrap.dedent('''
    import hashlib
    import numpy as np

    def run(st):
        out = {}
        tr = st.Tracer(0)
        try:
            terrain = st.TreeBuilder(st.SCENE_TERRAIN, seed=5).BuildTree(3, 8)
            tr.upload(terrain)
            tr.init_usage()
            views = [st.look_at((0.1, 0.15, 0.55), (0.7, 0.7, 0.9), 160, 90, 60.0, Tick=3),
                     st.look_at((0.9, 0.2, 0.6), (0.3, 0.6, 0.9), 64, 48, 70.0, Tick=3),
                     st.look_at((1.4, 1.3, 1.2), (0.5, 0.5, 0.4), 37, 21, 50.0, Tick=3)]
            r = tr.trace(views[0])
            for k in ("hit_index", "hit_depth", "t", "rgba"):
                out["trace_" + k] = np.asarray(getattr(r, k)).copy()
            for i, r in enumerate(tr.trace_batch(views, graph=True)):
                out["batch%d_rgba" % i] = r.rgba.copy()
                out["batch%d_hit" % i] = r.hit_index.copy()
            out["usage"] = tr.read_usage()["tick"].copy()
            sphere = st.TreeBuilder(st.SCENE_SPHERE, seed=1).BuildTree(3, 8)
            tr.upload(sphere)
            tr.init_usage()
            mv = st.orbit_views(seed=5, n=1, width=64, height=48)[0]
            m = tr.mega_trace(mv)
            out["mega_rgba"] = m.rgba.copy()
            out["mega_hit"] = m.hit_index.copy()
            dviews = st.orbit_views(seed=7, n=2, width=64, height=48, distance=0.75)
            nodes = len(sphere.Blocks)
            tr.diff_set_params(np.random.default_rng(3).uniform(0, 1, (nodes, 4)).astype(np.float32))
            rgb = tr.diff_forward(dviews).copy()
            out["diff_rgb"] = rgb
            target = np.random.default_rng(4).uniform(0, 1, rgb.shape).astype(np.float32)
            out["diff_loss"] = np.array([tr.diff_backward(dviews, target)])
            out["diff_grads"] = tr.diff_grads(nodes).copy()
            scene = st.Scene(st.SCENE_TERRAIN, seed=5, base_depth=3, depth=10)
            try:
                tree = scene.build_tree(8)
                budget = (len(tree.Blocks) + 7) // 8 + (1 << 14)
                tr.set_config(request_order=st.REQUESTS_PIXEL)
                tr.upload(tree, block_budget=budget * 8)
                tr.init_usage_tree(1)
                cams = st.camera_path(seed=3, frames=4, width=160, height=90, MaxChildRequestId=2048)
                for f, cam in enumerate(cams):
                    tr.trace(cam)
                    tr.gc(f + 1, 2)
                    tr.graft_generate(f + 1, scene)
                h = hashlib.sha256(tr.read_blocks(0, budget * 8).tobytes())
                h.update(tr.read_usage(budget).tobytes())
                out["stream_state"] = np.frombuffer(h.digest(), np.uint8).copy()
            finally:
                scene.close()
        finally:
            tr.close()
        return out
''')

CHILD = textwrap.dedent('''
    import sys
    sys.path.insert(0, sys.argv[1])
    import numpy as np
    import svo_tracer as st
    st.load_library(sys.argv[2])
    ns = {}
    exec(open(sys.argv[3]).read(), ns)
    np.savez(sys.argv[4], **ns["run"](st))
''')

BUILD = textwrap.dedent('''
    import sys
    sys.path.insert(0, sys.argv[1])
    import build_native as bn
    bn.BUILD = sys.argv[2] + "/obj"
    bn.LIB_DIR = sys.argv[2]
    bn.LIB = sys.argv[2] + "/libsvo.so"
    bn.NVCC_FLAGS = bn.NVCC_FLAGS + ["-DSVO_CHECKED=1"]
    print(bn.build())
''')


def test_checked_build_matches_the_normal_build(tmp_path):
    lib_dir = str(tmp_path / "checked")
    os.makedirs(lib_dir)
    b = subprocess.run([sys.executable, "-c", BUILD, PKG, lib_dir], capture_output=True, text=True, timeout=900)
    assert b.returncode == 0, b.stdout + b.stderr
    wl = tmp_path / "workloads.py"
    wl.write_text(WORKLOADS)
    res = tmp_path / "checked.npz"
    c = subprocess.run([sys.executable, "-c", CHILD, PKG, os.path.join(lib_dir, "libsvo.so"), str(wl), str(res)],
                       capture_output=True, text=True, timeout=900)
    assert c.returncode == 0, "the checked build reported an error:\n" + c.stdout + c.stderr
    got = dict(np.load(res))
    ns = {}
    exec(WORKLOADS, ns)
    want = ns["run"](st)
    assert sorted(got) == sorted(want)
    for k in want:
        if k in ("diff_loss", "diff_grads"):  # sums of atomics: equal up to the order of the additions
            np.testing.assert_allclose(got[k], want[k], rtol=1e-5, atol=1e-9, err_msg=k)
        else:
            assert got[k].tobytes() == want[k].tobytes(), k
