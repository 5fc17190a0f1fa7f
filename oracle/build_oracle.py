"""Build recipe of the oracle (TEST INFRASTRUCTURE ONLY).

Compiles oracle/svo_oracle.c (the C restatement of the reference's wavefront hot
path) into oracle/libsvo_oracle.so, and, through build_ref.py, the reference's own
wavefront.cl kernels into oracle/_ref/libsvo_ref.so and its megakernel kernel.cl into
oracle/_ref/libsvo_ref_mega.so where their rewritten sources are available. Only tests, __graft_entry__.smoke() and bench.py's CPU legs load these.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "libsvo_oracle.so")

sys.path.insert(0, HERE)
import build_ref  # noqa: E402


def build_oracle(cc: str = "gcc") -> str:
    srcs = [os.path.join(HERE, "svo_oracle.c"), os.path.join(HERE, "svo_tree_oracle.c")]
    hdr = os.path.join(HERE, "svo_oracle.h")
    api = os.path.join(os.path.dirname(HERE), "include", "svo.h")
    if os.path.exists(ORACLE_LIB) and all(os.path.getmtime(ORACLE_LIB) >= os.path.getmtime(d) for d in srcs + [hdr, api]):
        return ORACLE_LIB
    cmd = [cc, "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"] + srcs + [
        "-o", ORACLE_LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def build_all() -> dict:
    out = {"oracle": build_oracle()}
    for key, fn in (("ref", build_ref.compile_ref), ("ref_mega", build_ref.compile_ref_mega)):
        try:
            out[key] = fn()
        except subprocess.CalledProcessError as e:  # the reference harnesses are optional
            out[key] = None
            out[key + "_error"] = str(e)
    return out


if __name__ == "__main__":
    print(build_all())
