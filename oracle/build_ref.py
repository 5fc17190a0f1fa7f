"""Build recipe for oracle/_ref: the reference's own OpenCL kernels compiled for the CPU.

TEST INFRASTRUCTURE ONLY. Reads SvoTracer/SvoTracer.Kernel/wavefront.cl from the
reference checkout, applies two mechanical syntax rewrites that C needs and writes
the result to oracle/_ref/wavefront_ref.c:

* OpenCL vector literals ``(float3)(a, b, c)`` become GCC compound literals
  ``((float3){a, b, c})``;
* component access ``.x .y .z .w`` becomes ``[0] [1] [2] [3]`` (wavefront.cl has no
  swizzles and no struct member named x, y, z or w);
* the kernels' ``local uint localQueue[5];`` gets a zero initialiser. ``increment``
  (wavefront.cl:254-258) relies on work-items 0..4 of a group to clear the five
  entries; the harness runs one work-item per group, which would clear only entry 0.

Nothing else in the kernel source changes. ref_shim.h supplies the OpenCL types and
built-ins, ref_harness.c drives the kernels the way SvoTracer.Window/MainWindow.cs
does, and gcc links the three into oracle/_ref/libsvo_ref.so.

The rewritten source stays in oracle/_ref/ (git-ignored), so a machine without the
reference checkout can still compile it with ``compile_ref()``.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REF_SOURCE = os.environ.get(
    "SVO_REFERENCE_WAVEFRONT",
    "/root/reference/SvoTracer/SvoTracer.Kernel/wavefront.cl",
)
REWRITTEN = os.path.join(REF_DIR, "wavefront_ref.c")
REF_LIB = os.path.join(REF_DIR, "libsvo_ref.so")

_VEC = re.compile(r"\((float|int|uint|ulong|uchar|ushort|long|short|char)([234])\)\(")


def _rewrite_literals(src: str) -> str:
    out = []
    i = 0
    while True:
        m = _VEC.search(src, i)
        if not m:
            out.append(src[i:])
            break
        out.append(src[i : m.start()])
        # find the matching close paren of the literal's argument list
        depth = 1
        j = m.end()
        while depth:
            c = src[j]
            if c == "(":
                depth += 1
            elif c == ")":
                depth -= 1
            j += 1
        inner = _rewrite_literals(src[m.end() : j - 1])
        out.append("((%s%s){%s})" % (m.group(1), m.group(2), inner))
        i = j
    return "".join(out)


def rewrite(src: str) -> str:
    src = _rewrite_literals(src)
    src = src.replace("local uint localQueue[5];", "local uint localQueue[5] = {0, 0, 0, 0, 0};")
    src = re.sub(r"\.([xyzw])\b", lambda m: "[%d]" % "xyzw".index(m.group(1)), src)
    return src


def generate() -> bool:
    """Write oracle/_ref/wavefront_ref.c from the reference checkout, if present."""
    if not os.path.exists(REF_SOURCE):
        return os.path.exists(REWRITTEN)
    os.makedirs(REF_DIR, exist_ok=True)
    with open(REF_SOURCE, "r", encoding="utf-8-sig") as f:
        src = f.read()
    text = (
        "/* Generated by oracle/build_ref.py from the reference's wavefront.cl: "
        "vector literals and component access rewritten for C. */\n" + rewrite(src)
    )
    if not os.path.exists(REWRITTEN) or open(REWRITTEN).read() != text:
        with open(REWRITTEN, "w") as f:
            f.write(text)
    return True


def compile_ref(cc: str = "gcc") -> str | None:
    """Compile libsvo_ref.so; returns its path or None when the source is absent."""
    if not generate():
        return None
    deps = [REWRITTEN, os.path.join(HERE, "ref_harness.c"), os.path.join(HERE, "ref_shim.h")]
    if os.path.exists(REF_LIB) and all(os.path.getmtime(REF_LIB) >= os.path.getmtime(d) for d in deps):
        return REF_LIB
    cmd = [
        cc, "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
        "-fopenmp", "-w", "-Wno-psabi", "-include", os.path.join(HERE, "ref_shim.h"),
        os.path.join(HERE, "ref_harness.c"), "-o", REF_LIB + ".tmp", "-lm",
    ]
    subprocess.run(cmd, check=True, cwd=REF_DIR)
    os.replace(REF_LIB + ".tmp", REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    p = compile_ref()
    print(p if p else "reference source not available")
    sys.exit(0)
