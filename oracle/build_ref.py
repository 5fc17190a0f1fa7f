"""Build recipe for oracle/_ref: the reference's own OpenCL kernels compiled for the CPU.

TEST INFRASTRUCTURE ONLY. Reads SvoTracer/SvoTracer.Kernel/wavefront.cl (and the
megakernel SvoTracer/SvoTracer.Kernel/kernel.cl) from the reference checkout,
applies mechanical syntax rewrites that C needs and writes the results to
oracle/_ref/wavefront_ref.c (and oracle/_ref/kernel_ref.c):

* OpenCL vector literals ``(float3)(a, b, c)`` become GCC compound literals
  ``((float3){a, b, c})``;
* component access ``.x .y .z .w`` becomes ``[0] [1] [2] [3]`` (wavefront.cl has no
  swizzles and no struct member named x, y, z or w);
* floatToUlong's ``(ulong)(fabs(x) * ULONG_MAX)`` becomes
  ``ref_float_to_ulong(fabs(x) * ULONG_MAX)``: C leaves the conversion of NaN and
  of values >= 2^64 undefined (x86 gives 2^63, GPUs and Arm saturate), and the
  shim's function saturates (NaN -> 0), as the parity contract defines it;
* the material stage's float-to-uchar conversions (evaluateMaterial's
  ``(uchar)(ringWeighting * baseWeighting)`` and evaluateBackground's ambient
  blend) become ``ref_float_to_uchar(...)``: out-of-range values are undefined in
  C, and the shim's function saturates, as the parity contract defines it;
* the kernels' ``local uint localQueue[5];`` gets a zero initialiser. ``increment``
  (wavefront.cl:254-258) relies on work-items 0..4 of a group to clear the five
  entries; the harness runs one work-item per group, which would clear only entry 0.

Nothing else in the kernel source changes. ref_shim.h supplies the OpenCL types and
built-ins, ref_harness.c drives the kernels the way SvoTracer.Window/MainWindow.cs
does, and gcc links the three into oracle/_ref/libsvo_ref.so. The megakernel gets
its own library, oracle/_ref/libsvo_ref_mega.so (ref_mega_harness.c runs its
`trace` kernel once per pixel), because both sources define the same helpers.

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
# The reference checkout: $SVO_REFERENCE_ROOT, else a directory named
# "reference" beside this repository. SVO_REFERENCE_WAVEFRONT and
# SVO_REFERENCE_MEGAKERNEL name the two kernel files directly.
REF_ROOT = os.environ.get("SVO_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
REF_SOURCE = os.environ.get(
    "SVO_REFERENCE_WAVEFRONT",
    os.path.join(REF_ROOT, "SvoTracer", "SvoTracer.Kernel", "wavefront.cl"),
)
REWRITTEN = os.path.join(REF_DIR, "wavefront_ref.c")
REF_LIB = os.path.join(REF_DIR, "libsvo_ref.so")
MEGA_SOURCE = os.environ.get(
    "SVO_REFERENCE_MEGAKERNEL",
    os.path.join(REF_ROOT, "SvoTracer", "SvoTracer.Kernel", "kernel.cl"),
)
MEGA_REWRITTEN = os.path.join(REF_DIR, "kernel_ref.c")
MEGA_LIB = os.path.join(REF_DIR, "libsvo_ref_mega.so")

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
    src = src.replace("return (ulong)(fabs(x) * ULONG_MAX);", "return ref_float_to_ulong(fabs(x) * ULONG_MAX);")
    # the material stage's float-to-uchar conversions can leave uchar's range (a
    # negative or > 1 weighting; evaluateBackground's blend when the luminosity is
    # at most the ambient level wraps colourBoundary - baseColour to ~2^32)
    src = src.replace("(uchar)(ringWeighting * baseWeighting)", "ref_float_to_uchar(ringWeighting * baseWeighting)")
    src = re.sub(r"colour([RGB]) = \((baseColour\1 \+ lightQuotient \* colour\1 \* \(colourBoundary - baseColour\1\))\);",
                 r"colour\1 = ref_float_to_uchar(\2);", src)
    src = re.sub(r"\.([xyzw])\b", lambda m: "[%d]" % "xyzw".index(m.group(1)), src)
    return src


def _generate(source: str, rewritten: str, name: str) -> bool:
    if not os.path.exists(source):
        return os.path.exists(rewritten)
    os.makedirs(REF_DIR, exist_ok=True)
    with open(source, "r", encoding="utf-8-sig") as f:
        src = f.read()
    text = (
        "/* Generated by oracle/build_ref.py from the reference's %s: "
        "vector literals and component access rewritten for C. */\n" % name + rewrite(src)
    )
    if not os.path.exists(rewritten) or open(rewritten).read() != text:
        with open(rewritten, "w") as f:
            f.write(text)
    return True


def generate() -> bool:
    """Write oracle/_ref/wavefront_ref.c from the reference checkout, if present."""
    return _generate(REF_SOURCE, REWRITTEN, "wavefront.cl")


def _compile(rewritten: str, harness: str, lib: str, cc: str) -> str:
    deps = [rewritten, os.path.join(HERE, harness), os.path.join(HERE, "ref_shim.h")]
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(d) for d in deps):
        return lib
    cmd = [
        cc, "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
        "-fopenmp", "-w", "-Wno-psabi", "-include", os.path.join(HERE, "ref_shim.h"),
        os.path.join(HERE, harness), "-o", lib + ".tmp", "-lm",
    ]
    subprocess.run(cmd, check=True, cwd=REF_DIR)
    os.replace(lib + ".tmp", lib)
    return lib


def compile_ref(cc: str = "gcc") -> str | None:
    """Compile libsvo_ref.so; returns its path or None when the source is absent."""
    if not generate():
        return None
    return _compile(REWRITTEN, "ref_harness.c", REF_LIB, cc)


def compile_ref_mega(cc: str = "gcc") -> str | None:
    """Compile libsvo_ref_mega.so (kernel.cl); returns its path or None when the source is absent."""
    if not _generate(MEGA_SOURCE, MEGA_REWRITTEN, "kernel.cl"):
        return None
    return _compile(MEGA_REWRITTEN, "ref_mega_harness.c", MEGA_LIB, cc)


if __name__ == "__main__":
    for p in (compile_ref(), compile_ref_mega()):
        print(p if p else "reference source not available")
    sys.exit(0)
