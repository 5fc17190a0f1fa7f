"""The C ABI library loads, exports every entry point include/svo.h declares, and its
struct layouts match the OpenCL layouts of wavefront.cl. No GPU work is issued."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import svo_tracer as st

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"SVO_API\s+[\w\s\*]+?\b(svo_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("svo_create", "svo_destroy", "svo_upload_octree", "svo_init_usage", "svo_trace", "svo_trace_batch",
                 "svo_read_child_requests", "svo_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = st.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", st.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (svo_\w+)", out))
    assert set(declared_symbols()) <= exported


def test_struct_layouts():
    assert C.sizeof(st.TraceInputC) == 104
    assert st.TraceInputC.screen_size.offset == 64
    assert st.TraceInputC.max_opacity.offset == 72
    assert st.TraceInputC.tick.offset == 74
    assert st.TraceInputC.ambient_light_level.offset == 96
    assert st.BLOCK_DTYPE.itemsize == 16 and st.BLOCK_DTYPE.fields["colour_r"][1] == 10
    assert st.USAGE_DTYPE.itemsize == 8 and st.USAGE_DTYPE.fields["parent"][1] == 4
    assert st.CHILD_REQUEST_DTYPE.itemsize == 40 and st.CHILD_REQUEST_DTYPE.fields["location"][1] == 8
    assert st.CHILD_REQUEST_DTYPE.fields["tree_size"][1] == 32


def test_version_and_error_string():
    lib = st.load_library()
    assert b"sm_103a" in lib.svo_version()
    # a null argument is rejected with a message, like ComputeManager.HandleResultCode
    assert lib.svo_create(0, None) == 1
    assert b"svo_create" in lib.svo_last_error_string()


def test_errors_raise_with_method_and_code():
    with pytest.raises(st.SvoError) as e:
        st._check("EnqueueNDRangeKernel", 4)
    assert str(e.value).startswith("EnqueueNDRangeKernel: QueueFull")


def test_null_context_is_rejected():
    lib = st.load_library()
    assert lib.svo_trace(None, None, None) == 1
    assert lib.svo_upload_octree(None, 4, None, 0, None, 0, 0) == 1
