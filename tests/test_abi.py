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


_SCALARS = {"int32_t": C.c_int32, "uint32_t": C.c_uint32, "uint16_t": C.c_uint16, "uint8_t": C.c_uint8,
            "size_t": C.c_size_t, "float": C.c_float, "double": C.c_double, "char": C.c_char}
_STRUCTS = {"svo_trace_input": "TraceInputC", "svo_trace_output": "TraceOutputC", "svo_trace_config": "TraceConfigC",
            "svo_trace_stats": "TraceStatsC", "svo_mega_stats": "MegaStatsC", "svo_update_input": "UpdateInputC",
            "svo_gc_report": "GcReportC", "svo_graft_report": "GraftReportC", "svo_prune_report": "PruneReportC",
            "svo_scene_params": "SceneParamsC"}


def declarations():
    """(name, [parameter type strings]) of every SVO_API function in include/."""
    out = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        text = re.sub(r"/\*.*?\*/", " ", open(os.path.join(ROOT, "include", fn)).read(), flags=re.S)
        for m in re.finditer(r"SVO_API\s+[\w\s\*]+?\b(svo_\w+)\s*\(([^)]*)\)\s*;", text):
            params = [" ".join(p.split()) for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
            out.append((m.group(1), [re.sub(r"\s*\b\w+$", "", p) for p in params]))
    return out


def _accepts(ctype_str, binding):
    """Whether a ctypes argtype can carry the C parameter type `ctype_str`."""
    t = ctype_str.replace("const ", "").strip()
    stars = t.count("*")
    base = t.replace("*", "").strip()
    if stars == 0:
        return binding is _SCALARS[base]
    if stars == 2:
        return binding is C.POINTER(C.c_void_p)
    if base == "char":
        return binding is C.c_char_p
    if binding is C.c_void_p:  # arrays and opaque handles
        return base not in _STRUCTS
    if base in _STRUCTS:
        return binding is C.POINTER(getattr(st, _STRUCTS[base]))
    return binding is C.POINTER(_SCALARS[base])


def test_binding_signatures_match_the_header():
    """Every declared entry point, svo_trace_noalloc among them, is bound with its
    header's parameter count and types in order (an argument reordered or
    retyped in svo.h fails here, without a GPU)."""
    lib = st.load_library()
    decls = declarations()
    assert {n for n, _ in decls} == set(declared_symbols())
    for name, params in decls:
        f = getattr(lib, name)
        assert f.argtypes is not None, name + " has no bound signature"
        assert len(f.argtypes) == len(params), name
        for i, (cp, bt) in enumerate(zip(params, f.argtypes)):
            assert _accepts(cp, bt), "%s argument %d: %s bound as %r" % (name, i, cp, bt)
    assert ("svo_trace_noalloc", ["int32_t", "void *", "uint8_t", "const uint16_t *", "size_t", "const svo_block *",
                                  "size_t", "svo_usage *", "size_t", "int32_t", "const svo_trace_input *",
                                  "const svo_trace_output *", "svo_child_request *", "uint32_t",
                                  "uint32_t *"]) in decls


def test_trace_config_layout():
    names = [n for n, _ in st.TraceConfigC._fields_]
    assert names[-3:] == ["pass_limit", "request_order", "gi_stage"]
    assert C.sizeof(st.TraceConfigC) == 4 * len(names)


def test_state_io_rejects_null_arguments():
    """svo_state_save / svo_state_load refuse a null context or path (no GPU work)."""
    lib = st.load_library()
    assert lib.svo_state_save(None, b"x.svostate") == 1
    assert b"svo_state_save" in lib.svo_last_error_string()
    assert lib.svo_state_load(None, b"x.svostate") == 1
    assert b"svo_state_load" in lib.svo_last_error_string()
