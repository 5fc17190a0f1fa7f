"""Hand-derived cases for the oracle's fixed-point helpers (wavefront.cl:200-497)."""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po

U64 = (1 << 64) - 1


@pytest.fixture(scope="module")
def lib():
    return po.oracle_lib()


def test_float_to_ulong(lib):
    f = lib.oracle_float_to_ulong
    assert f(0.0) == 0
    assert f(0.5) == 1 << 63
    assert f(0.25) == 1 << 62
    assert f(-0.25) == 1 << 62  # fabs(x) * ULONG_MAX
    assert f(1.0) == U64
    assert f(np.float32(0.999999911)) == U64  # the float 1 - 2^-24 clamps
    assert f(float(np.nextafter(np.float32(1 - 2 ** -24), np.float32(0)))) == int((1 - 2 ** -23) * 2 ** 64)
    assert f(float("nan")) == 0
    assert f(-1.5) == U64  # out of range saturates


def test_ulong_to_float(lib):
    g = lib.oracle_ulong_to_float
    assert g(0) == 0.0
    assert g(1 << 63) == 0.5
    assert g(U64) == 1.0  # (float)ULONG_MAX rounds to 2^64
    assert g((1 << 62) + 1) == 0.25


def test_round_ulong(lib):
    r = lib.oracle_round_ulong
    # depth 0: level-1 cells of size 2^63
    assert r(0, 0, 1) == 1 << 63
    assert r(5, 0, 1) == (1 << 63) - 5
    assert r(1 << 63, 0, 1) == 1 << 63  # wraps to 0 at the top: ((v&m)+2^63)-v = 2^64-2^63
    # down: distance to the last position of the previous cell
    assert r((1 << 63) + 7, 0, 0) == 8
    assert r(7, 0, 0) == 7  # no previous cell: returns value
    # depth 2: cells of 2^61
    v = (3 << 61) + 12345
    assert r(v, 2, 1) == (1 << 61) - 12345
    assert r(v, 2, 0) == 12346


def test_pow_sum(lib):
    for d in range(0, 9):
        assert lib.oracle_pow_sum(d) == sum(8 ** i for i in range(1, d + 1))


def _loc(*v):
    return (C.c_uint64 * 3)(*v)


def _sign(*v):
    return (C.c_int * 3)(*v)


def test_compare_positions(lib):
    cp = lib.oracle_compare_positions
    # moving +x from the last level-3 octant of a level-2 cell into the next level-2 cell
    prev = _loc((1 << 61) - 1, 0, 0)
    new = _loc(1 << 61, 0, 0)
    # bit 61 (level 2 octant) 0->1: no carry past level 2, so depth 2 stays ... at depth 3 bit 60 flipped 1->0
    assert cp(3, prev, new, _sign(1, 1, 1)) == 2
    # stepping within a cell keeps the depth
    assert cp(3, _loc(0, 0, 0), _loc(1 << 60, 0, 0), _sign(1, 1, 1)) == 3
    # carry all the way to the top stops at depth 1
    assert cp(5, _loc((1 << 63) - 1, 0, 0), _loc(1 << 63, 0, 0), _sign(1, 1, 1)) == 1
    # negative direction: a 0->1 flip is the carry
    assert cp(3, _loc(1 << 61, 0, 0), _loc((1 << 61) - 1, 0, 0), _sign(0, 1, 1)) == 2


def test_traverse_chunk_axis_aligned(lib):
    loc = _loc(1 << 62, 1 << 62, 1 << 62)
    d = (C.c_float * 3)(1.0, 0.0, 0.0)
    inv = (C.c_float * 3)(1.0, float("inf"), float("inf"))
    lib.oracle_traverse_chunk(1, d, inv, _sign(1, 1, 1), loc)
    # to the next level-2 boundary along +x; y and z move by dir * inv.x * dx = 0
    assert loc[0] == 1 << 63
    assert loc[1] == 1 << 62 and loc[2] == 1 << 62


def test_trace_into_volume(lib):
    o = (C.c_float * 3)(-1.0, 0.5, 0.5)
    d = (C.c_float * 3)(1.0, 0.0, 0.0)
    inv = (C.c_float * 3)(1.0, float("inf"), float("inf"))
    dof = (C.c_float * 2)(0.0, 0.0)
    loc = _loc(0, 0, 0)
    assert lib.oracle_trace_into_volume(o, d, inv, 0.01, dof, loc) == 1
    assert loc[0] == 0 and loc[1] == 1 << 63 and loc[2] == 1 << 63
    # pointing away from the cube
    d2 = (C.c_float * 3)(-1.0, 0.0, 0.0)
    inv2 = (C.c_float * 3)(-1.0, float("inf"), float("inf"))
    assert lib.oracle_trace_into_volume(o, d2, inv2, 0.01, dof, loc) == 0
    # parallel to an axis whose slab the origin is outside of
    o3 = (C.c_float * 3)(0.5, 2.0, 0.5)
    assert lib.oracle_trace_into_volume(o3, d, inv, 0.01, dof, loc) == 0
    # inside: location is the origin itself
    o4 = (C.c_float * 3)(0.25, 0.5, 0.75)
    assert lib.oracle_trace_into_volume(o4, d, inv, 0.01, dof, loc) == 1
    assert (loc[0], loc[1], loc[2]) == (1 << 62, 1 << 63, 3 << 62)
