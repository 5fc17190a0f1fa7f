"""The integer forms of the fixed-point conversions that the kernels can use
instead of the 64-bit conversion instructions (trace_core.cuh):
* ulong_to_float (u64 -> f32, round to nearest even): top 32 significant bits
  with a sticky LSB, a 32-bit round-to-nearest conversion, and the exponent
  shift;
* unit_to_ulong (floatToUlong, wavefront.cl:200-207: |x| * 2^64 truncated,
  saturating, NaN -> 0): the significand shifted by the exponent.
Each is restated in numpy and checked against numpy's own conversions on random
values of every magnitude and on the rounding and range edge cases. The CUDA code
itself is checked bit-exactly by the GPU parity tests."""
import numpy as np

U = np.uint64


def clz32(v):
    """Leading zeros of 32-bit words (32 for zero)."""
    v = v.astype(np.uint64)
    n = np.full(v.shape, 32, np.uint64)
    for b in range(31, -1, -1):
        hit = ((v >> U(b)) & U(1)).astype(bool) & (n == 32)
        n[hit] = U(31 - b)
    return n


def ulong_to_float_integer(x):
    hi, lo = x >> U(32), x & U(0xFFFFFFFF)
    n = clz32(hi)
    safe = np.minimum(n, U(31))
    top = np.where(n >= 32, lo, ((hi << safe) | np.where(safe == 0, U(0), lo >> (U(32) - safe))) & U(0xFFFFFFFF))
    rest = np.where(n >= 32, U(0), (lo << safe) & U(0xFFFFFFFF))
    t = (top | (rest != 0).astype(np.uint64)).astype(np.uint32)
    f = t.astype(np.float32)  # a 32-bit value, rounded to nearest even
    bits = f.view(np.uint32).astype(np.int64) + ((32 - n.astype(np.int64)) << 23)
    return bits.astype(np.uint32).view(np.float32)


def test_matches_round_to_nearest():
    rng = np.random.default_rng(1)
    x = rng.integers(0, 2**63, 400_000, dtype=np.uint64) * U(2) + rng.integers(0, 2, 400_000, dtype=np.uint64)
    x >>= rng.integers(0, 64, len(x)).astype(np.uint64)
    edges = np.array([0, 1, 3, 2**24 - 1, 2**24, 2**24 + 1, 2**25 + 1, 2**32 - 1, 2**32, 2**32 + 1, 2**40 + 2**16,
                      2**63, 2**64 - 1, 2**64 - 2**39, 2**64 - 2**40, 2**64 - 2**40 - 1, 0x8000008000000000,
                      0x8000018000000000, 0x8000008000000001, 0x0000000100000080, 0x00000001000000C0], dtype=np.uint64)
    x = np.concatenate([x, edges])
    got = ulong_to_float_integer(x)
    want = x.astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


K_ALL = U(2**64 - 1)


def unit_to_ulong_integer(x):
    """The integer form, one value at a time (x a numpy float32)."""
    if x >= np.float32(0.999999911):
        return K_ALL
    u = int(np.array([x], np.float32).view(np.uint32)[0]) & 0x7FFFFFFF
    if u > 0x7F800000:
        return U(0)
    if u >= 0x3F800000:
        return K_ALL
    e = (u >> 23) - 86
    m = (u & 0x7FFFFF) | 0x800000
    if e >= 0:
        return U(m << e)
    return U(m >> -e) if e > -24 else U(0)


def unit_to_ulong_reference(x):
    """floatToUlong as the instruction computes it: |x| * 2^64 (exact) truncated,
    saturating at 2^64 - 1, NaN -> 0; x >= 0.999999911 gives 2^64 - 1."""
    if x >= np.float32(0.999999911):
        return K_ALL
    if np.isnan(x):
        return U(0)
    v = abs(float(x)) * 2.0**64  # exact in double: a power-of-two scale of a float
    if v >= 2.0**64:
        return K_ALL
    return U(int(v))


def test_unit_to_ulong_integer_form():
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 2**32, 50_000, dtype=np.uint64).astype(np.uint32)
    xs = list(bits.view(np.float32))
    xs += [np.float32(v) for v in (0.0, -0.0, 1.0, -1.0, 0.999999911, -0.999999911, 0.99999988, -0.99999994,
                                   2.0**-64, 2.0**-65, 1.5 * 2.0**-64, 2.0**-40, 2.0**-41 * 3, 0.5, -0.5, 1e-30,
                                   1.4e-45, -1.4e-45, np.inf, -np.inf, np.nan, 3.0, -3.0)]
    xs += list(np.nextafter(np.float32(0.999999911), np.float32(0), dtype=np.float32) for _ in range(1))
    for x in xs:
        assert unit_to_ulong_integer(x) == unit_to_ulong_reference(x), repr(x)
