"""The integer form of the u64 -> f32 round-to-nearest conversion that some
kernels use instead of the 64-bit conversion instruction (trace_core.cuh,
ulong_to_float): top 32 significant bits with a sticky LSB, a 32-bit
round-to-nearest conversion, and the exponent shift. Restated in numpy and
checked against numpy's own u64 -> f32 conversion (round to nearest even) on
random values of every magnitude and on the rounding edge cases. The CUDA
code itself is checked bit-exactly by the GPU parity tests."""
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
