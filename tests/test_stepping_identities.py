"""The identities the device stepping code (trace_core.cuh) relies on when it
replaces the reference's 64-bit formulations by cheaper ones, checked here in
integer arithmetic against the direct restatements of wavefront.cl:

* roundUlong's boundary distance from the level mask's high word only;
* traverseChunk's clamp plus leaving() as one test of the moved coordinates;
* comparePositions, chunkPosition and the path check on the high words;
* the operand selection that gives each lane exactly two float->fixed conversions.

Levels run 1..24 (SVO_MAX_TREE_DEPTH), as on the device."""
import numpy as np
import pytest

M64 = (1 << 64) - 1
M32 = (1 << 32) - 1
MAX_DEPTH = 24


def coords(rng, n):
    """Random 64-bit coordinates with the edge values the stepping meets."""
    out = [0, 1, M64, M64 - 1, 1 << 63, (1 << 63) - 1, 1 << 32, (1 << 32) - 1]
    hi = rng.integers(0, 1 << 32, n, dtype=np.uint64)
    lo = rng.integers(0, 1 << 32, n, dtype=np.uint64)
    out += [int(h) << 32 | int(l) for h, l in zip(hi, lo)]
    # coordinates at and next to level boundaries
    for d in range(1, MAX_DEPTH + 1):
        b = 1 << (63 - d)
        k = int(rng.integers(0, 1 << d))
        out += [(k * b) & M64, (k * b - 1) & M64, (k * b + 1) & M64]
    return out


def boundary_reference(w, depth, positive):
    # (~w & low) + 1, or ~w for a negative direction in the lowest cell
    low = M64 >> (depth + 1)
    d = ((~w & M64) & low) + 1
    return (~w & M64) if (not positive and (w | low) == M64) else d & M64


def boundary_device(w, depth, positive):
    low_hi = M32 >> (depth + 1)
    wh = w >> 32
    t = (((~wh & M32) & low_hi) << 32) | (~w & M32)
    special = (not positive) and (wh | low_hi) == M32
    return (t + (0 if special else 1)) & M64


def test_boundary_distance_from_the_mask_high_word():
    rng = np.random.default_rng(1)
    for w in coords(rng, 300):
        for depth in range(1, MAX_DEPTH + 1):
            for positive in (True, False):
                assert boundary_device(w, depth, positive) == boundary_reference(w, depth, positive), (w, depth)


def test_leaving_after_a_move_is_one_test_of_the_sums():
    """traverseChunk clamps a sum of 0 to all ones, and leaving() then tests for
    all ones: the same as testing the unclamped sum for 0 or all ones."""
    rng = np.random.default_rng(2)
    ws = coords(rng, 200)
    ds = [0, 1, 2, M64, 1 << 40] + [int(x) for x in rng.integers(0, 1 << 63, 50, dtype=np.uint64)]
    for w in ws:
        for d in ds:
            s = (w + d) & M64
            clamped = M64 if s == 0 else s
            reference = clamped == M64
            lo, hi = s & M32, s >> 32
            device = lo == hi and ((hi + 1) & M32) <= 1
            assert reference == device, (w, d)
            if not reference:
                assert clamped == s  # a sum that stays inside is never clamped


def pop_reference(before, after, depth):
    m = 0
    for p, n in zip(before, after):
        m |= p & (~n & M64)
    run = ~(m >> (63 - depth)) & M64
    ones = (run & -run).bit_length() - 1 if run else 64
    return depth - ones if ones < depth else 1


def pop_device(before, after, depth):
    m = 0
    for p, n in zip(before, after):
        m |= (p >> 32) & (~(n >> 32) & M32)
    run = ~(m >> (31 - depth)) & M32
    ones = (run & -run).bit_length() - 1 if run else 32
    return depth - ones if ones < depth else 1


def test_compare_positions_on_the_high_words():
    rng = np.random.default_rng(3)
    cs = coords(rng, 120)
    for _ in range(4000):
        before = [cs[int(i)] for i in rng.integers(0, len(cs), 3)]
        after = [(b + int(rng.integers(0, 1 << 62))) & M64 if rng.random() < 0.7 else cs[int(rng.integers(0, len(cs)))]
                 for b in before]
        depth = int(rng.integers(1, MAX_DEPTH + 1))
        assert pop_device(before, after, depth) == pop_reference(before, after, depth)


def test_octant_and_path_check_on_the_high_words():
    rng = np.random.default_rng(4)
    cs = coords(rng, 200)
    for _ in range(3000):
        w = [cs[int(i)] for i in rng.integers(0, len(cs), 3)]
        p = [cs[int(i)] for i in rng.integers(0, len(cs), 3)]
        flip = int(rng.integers(0, 8))
        depth = int(rng.integers(0, MAX_DEPTH + 1))
        s = 63 - depth
        ref = (((w[0] >> s) & 1) | (((w[1] >> s) & 1) << 1) | (((w[2] >> s) & 1) << 2)) ^ flip
        s32 = 31 - depth
        dev = ((((w[0] >> 32) >> s32) & 1) | ((((w[1] >> 32) >> s32) & 1) << 1)
               | ((((w[2] >> 32) >> s32) & 1) << 2)) ^ flip
        assert ref == dev
        nd = int(rng.integers(3, MAX_DEPTH + 1))
        ref_changed = (((p[0] ^ w[0]) | (p[1] ^ w[1]) | (p[2] ^ w[2])) >> (64 - nd)) != 0
        dev_changed = ((((p[0] ^ w[0]) | (p[1] ^ w[1]) | (p[2] ^ w[2])) >> 32) >> (32 - nd)) != 0
        assert ref_changed == dev_changed


@pytest.mark.parametrize("ax", [0, 1, 2])
def test_two_conversions_reach_the_other_axes(ax):
    """The selected operands (A: y if x was chosen else x; B: y if z was chosen
    else z) and the scatter back give every axis but the chosen one its own move."""
    d = ["dx", "dy", "dz"]
    c0, c2 = ax == 0, ax == 2
    a_src = d[1] if c0 else d[0]
    b_src = d[1] if c2 else d[2]
    moves = {0: "keep", 1: "keep", 2: "keep"}
    moves[1] = a_src if c0 else (b_src if c2 else "keep")
    if not c0:
        moves[0] = a_src
    if not c2:
        moves[2] = b_src
    for k in range(3):
        assert moves[k] == ("keep" if k == ax else d[k])
