"""The segmented warp scans (COO, CSR stream / merge-path / batched, CSR5)
stop at the longest run of lanes without a segment start (`unflagged_run` in
csrc/common.cuh): a restatement of the 32-lane Kogge-Stone scan in numpy
checks that the shortened scan gives the full scan's sums bit for bit, on
random flag patterns and values (no GPU needed)."""
import numpy as np


def _scan(vals, flags, max_offset):
    """The device loop: for o = 1, 2, 4, ... (o <= max_offset, o < 32), each
    lane >= o without a flag adds the value o lanes up, then takes its flag."""
    S = vals.copy()
    f = flags.copy()
    o = 1
    while o < 32 and o <= max_offset:
        up = np.concatenate([np.zeros(o), S[:-o]])
        fu = np.concatenate([np.zeros(o, bool), f[:-o]])
        lane = np.arange(32)
        add = (lane >= o) & ~f
        S = np.where(add, S + up, S)
        f = np.where(lane >= o, f | fu, f)
        o <<= 1
    return S


def _unflagged_run(flags):
    z = 0
    for i, b in enumerate(flags):
        if not b:
            z |= 1 << i
    run = 0
    while z:
        z &= (z << 1) & 0xFFFFFFFF
        run += 1
    return run


def test_unflagged_run_counts_the_longest_gap():
    assert _unflagged_run([True] * 32) == 0
    assert _unflagged_run([False] * 32) == 32
    f = [False] * 32
    for i in (3, 7, 11, 15, 19, 23, 27, 31):
        f[i] = True
    assert _unflagged_run(f) == 3
    f = [True] + [False] * 9 + [True] * 22
    assert _unflagged_run(f) == 9


def test_shortened_scan_is_bit_identical():
    rng = np.random.default_rng(5)
    for trial in range(3000):
        p = rng.choice([0.02, 0.1, 0.25, 0.5, 0.9])
        flags = rng.random(32) < p
        vals = rng.standard_normal(32) * 10.0 ** rng.integers(-8, 8, 32)
        full = _scan(vals, flags, 31)
        short = _scan(vals, flags, _unflagged_run(flags))
        assert np.array_equal(full.view(np.uint64), short.view(np.uint64)), (trial, flags)


def test_keyed_scan_flags_are_key_changes():
    """The keyed scans flag lane 0 and every lane whose key differs from the
    lane before; with non-decreasing keys (rows, segment numbers) the runs
    of equal keys are the segments, and the shortened scan is exact."""
    rng = np.random.default_rng(6)
    for _ in range(1000):
        keys = np.sort(rng.integers(0, rng.integers(1, 33), 32))
        flags = np.concatenate([[True], keys[1:] != keys[:-1]])
        vals = rng.standard_normal(32)
        full = _scan(vals, flags, 31)
        short = _scan(vals, flags, _unflagged_run(flags))
        assert np.array_equal(full, short)
        # each lane's sum covers exactly its key's lanes up to itself
        for j in range(32):
            same = [i for i in range(j + 1) if keys[i] == keys[j]]
            assert np.isclose(full[j], vals[same].sum())
