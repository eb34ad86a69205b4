"""The staged optimizer's noise rows are uniform over the problem's rows.

The staged kernels draw a round's noise samples from a window of Y instead of
from all of it: 256-row segments at Philox-drawn uniform starts (wrapping at
N), the window picks taken from 16-bit halves of one Philox block per eight
samples, masked to the power-of-two window size; the batched kernel takes
multiply-shift picks from 32-bit words, over a whole small problem or over
the segments of a larger one.
Each sample is then uniform over the rows (before the redraw that skips the
edge's source row).  These tests replay those exact draws (the Philox
restatement of oracle/nce_oracle.py, vectorised) for independent samples and
check the row histogram with a chi-square statistic (within 6 standard
deviations of its mean).
"""
import numpy as np

from oracle.nce_oracle import MASK, bounded_index, noise_key, philox4x32_10

SEG = 256


def _chi2_ok(counts, expected):
    chi2 = float(((counts - expected) ** 2 / expected).sum())
    dof = counts.size - 1
    return abs(chi2 - dof) <= 6.0 * np.sqrt(2.0 * dof), chi2, dof


def _segmented_rows(N, W, rounds, edges_per_round, seed, epoch, block=0, mul_shift=False):
    """One noise sample per round: the first edge of round r, window pick
    r mod 8 of its Philox block (mul_shift: word r mod 4 of the block scaled
    to W by multiply-shift, the batched kernel's picks), through that round's
    segment starts.  Different rounds use disjoint Philox counters, so the
    samples are independent; samples of one round share its window and are
    not."""
    k0, k1 = noise_key(seed)
    nseg = W // SEG
    r = np.arange(rounds, dtype=np.uint64)
    rr = np.repeat(r, nseg)
    t = np.tile(np.arange(nseg, dtype=np.uint64), rounds)
    x = philox4x32_10(np.full(rr.size, block, np.uint64), rr, np.full(rr.size, epoch, np.uint64),
                      t | np.uint64(0x20000000), (k0 ^ 0x3C6EF372) & 0xFFFFFFFF, k1)
    seg = bounded_index(x[0], x[1], N).reshape(rounds, nseg)
    e = r * np.uint64(edges_per_round)
    if mul_shift:
        b = philox4x32_10(e & MASK, e >> np.uint64(32), np.full(rounds, epoch, np.uint64),
                          np.full(rounds, 0x50000000, np.uint64), k0, k1)
        word = np.stack(b)[(r % np.uint64(4)).astype(np.int64), np.arange(rounds)]
        u = ((word * np.uint64(W)) >> np.uint64(32)).astype(np.int64)
    else:
        b = philox4x32_10(e & MASK, e >> np.uint64(32), np.full(rounds, epoch, np.uint64),
                          np.full(rounds, 0x40000000, np.uint64), k0, k1)
        half = (r % np.uint64(8)).astype(np.int64)
        word = np.stack(b)[half >> 1, np.arange(rounds)]
        u = ((word >> (np.uint64(16) * (half & 1).astype(np.uint64))) &
             np.uint64(W - 1)).astype(np.int64)
    rows = seg[np.arange(rounds), u // SEG] + u % SEG
    return np.where(rows >= N, rows - N, rows)


def test_segmented_window_rows_are_uniform():
    N, W = 16384, 1024
    rows = _segmented_rows(N, W, rounds=N * 24, edges_per_round=256, seed=42, epoch=7)
    counts = np.bincount(rows, minlength=N).astype(np.float64)
    ok, chi2, dof = _chi2_ok(counts, rows.size / N)
    assert ok, (chi2, dof)


def test_segmented_window_rows_are_uniform_when_n_is_not_a_multiple():
    # N not a multiple of the segment length: segments wrap at N.
    N, W = 20011, 1024
    rows = _segmented_rows(N, W, rounds=N * 24, edges_per_round=64, seed=3, epoch=1)
    counts = np.bincount(rows, minlength=N).astype(np.float64)
    ok, chi2, dof = _chi2_ok(counts, rows.size / N)
    assert ok, (chi2, dof)


def test_batched_segmented_window_rows_are_uniform():
    # Batched problems larger than the window: 256-row segments of the
    # problem, picks by multiply-shift of 32-bit words over the 1,024 rows.
    N, W = 20011, 1024
    rows = _segmented_rows(N, W, rounds=N * 24, edges_per_round=64, seed=9, epoch=4, block=3,
                           mul_shift=True)
    counts = np.bincount(rows, minlength=N).astype(np.float64)
    ok, chi2, dof = _chi2_ok(counts, rows.size / N)
    assert ok, (chi2, dof)


def test_whole_problem_picks_are_uniform():
    # Batched problems that fit the window: four picks per Philox block by
    # multiply-shift of 32-bit words over the problem's N rows.
    k0, k1 = noise_key(5)
    N = 1000
    e = np.arange(200000, dtype=np.uint64)
    b = philox4x32_10(e & MASK, e >> np.uint64(32), np.full(e.size, 2, np.uint64),
                      np.full(e.size, 0x50000000, np.uint64), k0, k1)
    u = np.concatenate([(w * np.uint64(N)) >> np.uint64(32) for w in b]).astype(np.int64)
    assert u.min() >= 0 and u.max() < N
    counts = np.bincount(u, minlength=N).astype(np.float64)
    ok, chi2, dof = _chi2_ok(counts, u.size / N)
    assert ok, (chi2, dof)
