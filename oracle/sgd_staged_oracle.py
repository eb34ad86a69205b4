"""ORACLE — test infrastructure, not product code.

Sequential numpy restatement of the engine's staged-noise optimizer
(ncvis_optimize_staged_device) for ONE chain, used to check the kernel's
sampling and update semantics on the GPU.  It follows NCVis::optimize
(src/ncvis.cpp:275-352): per epoch step = alpha (1 - (e/n_epochs)^2); every
edge (i, j) is followed by nu noise samples; per sample
  d2 = |y_i - y_o|^2, Ph = 1/(1 + a d2^b),
  w = 1/(1 + Ph/(nu e^Q)) (positive) | -1/(1 + nu e^Q / Ph) (noise),
  Q -= alpha_Q w, w <- 2 w Ph a b d2^(b-1), dx = clip((y_o - y_i) w step, +-4),
  y_i += dx, y_o -= dx,
with the noise draw restated for the staged form: the chain runs its edges in
rounds of `round_edges`; each round copies a window of W rows (W/256
segments of 256 consecutive rows, each starting at a Philox-drawn uniform
row, wrapping at N); every noise sample is a uniform pick among the window
rows (samples 8q..8q+7 of an edge take the eight 16-bit halves of one
Philox block, masked to the power-of-two window size; a pick whose row is the
edge source is redrawn); noise updates go to
the window, and the window's change is added to Y at the end of the round.
The source row is held aside (as the kernel holds it in registers) and
written back when the source changes and after the last round: stored when
Y still holds the value the chain read, else the chain's change is added
(a window write-back may have changed the row meanwhile).
"""
from __future__ import annotations

import numpy as np

from .nce_oracle import bounded_index, noise_key, philox4x32_10

SEG_ROWS = 256


def window_rows(d: int) -> int:
    """Rows of a window: the largest power of two <= 4096 whose two copies
    of d floats per row fit in 64 KiB."""
    w = 4096
    while w > SEG_ROWS and w * d * 8 > 65536:
        w >>= 1
    return w


def _philox(c0, c1, c2, c3, k0, k1):
    r = philox4x32_10(c0, c1, c2, c3, k0, k1)
    return [np.uint64(v) for v in r]


def _segments(k0, k1, block, rnd, epoch, W, N):
    out = []
    for t in range(W // SEG_ROWS):
        r = _philox(block, rnd, epoch, t | 0x20000000, (k0 ^ 0x3C6EF372) & 0xFFFFFFFF, k1)
        out.append(int(bounded_index(r[0], r[1], N)))
    return out


def _row(seg, u, N):
    r = seg[u // SEG_ROWS] + (u % SEG_ROWS)
    return r - N if r >= N else r


def _redraw(k0, k1, e, epoch, s, u, i, seg, W, N):
    retry = 1
    while _row(seg, u, N) == i:
        if retry > 64:
            u = 0 if u + 1 == W else u + 1
            break
        rr = _philox(e & 0xFFFFFFFF, ((e >> 32) ^ (retry << 16)) & 0xFFFFFFFF, epoch,
                     (s >> 1) | 0xC0000000, (k0 ^ retry) & 0xFFFFFFFF, k1)
        h = s & 1
        u = int(bounded_index(rr[2 * h], rr[2 * h + 1], W))
        retry += 1
    return u


def _weight(d2, positive, nu, step, a, b, alpha_Q, Q):
    if nu == 0:
        return step, Q
    if d2 > 0:
        p = d2 ** b
        p1 = p / d2
    else:
        p = 0.0
        p1 = 0.0 ** (b - 1) if b != 1 else 1.0
    denom = a * p + 1.0
    ph = 1.0 / denom
    nm = nu * np.exp(Q)
    w = 1.0 / (ph / nm + 1.0) if positive else -1.0 / (nm * denom + 1.0)
    Q = Q - w * alpha_Q
    w = w * p1 * (2.0 * a * b * ph)
    return w * step, Q


def _put(Y, ci, yi, yi0):
    """The kernel's write-back of a held source row (put_row)."""
    if np.array_equal(Y[ci], yi0):
        Y[ci] = yi
    else:
        Y[ci] += yi - yi0


def optimize_staged_one_chain(Y, Q, src, dst, seed, n_noise, a, b, alpha=1.0, alpha_Q=1.0,
                              epoch_begin=0, epoch_end=None, round_edges=8):
    """Y [N, d] and Q after epochs [epoch_begin, epoch_end) of the staged
    optimizer run as one chain (FP64)."""
    Y = np.array(Y, dtype=np.float64)
    N, d = Y.shape
    W = window_rows(d)
    plan = [int(v) for v in n_noise]
    n_epochs = len(plan)
    if epoch_end is None:
        epoch_end = n_epochs
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    E = src.size
    k0, k1 = noise_key(seed)
    chunk = (E + 3) & ~3
    re = (round_edges + 3) & ~3
    rounds = (chunk + re - 1) // re
    Q = float(Q)
    for ep in range(epoch_begin, epoch_end):
        nu = plan[ep]
        frac = float(np.float32(ep) / np.float32(n_epochs))
        step = alpha * (1.0 - frac * frac)
        have, ci, yi, yi0 = False, 0, None, None
        for r in range(rounds):
            seg = _segments(k0, k1, 0, r, ep, W, N)
            rows = np.array([_row(seg, u, N) for u in range(W)], dtype=np.int64)
            win = Y[rows].copy()
            loaded = win.copy()
            lo = min(E, r * re)
            hi = min(E, lo + re)
            for e in range(lo, hi):
                i, j = int(src[e]), int(dst[e])
                if not have or i != ci:
                    if have:
                        _put(Y, ci, yi, yi0)
                    ci, yi, have = i, Y[i].copy(), True
                    yi0 = yi.copy()
                if j != i:
                    yj = Y[j].copy()
                    diff = yi - yj
                    ws, Q = _weight(float(diff @ diff), True, nu, step, a, b, alpha_Q, Q)
                    dx = np.clip((yj - yi) * ws, -4.0, 4.0)
                    yi = yi + dx
                    Y[j] -= dx
                else:
                    _, Q = _weight(0.0, True, nu, step, a, b, alpha_Q, Q)
                for s0 in range(0, nu, 8):
                    rb = _philox(e & 0xFFFFFFFF, (e >> 32) & 0xFFFFFFFF, ep,
                                 (s0 >> 3) | 0x40000000, k0, k1)
                    for t in range(min(8, nu - s0)):
                        u = (int(rb[t >> 1]) >> (16 * (t & 1))) & (W - 1)
                        u = _redraw(k0, k1, e, ep, s0 + t, u, i, seg, W, N)
                        yo = win[u].copy()
                        diff = yi - yo
                        ws, Q = _weight(float(diff @ diff), False, nu, step, a, b, alpha_Q, Q)
                        dx = np.clip((yo - yi) * ws, -4.0, 4.0)
                        yi = yi + dx
                        win[u] = yo - dx
            np.add.at(Y, rows, win - loaded)
        if have:
            _put(Y, ci, yi, yi0)
    return Y, Q
