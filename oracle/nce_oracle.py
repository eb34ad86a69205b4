"""ORACLE — test infrastructure, not product code.

FP64 numpy restatement of the NCE objective that NCVis::optimize descends
(src/ncvis.cpp:304-323) and of the counter-based noise stream the engine's
loss kernels draw from, used to check ncvis_gb300.nce on the GPU:
  * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), multiply-shift bounded
    indices, and the retry rule for samples equal to the edge source;
  * loss = sum_e softplus(log nu + Q - log Ph(d2_ij))
           + sum_s softplus(log Ph(d2_io) - Q - log nu),  Ph = 1/(1 + a d2^b);
  * its analytic gradient, which equals the reference's per-sample update
    weights: dL/dQ = w, dL/dy_i = 2 w a b Ph d2^(b-1) (y_i - y_o).
"""
from __future__ import annotations

import numpy as np

MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) & MASK for v in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint64) & MASK
    k1 = np.asarray(k1, dtype=np.uint64) & MASK
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def bounded_index(lo, hi, n):
    n = np.uint64(n)
    return ((hi * n + ((lo * n) >> np.uint64(32))) >> np.uint64(32)).astype(np.int64)


def noise_key(seed: int):
    return seed & 0xFFFFFFFF, ((seed >> 32) & 0xFFFFFFFF) ^ 0x5EED1


def noise_indices(src, N: int, nu: int, seed: int, tag: int, edge_offset: int = 0) -> np.ndarray:
    src = np.asarray(src, dtype=np.int64)
    E = src.size
    k0, k1 = noise_key(seed)
    e = np.arange(E, dtype=np.uint64) + np.uint64(edge_offset)
    out = np.empty((E, nu), np.int64)
    for s in range(nu):
        r = philox4x32_10(e & MASK, e >> np.uint64(32), np.full(E, tag, np.uint64),
                          np.full(E, s >> 1, np.uint64), k0, k1)
        h = s & 1
        o = bounded_index(r[2 * h], r[2 * h + 1], N)
        retry = 1
        bad = o == src
        while bad.any():
            idx = np.nonzero(bad)[0]
            if retry > 64:
                o[idx] = (o[idx] + 1) % N
                break
            eb = e[idx]
            rr = philox4x32_10(eb & MASK, (eb >> np.uint64(32)) ^ np.uint64(retry << 16),
                               np.full(idx.size, tag, np.uint64),
                               np.full(idx.size, (s >> 1) | 0x80000000, np.uint64),
                               (k0 ^ retry) & 0xFFFFFFFF, k1)
            o[idx] = bounded_index(rr[0], rr[1], N)
            bad[idx] = o[idx] == src[idx]
            retry += 1
        out[:, s] = o
    return out


def _softplus(u):
    return np.maximum(u, 0) + np.log1p(np.exp(-np.abs(u)))


def _sigmoid(u):
    return np.where(u >= 0, 1 / (1 + np.exp(-np.minimum(np.abs(u), 700))),
                    np.exp(-np.minimum(np.abs(u), 700)) / (1 + np.exp(-np.minimum(np.abs(u), 700))))


def loss_and_grad(Y, Q, src, dst, noise, a, b):
    """FP64 loss, dL/dY, dL/dQ for edges (src, dst) with noise [E, nu]."""
    Y = np.asarray(Y, dtype=np.float64)
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    nu = noise.shape[1]
    log_nu = np.log(nu)
    loss = 0.0
    dQ = 0.0
    dY = np.zeros_like(Y)
    for s in range(nu + 1):
        o = dst if s == 0 else noise[:, s - 1]
        diff = Y[src] - Y[o]
        d2 = (diff * diff).sum(1)
        with np.errstate(divide="ignore", invalid="ignore"):
            p = np.where(d2 > 0, d2 ** b, 0.0)
            p1 = np.where(d2 > 0, d2 ** (b - 1), 0.0 ** (b - 1) if b != 1 else 1.0)
        log_ph = -np.log1p(a * p)
        ph = 1.0 / (1.0 + a * p)
        if s == 0:
            u = log_nu + Q - log_ph
            w = _sigmoid(u)
        else:
            u = log_ph - Q - log_nu
            w = -_sigmoid(u)
        loss += _softplus(u).sum()
        dQ += w.sum()
        g = 2 * w * a * b * ph * p1
        gd = g[:, None] * diff
        gd[o == src] = 0.0
        np.add.at(dY, src, gd)
        np.add.at(dY, o, -gd)
    return loss, dY, dQ


def loss_only(Y, Q, src, dst, noise, a, b):
    return loss_and_grad(Y, Q, src, dst, noise, a, b)[0]
