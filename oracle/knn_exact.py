"""ORACLE — test infrastructure, not product code.

FP64 exact kNN rows, the checker for the kNN stage.  The reference's kNN
(NCVis::buildKNN / findKNN, src/ncvis.cpp:72-153) asks hnswlib for the k+1
nearest points of every point, drops the nearest (the point itself) and keeps
the other k; distances are squared L2 (L2Space) or 1 - <x, y> on the
preprocessed points (InnerProductSpace for inner_product, cosine and
correlation, src/ncvis.cpp:78-92).  hnswlib's search is approximate and its
source is absent, so this oracle pins the rows to exact search in FP64: the
k+1 smallest distances ordered by (distance, index), the first dropped.  Rows
come back nearest first; the engine's table is farthest first, and the
tests compare sets.

Two backends: numpy on the host, or torch FP64 on a device (the GEMM of a
full-set check at 131,072 points takes seconds on a GPU and minutes on the
host)."""
from __future__ import annotations

import numpy as np


def _select(vals: np.ndarray, idx: np.ndarray, k: int) -> np.ndarray:
    """Rows of the k+2 smallest candidates (vals, idx) -> the k+1 smallest by
    (distance, index), the first dropped."""
    order = np.lexsort((idx, vals), axis=-1)[:, :k + 1]
    return np.take_along_axis(idx, order, 1)[:, 1:]


def exact_rows(Xp, queries, k: int, dist: int, device: str | None = None,
               block: int | None = None) -> np.ndarray:
    """kNN rows [len(queries), k] (int64) of the preprocessed points Xp [N, D]
    for the given query rows; dist 0 = squared L2, else 1 - <x, y>.  device:
    None for numpy on the host, else a torch device name ('cuda')."""
    Xp = np.ascontiguousarray(Xp)
    N = Xp.shape[0]
    queries = np.asarray(queries, dtype=np.int64)
    if block is None:
        block = max(64, min(512, int(2e9 // (8 * N))))  # about 2 GB of distances per block
    out = np.empty((len(queries), k), np.int64)
    if device is None:
        X = Xp.astype(np.float64)
        sq = (X * X).sum(1)
        for s in range(0, len(queries), block):
            q = queries[s:s + block]
            G = X[q] @ X.T
            d = sq[q, None] + sq[None, :] - 2.0 * G if dist == 0 else 1.0 - G
            idx = np.argpartition(d, k + 1, axis=1)[:, :k + 2]
            out[s:s + len(q)] = _select(np.take_along_axis(d, idx, 1), idx, k)
        return out
    import torch
    X = torch.as_tensor(Xp, device=device).double()
    sq = (X * X).sum(1)
    for s in range(0, len(queries), block):
        q = torch.as_tensor(queries[s:s + block], device=device)
        G = X[q] @ X.T
        d = sq[q, None] + sq[None, :] - 2.0 * G if dist == 0 else 1.0 - G
        vals, idx = torch.topk(d, k + 2, dim=1, largest=False)
        out[s:s + len(q)] = _select(vals.cpu().numpy(), idx.cpu().numpy(), k)
    return out


def recall(found: np.ndarray, exact: np.ndarray) -> float:
    """Mean over rows of |found ∩ exact| / k (rows of distinct indices)."""
    found = np.asarray(found, dtype=np.int64)
    exact = np.asarray(exact, dtype=np.int64)
    hits = 0
    for s in range(0, len(found), 8192):
        hits += int((found[s:s + 8192, :, None] == exact[s:s + 8192, None, :]).sum())
    return hits / exact.size
