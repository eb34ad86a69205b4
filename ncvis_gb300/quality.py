"""Embedding quality measures used to compare embeddings end to end:
trustworthiness (Venna & Kaski, 2001; the definition scikit-learn's
manifold.trustworthiness implements) and kNN preservation (mean overlap of
the k nearest neighbours in the input and in the embedding).  Written with
torch so that they run on the GPU for large N and on the CPU for small N;
exact neighbours by brute force in row blocks.
"""
from __future__ import annotations

import numpy as np


def _torch():
    import torch
    return torch


def _as_tensor(a, device):
    torch = _torch()
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.float32)
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=device)


def _sqdist(A, B):
    torch = _torch()
    d = (A * A).sum(1, keepdim=True) - 2.0 * (A @ B.T) + (B * B).sum(1)[None, :]
    return torch.clamp_min(d, 0.0)


def knn_indices(X, k: int, device=None, block: int = 2048):
    """Indices [N, k] of each row's k nearest other rows (squared L2, FP64 on
    the device for ranking stability)."""
    torch = _torch()
    device = device or ("cuda" if torch.cuda.is_available() else "cpu")
    X = _as_tensor(X, device).double()
    N = X.shape[0]
    out = torch.empty((N, k), dtype=torch.int64, device=device)
    for s in range(0, N, block):
        e = min(N, s + block)
        d = _sqdist(X[s:e], X)
        d[torch.arange(e - s, device=device), torch.arange(s, e, device=device)] = float("inf")
        out[s:e] = torch.topk(d, k, dim=1, largest=False).indices
    return out


def knn_preservation(X, Y, k: int = 15, device=None) -> float:
    """Mean |kNN_X(i) ∩ kNN_Y(i)| / k."""
    torch = _torch()
    device = device or ("cuda" if torch.cuda.is_available() else "cpu")
    ix = knn_indices(X, k, device)
    iy = knn_indices(Y, k, device)
    N = ix.shape[0]
    hits = 0
    for s in range(0, N, 4096):
        a, b = ix[s:s + 4096], iy[s:s + 4096]
        hits += (a[:, :, None] == b[:, None, :]).any(2).sum().item()
    return hits / (N * k)


def trustworthiness(X, Y, k: int = 15, device=None, block: int = 1024) -> float:
    """1 - 2/(N k (2N - 3k - 1)) * sum_i sum_{j in kNN_Y(i)} max(0, r_X(i, j) - k),
    r_X(i, j) the 1-based rank of j among i's neighbours in X."""
    torch = _torch()
    device = device or ("cuda" if torch.cuda.is_available() else "cpu")
    Xt = _as_tensor(X, device).double()
    iy = knn_indices(Y, k, device)
    N = Xt.shape[0]
    penalty = 0
    for s in range(0, N, block):
        e = min(N, s + block)
        d = _sqdist(Xt[s:e], Xt)
        rows = torch.arange(e - s, device=device)
        d[rows, torch.arange(s, e, device=device)] = float("inf")
        order = torch.argsort(d, dim=1)
        rank = torch.empty_like(order)
        rank.scatter_(1, order, torch.arange(1, N + 1, device=device).expand(e - s, N))
        r = torch.gather(rank, 1, iy[s:e])
        penalty += torch.clamp_min(r - k, 0).sum().item()
    return 1.0 - penalty * (2.0 / (N * k * (2.0 * N - 3.0 * k - 1.0)))


def knn_preservation_device(X, Y, k: int = 15, distance: int = 0, x_inds=None) -> float:
    """kNN preservation at full size on the GPU: the exact kNN tables of X (in
    the engine's distance) and of Y (squared L2) come from the engine's own
    kNN kernels (one CUDA launch set each, O(N^2) work on the device), then
    the mean overlap |kNN_X(i) & kNN_Y(i)| / k.  Both tables follow the
    reference's row contract (the nearest of the k+1 dropped, normally the
    point itself).  `x_inds` may pass a precomputed table of X."""
    torch = _torch()
    from . import stages
    if x_inds is None:
        x_inds, _ = stages.knn(_as_tensor(X, "cuda"), k, distance)
    y_inds, _ = stages.knn(_as_tensor(Y, "cuda"), k, 0)
    a = x_inds.to(torch.int64)
    b = y_inds.to(torch.int64)
    hits = 0
    for s in range(0, a.shape[0], 1 << 16):
        aa, bb = a[s:s + (1 << 16)], b[s:s + (1 << 16)]
        hits += (aa[:, :, None] == bb[:, None, :]).any(2).sum().item()
    return hits / (a.shape[0] * k)


def trustworthiness_device(X, Y, k: int = 15, distance: int = 0) -> float:
    """Trustworthiness at k over all N points on the GPU (the engine's
    ncvis_trustworthiness_device): the embedding's exact kNN, then each
    neighbour's rank in X under the engine's `distance` (0 squared L2,
    1 inner product, 2 cosine, 3 correlation; for unit vectors the cosine
    ranks are the Euclidean ranks), counted over all points."""
    import ctypes as C
    from . import _lib, stages
    torch = _torch()
    Xd = _as_tensor(X, "cuda").contiguous()
    Yd = _as_tensor(Y, "cuda").contiguous()
    out = C.c_double(0.0)
    _lib.check(_lib.lib().ncvis_trustworthiness_device(
        Xd.data_ptr(), Xd.shape[0], Xd.shape[1], distance, Yd.data_ptr(), Yd.shape[1], k,
        C.byref(out), stages._stream()))
    return out.value


def recall_at_k(found, exact) -> float:
    """Mean fraction of each row of `exact` (index sets) present in `found`."""
    found = np.asarray(found)
    exact = np.asarray(exact)
    hits = 0
    for a, b in zip(found, exact):
        hits += len(np.intersect1d(a, b, assume_unique=False))
    return hits / exact.size
