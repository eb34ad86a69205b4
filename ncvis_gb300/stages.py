"""Stage-level entry points of the engine on CUDA torch tensors.

Each function calls the matching C-ABI entry point of libncvis_gb300.so
(include/ncvis_gb300.h) on the current torch stream; torch only provides the
device memory.  Indices are int32.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _torch():
    import torch
    return torch


def _stream():
    return _torch().cuda.current_stream().cuda_stream


def _f32(t):
    torch = _torch()
    assert t.is_cuda, "expected a CUDA tensor"
    return t.to(torch.float32).contiguous()


def _i32(t):
    torch = _torch()
    assert t.is_cuda, "expected a CUDA tensor"
    return t.to(torch.int32).contiguous()


def knn(X, k: int, distance: int = 0, precision: int = _lib.KNN_FP32, rerank_factor: int = 0,
        order: bool = True):
    """Exact kNN table (reference row contract, src/ncvis.cpp:128-153):
    returns (inds int32 [N, k], dists float32 [N, k]), rows in descending
    distance order, the nearest of the k+1 dropped.  order=False keeps the
    BF16 search in the caller's row order (no k-means cell ordering)."""
    torch = _torch()
    X = _f32(X)
    N, D = X.shape
    if not order:
        precision |= _lib.KNN_CALLER_ORDER
    inds = torch.empty((N, k), dtype=torch.int32, device=X.device)
    dists = torch.empty((N, k), dtype=torch.float32, device=X.device)
    _lib.check(_lib.lib().ncvis_knn_device(X.data_ptr(), N, D, distance, k, precision,
                                           rerank_factor, inds.data_ptr(), dists.data_ptr(),
                                           _stream()))
    return inds, dists


def knn_ivf(X, k: int, distance: int = 0, lists: int = 0, probe: int = 0,
            rerank_factor: int = 0):
    """Approximate kNN table (inverted file: k-means cells on BF16 rows,
    each cell searched against its `probe` nearest cells on the tensor cores,
    exact FP32 rerank); the row contract of `knn`."""
    torch = _torch()
    X = _f32(X)
    N, D = X.shape
    inds = torch.empty((N, k), dtype=torch.int32, device=X.device)
    dists = torch.empty((N, k), dtype=torch.float32, device=X.device)
    _lib.check(_lib.lib().ncvis_knn_ivf_device(X.data_ptr(), N, D, distance, k, rerank_factor,
                                               lists, probe, inds.data_ptr(), dists.data_ptr(),
                                               _stream()))
    return inds, dists


def symmetrize(inds, dists):
    """Bit-exact symmetrized CSR of a kNN table: (row_ptr int64 [N+1],
    cols int32 [E], vals float32 [E], src int32 [E])."""
    torch = _torch()
    inds, dists = _i32(inds), _f32(dists)
    N, k = inds.shape
    row_ptr = torch.empty(N + 1, dtype=torch.int64, device=inds.device)
    cap = max(2 * N * k, 1)
    cols = torch.empty(cap, dtype=torch.int32, device=inds.device)
    vals = torch.empty(cap, dtype=torch.float32, device=inds.device)
    src = torch.empty(cap, dtype=torch.int32, device=inds.device)
    E = C.c_size_t(0)
    _lib.check(_lib.lib().ncvis_symmetrize_device(N, k, inds.data_ptr(), dists.data_ptr(),
                                                  row_ptr.data_ptr(), cols.data_ptr(),
                                                  vals.data_ptr(), src.data_ptr(), C.byref(E),
                                                  _stream()))
    n = E.value
    return row_ptr, cols[:n], vals[:n], src[:n]


def init_embedding(row_ptr, cols, d: int, seed: int, n_init_epochs: int, alpha: float,
                   sequential_stats: bool = False):
    """Y [N, d]: one-thread pcg64(seed) uniforms, then n_init_epochs of
    neighbour averaging and standardisation (src/ncvis.cpp:184-273);
    sequential_stats: the statistics as the reference's one thread sums them."""
    torch = _torch()
    N = row_ptr.shape[0] - 1
    row_ptr = row_ptr.to(torch.int64).contiguous()
    cols = _i32(cols)
    Y = torch.empty((N, d), dtype=torch.float32, device=row_ptr.device)
    _lib.check(_lib.lib().ncvis_init_embedding_device(N, d, row_ptr.data_ptr(), cols.data_ptr(),
                                                      seed, n_init_epochs, alpha,
                                                      int(bool(sequential_stats)), Y.data_ptr(),
                                                      _stream()))
    return Y


def optimize(Y, Q, src, dst, seed: int, n_noise, a: float, b: float, alpha: float = 1.0,
             alpha_Q: float = 1.0, epoch_begin: int = 0, epoch_end=None, chains: int = 0,
             staged: bool = False, round_edges: int = 0):
    """Hogwild NCE SGD in place on Y (CUDA float32 [N, d]) and Q (CUDA float32
    scalar tensor); returns (Y, Q).  staged=True draws the noise samples from
    shared-memory windows of Y (ncvis_optimize_staged_device)."""
    plan = np.ascontiguousarray(n_noise, dtype=np.uintp)
    n_epochs = plan.shape[0]
    if epoch_end is None:
        epoch_end = n_epochs
    src, dst = _i32(src), _i32(dst)
    N, d = Y.shape
    assert Y.is_contiguous() and Y.dtype == _torch().float32
    arr = (C.c_size_t * max(1, n_epochs))(*[int(v) for v in plan])
    L = _lib.lib()
    if staged:
        rc = L.ncvis_optimize_staged_device(N, d, src.shape[0], src.data_ptr(), dst.data_ptr(),
                                            Y.data_ptr(), Q.data_ptr(), seed, epoch_begin,
                                            epoch_end, n_epochs, arr, a, b, alpha, alpha_Q,
                                            chains, round_edges, _stream())
    else:
        rc = L.ncvis_optimize_device(N, d, src.shape[0], src.data_ptr(), dst.data_ptr(),
                                     Y.data_ptr(), Q.data_ptr(), seed, epoch_begin, epoch_end,
                                     n_epochs, arr, a, b, alpha, alpha_Q, chains, _stream())
    _lib.check(rc)
    return Y, Q


def optimize_replay(Y, Q, src, dst, stream, stream_offset: int, epoch: int, n_epochs: int,
                    nu: int, a: float, b: float, alpha: float = 1.0, alpha_Q: float = 1.0,
                    edge_begin: int = 0, edge_end=None):
    """One chain replays edges [edge_begin, edge_end) of `epoch` in the
    reference's one-thread order with recorded noise indices; in place."""
    src, dst = _i32(src), _i32(dst)
    stream = _i32(stream)
    N, d = Y.shape
    if edge_end is None:
        edge_end = src.shape[0]
    _lib.check(_lib.lib().ncvis_optimize_replay_device(
        N, d, src.data_ptr(), dst.data_ptr(), edge_begin, edge_end, stream.data_ptr(),
        stream_offset, Y.data_ptr(), Q.data_ptr(), epoch, n_epochs, nu, a, b, alpha, alpha_Q,
        _stream()))
    return Y, Q


def launch_count() -> int:
    return int(_lib.lib().ncvis_kernel_launch_count())
