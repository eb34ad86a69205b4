"""ORACLE — test infrastructure, not product code.

numpy front end for the CPU restatement in ``ncvis_oracle.cpp`` (built into
``oracle/liboracle.so``) and, where the reference checkout exists, for the
reference's own code in ``oracle/_ref/libncvis_ref.so``.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module;
the engine in ``ncvis_gb300`` never does.

Distances follow ``ncvis::Distance`` (src/ncvis.hpp:27-32): 0 squared_L2,
1 inner_product, 2 cosine_similarity, 3 correlation.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libncvis_ref.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_sz = C.c_size_t

_lib = None
_ref = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (seconds)."""
    sources = ["ncvis_oracle.cpp", "ncvis_oracle_sgd.cpp", "oracle_rng.h", "build_oracle.sh"]
    newest = max(os.path.getmtime(os.path.join(HERE, f)) for f in sources)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_pcg64.argtypes = [C.c_uint64, _sz, _u64p]
        L.orc_uniform_real.argtypes = [C.c_uint64, _sz, _f32p]
        L.orc_uniform_int.argtypes = [C.c_uint64, C.c_uint64, _sz, _u64p]
        L.orc_preprocess.argtypes = [_f32p, _sz, _sz, C.c_int, _f32p]
        L.orc_knn.argtypes = [_f32p, _sz, _sz, C.c_int, _sz, C.c_int, C.c_int, _i64p, _f32p]
        L.orc_symmetrize.argtypes = [_sz, _sz, _i64p, _f32p, C.c_int, _i64p, _i64p, _f32p]
        L.orc_symmetrize.restype = _sz
        L.orc_init_embedding.argtypes = [_sz, _sz, _sz, _i64p, _i64p, C.c_uint64, C.c_int,
                                         C.c_float, C.c_int, _f32p]
        L.orc_init_embedding_stats.argtypes = [_sz, _sz, _sz, _i64p, _i64p, C.c_uint64, C.c_int,
                                               C.c_float, C.c_int, C.c_int, _f32p]
        L.orc_negative_stream.argtypes = [_sz, _sz, _i64p, C.c_uint64, C.c_int, _u64p, _i32p]
        L.orc_negative_stream.restype = _sz
        L.orc_optimize.argtypes = [_sz, _sz, _sz, _i64p, _i64p, _f32p, C.POINTER(C.c_float),
                                   C.c_uint64, C.c_int, C.c_int, C.c_int, _u64p, C.c_float,
                                   C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]
        L.orc_optimize_block.argtypes = [_sz, _i64p, _i64p, _f32p, C.POINTER(C.c_float), C.c_int,
                                         C.c_int, C.c_uint64, _sz, _sz, _i32p, _sz, C.c_float,
                                         C.c_float, C.c_float, C.c_float]
        L.orc_optimize_block.restype = _sz
        L.orc_fit_transform.argtypes = [_f32p, _sz, _sz, _sz, C.c_int, _sz, C.c_uint64, C.c_int,
                                        C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                        _u64p, C.c_int, _f32p]
        L.orc_fit_transform.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own code (oracle/_ref), or None where it was not built."""
    global _ref
    if _ref is None and ref_available():
        R = C.CDLL(REF_PATH)
        R.ref_knn.argtypes = [_f32p, _sz, _sz, C.c_int, _sz, C.c_int, _i64p, _f32p]
        R.ref_knn.restype = C.c_int
        R.ref_symmetrize.argtypes = [_sz, _sz, _i64p, _f32p, C.c_int, _i64p, _i64p, _f32p]
        R.ref_symmetrize.restype = _sz
        R.ref_build_edges.argtypes = [_sz, _i64p, _i64p, _i64p, _i64p]
        R.ref_init_embedding.argtypes = [_sz, _sz, _sz, _i64p, _i64p, C.c_uint64, C.c_int,
                                         C.c_float, C.c_int, _f32p]
        R.ref_optimize.argtypes = [_sz, _sz, _sz, _i64p, _i64p, C.c_uint64, C.c_int, _u64p,
                                   C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, _f32p,
                                   C.POINTER(C.c_float)]
        R.ref_fit_transform.argtypes = [_f32p, _sz, _sz, _sz, C.c_int, _sz, C.c_uint64, C.c_int,
                                        C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                        _u64p, C.c_int, _f32p]
        R.ref_fit_transform.restype = C.c_int
        R.ref_pcg64.argtypes = [C.c_uint64, _sz, _u64p]
        R.ref_uniform_real.argtypes = [C.c_uint64, _sz, _f32p]
        R.ref_uniform_int.argtypes = [C.c_uint64, C.c_uint64, _sz, _u64p]
        _ref = R
    return _ref


# ----------------------------------------------------------------- wrappers

def pcg64(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.uint64)
    lib().orc_pcg64(seed, n, out)
    return out


def uniform_real(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().orc_uniform_real(seed, n, out)
    return out


def uniform_int(seed: int, hi: int, n: int) -> np.ndarray:
    out = np.empty(n, np.uint64)
    lib().orc_uniform_int(seed, hi, n, out)
    return out


def preprocess(X: np.ndarray, dist: int) -> np.ndarray:
    X = np.ascontiguousarray(X, np.float32)
    out = np.empty_like(X)
    lib().orc_preprocess(X, X.shape[0], X.shape[1], dist, out)
    return out


def knn(Xp: np.ndarray, dist: int, k: int, use_f64: bool = False, n_threads: int = 0):
    """Exact kNN table (N x k) of preprocessed points, reference row contract."""
    Xp = np.ascontiguousarray(Xp, np.float32)
    N, D = Xp.shape
    inds = np.empty((N, k), np.int64)
    dists = np.empty((N, k), np.float32)
    lib().orc_knn(Xp, N, D, dist, k, int(use_f64), n_threads or os.cpu_count(), inds, dists)
    return inds, dists


def symmetrize(inds: np.ndarray, dists: np.ndarray, n_threads: int = 0):
    """One-thread reference symmetrization → (row_ptr[N+1], cols[E], vals[E])."""
    inds = np.ascontiguousarray(inds, np.int64)
    dists = np.ascontiguousarray(dists, np.float32)
    N, k = inds.shape
    row_ptr = np.empty(N + 1, np.int64)
    cols = np.empty(2 * N * k, np.int64)
    vals = np.empty(2 * N * k, np.float32)
    E = lib().orc_symmetrize(N, k, inds, dists, n_threads or os.cpu_count(), row_ptr, cols, vals)
    return row_ptr, cols[:E].copy(), vals[:E].copy()


def edges_from_csr(row_ptr: np.ndarray) -> np.ndarray:
    """Source index of each CSR entry (build_edges order, src/ncvis.cpp:155-173)."""
    N = row_ptr.shape[0] - 1
    return np.repeat(np.arange(N, dtype=np.int64), np.diff(row_ptr))


def init_embedding(N: int, d: int, src, dst, seed: int, n_init_epochs: int, alpha: float,
                   n_threads: int = 1, stats64: bool = False) -> np.ndarray:
    """init_embedding as the reference computes it (src/ncvis.cpp:184-273);
    stats64: one thread with the per-dimension sums in double, rounded once
    (the checker of the engine's default statistics)."""
    src = np.ascontiguousarray(src, np.int64)
    dst = np.ascontiguousarray(dst, np.int64)
    Y = np.empty((N, d), np.float32)
    lib().orc_init_embedding_stats(N, d, src.shape[0], src, dst, seed, n_init_epochs, alpha,
                                   n_threads, int(bool(stats64)), Y)
    return Y


def negative_stream(N: int, src, seed: int, n_noise) -> np.ndarray:
    src = np.ascontiguousarray(src, np.int64)
    plan = np.ascontiguousarray(n_noise, np.uint64)
    total = int(src.shape[0]) * int(plan.sum())
    out = np.empty(max(total, 1), np.int32)
    n = lib().orc_negative_stream(N, src.shape[0], src, seed, plan.shape[0], plan, out)
    assert n == total
    return out[:total]


def optimize(Y: np.ndarray, Q: float, src, dst, seed: int, n_noise, a: float, b: float,
             alpha: float = 1.0, alpha_Q: float = 1.0, epoch_begin: int = 0,
             epoch_end: int | None = None, n_threads: int = 1, stream=None):
    """Reference SGD over epochs [epoch_begin, epoch_end); returns (Y, Q) copies."""
    Y = np.ascontiguousarray(Y, np.float32).copy()
    N, d = Y.shape
    src = np.ascontiguousarray(src, np.int64)
    dst = np.ascontiguousarray(dst, np.int64)
    plan = np.ascontiguousarray(n_noise, np.uint64)
    n_epochs = plan.shape[0]
    if epoch_end is None:
        epoch_end = n_epochs
    q = C.c_float(Q)
    sp = None
    if stream is not None:
        stream = np.ascontiguousarray(stream, np.int32)
        sp = stream.ctypes.data_as(C.c_void_p)
    lib().orc_optimize(N, d, src.shape[0], src, dst, Y, C.byref(q), seed, epoch_begin, epoch_end,
                       n_epochs, plan, a, b, alpha, alpha_Q, n_threads, sp)
    return Y, q.value


def optimize_block(Y: np.ndarray, Qc: float, src, dst, epoch: int, n_epochs: int, nu: int,
                   edge_begin: int, edge_end: int, stream, stream_pos: int, a: float, b: float,
                   alpha: float = 1.0, alpha_Q: float = 1.0):
    """One replay step of the one-thread optimizer; returns (Y, Qc, stream_pos)."""
    Y = np.ascontiguousarray(Y, np.float32).copy()
    q = C.c_float(Qc)
    pos = lib().orc_optimize_block(Y.shape[1], np.ascontiguousarray(src, np.int64),
                                   np.ascontiguousarray(dst, np.int64), Y, C.byref(q), epoch,
                                   n_epochs, nu, edge_begin, edge_end,
                                   np.ascontiguousarray(stream, np.int32), stream_pos, a, b,
                                   alpha, alpha_Q)
    return Y, q.value, pos


def fit_transform(X: np.ndarray, d: int = 2, n_neighbors: int = 15, seed: int = 42,
                  n_epochs: int = 50, n_init_epochs: int = 20, a: float = 1.0, b: float = 1.0,
                  alpha: float = 1.0, alpha_Q: float = 1.0, n_noise=None, dist: int = 0,
                  n_threads: int = 1) -> np.ndarray:
    X = np.ascontiguousarray(X, np.float32)
    N, D = X.shape
    plan = np.full(n_epochs, 3, np.uint64) if n_noise is None else np.ascontiguousarray(
        n_noise, np.uint64)
    Y = np.empty((N, d), np.float32)
    rc = lib().orc_fit_transform(X, N, D, d, n_threads, n_neighbors, seed, plan.shape[0],
                                 n_init_epochs, a, b, alpha, alpha_Q, plan, dist, Y)
    if rc != 0:
        raise RuntimeError(f"oracle fit_transform failed ({rc})")
    return Y


# ------------------------------------------------------------ policy (Python)

def noise_plan(n_epochs: int = 50, n_negative: int = 5) -> np.ndarray:
    """Default noise schedule of wrapper/ncvis.pyx:103-112."""
    plan = np.linspace(0, 1, n_epochs) ** 3
    plan /= plan.sum()
    plan *= n_epochs * n_negative
    plan = plan.round().astype(np.uintp)
    plan[plan < 1] = 1
    return plan.astype(np.uint64)
