"""Generates the golden fixtures in tests/golden/ from the reference's own
code (oracle/_ref/libncvis_ref.so: the reference's src/ncvis.cpp and
src/knntable.cpp compiled unmodified, with a brute-force hnswlib stand-in and
pyarrow's vendored pcg-cpp; see oracle/build_ref.sh).

Run where the reference checkout exists:
    bash oracle/build_ref.sh && python tests/golden/make_golden.py [out_dir]
(out_dir defaults to this folder; tests/test_golden_regenerate.py writes to a
temporary one and compares).
Every stage runs with one OpenMP thread, the reference's deterministic form.
The fixtures pin the oracle restatement (oracle/) and, through it, the CUDA
engine; they are inputs and outputs only.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

# Python-side defaults of the reference (wrapper/ncvis.pyx:49, 137-141).
A_DEFAULT, B_DEFAULT = 0.76687364, 1.22256382


def ref_knn(R, X, dist, k):
    N, D = X.shape
    inds = np.empty((N, k), np.int64)
    dists = np.empty((N, k), np.float32)
    assert R.ref_knn(np.ascontiguousarray(X, np.float32), N, D, dist, k, 1, inds, dists) == 0
    return inds, dists


def ref_sym(R, inds, dists):
    N, k = inds.shape
    rp = np.empty(N + 1, np.int64)
    cols = np.empty(2 * N * k, np.int64)
    vals = np.empty(2 * N * k, np.float32)
    E = R.ref_symmetrize(N, k, np.ascontiguousarray(inds, np.int64),
                         np.ascontiguousarray(dists, np.float32), 1, rp, cols, vals)
    return rp, cols[:E].copy(), vals[:E].copy()


def main(out_dir: str = HERE):
    R = O.ref()
    if R is None:
        raise SystemExit("oracle/_ref/libncvis_ref.so is missing: run oracle/build_ref.sh first")
    rng = np.random.default_rng(20240601)
    out = {}

    # --- random streams (src/ncvis.cpp:195-200, 281-283, 300)
    for seed, n in [(42, 256), (0, 64), (43, 64)]:
        a = np.empty(n, np.uint64)
        R.ref_pcg64(seed, n, a)
        out[f"pcg64_{seed}"] = a
    u = np.empty(4096, np.float32)
    R.ref_uniform_real(42, 4096, u)
    out["uniform_real_42"] = u
    for seed, hi in [(42, 9999), (7, 2**33 + 5), (11, 1)]:
        v = np.empty(1024, np.uint64)
        R.ref_uniform_int(seed, hi, 1024, v)
        out[f"uniform_int_{seed}_{hi}"] = v
    np.savez_compressed(os.path.join(out_dir, "rng.npz"), **out)

    # --- kNN tables and symmetrization (src/ncvis.cpp:72-153, src/knntable.cpp:24-99)
    sym = {}
    X = rng.normal(size=(300, 8)).astype(np.float32)
    sym["X"] = X
    for dist in range(4):
        inds, dists = ref_knn(R, X, dist, 15)
        sym[f"knn_inds_{dist}"], sym[f"knn_dists_{dist}"] = inds, dists
        rp, cols, vals = ref_sym(R, inds, dists)
        sym[f"sym_rp_{dist}"], sym[f"sym_cols_{dist}"], sym[f"sym_vals_{dist}"] = rp, cols, vals
    # Tie-heavy table: 4 distance levels, symmetric distances for mutual pairs.
    N, k = 200, 10
    inds = np.stack([rng.choice(np.delete(np.arange(N), i), k, replace=False) for i in range(N)])
    level = rng.integers(0, 4, size=(N, N)).astype(np.float32)
    level = np.minimum(level, level.T)
    dists = np.take_along_axis(level, inds, axis=1)
    order = np.argsort(-dists, axis=1, kind="stable")
    inds, dists = np.take_along_axis(inds, order, 1), np.take_along_axis(dists, order, 1)
    sym["ties_inds"], sym["ties_dists"] = inds, dists
    sym["ties_rp"], sym["ties_cols"], sym["ties_vals"] = ref_sym(R, inds, dists)
    # Hub-heavy table: most rows point at a few hubs, so hub rows exceed 64 entries.
    N, k = 400, 12
    hubs = np.arange(8)
    inds = np.empty((N, k), np.int64)
    for i in range(N):
        pool = np.setdiff1d(np.concatenate([hubs, rng.integers(0, N, 20)]), [i])
        inds[i] = rng.choice(np.unique(pool), k, replace=False)
    dists = np.round(rng.random((N, k)).astype(np.float32) * 8) / 8
    order = np.argsort(-dists, axis=1, kind="stable")
    inds, dists = np.take_along_axis(inds, order, 1), np.take_along_axis(dists, order, 1)
    sym["hub_inds"], sym["hub_dists"] = inds, dists.astype(np.float32)
    sym["hub_rp"], sym["hub_cols"], sym["hub_vals"] = ref_sym(R, inds, dists.astype(np.float32))
    # Smallest tables: N=2 (k=1) and N=5 (k=4).
    for N in (2, 5):
        Xs = rng.random((N, 3)).astype(np.float32)
        inds, dists = ref_knn(R, Xs, 0, N - 1)
        sym[f"tiny{N}_inds"], sym[f"tiny{N}_dists"] = inds, dists
        sym[f"tiny{N}_rp"], sym[f"tiny{N}_cols"], sym[f"tiny{N}_vals"] = ref_sym(R, inds, dists)
    np.savez_compressed(os.path.join(out_dir, "symmetrize.npz"), **sym)

    # --- init_embedding and optimize on the L2 graph above (src/ncvis.cpp:184-352)
    rp, cols = sym["sym_rp_0"], sym["sym_cols_0"]
    N = rp.shape[0] - 1
    src = O.edges_from_csr(rp)
    emb = {"rp": rp, "cols": cols}
    for d, n_init in [(2, 20), (2, 1), (1, 20), (5, 3)]:
        Y = np.empty((N, d), np.float32)
        R.ref_init_embedding(N, d, src.shape[0], src, cols, 42, n_init, np.float32(1 / 15), 1, Y)
        emb[f"init_d{d}_e{n_init}"] = Y
    plan = O.noise_plan(50)
    emb["plan"] = plan
    for d in (2, 5):
        Y0 = emb[f"init_d{d}_e20"] if d == 2 else emb["init_d5_e3"]
        Y = Y0.copy()
        q = C.c_float(0.0)
        R.ref_optimize(N, d, src.shape[0], src, cols, 42, 50, plan, A_DEFAULT, B_DEFAULT, 1.0, 1.0,
                       1, Y, C.byref(q))
        emb[f"opt_d{d}_Y"], emb[f"opt_d{d}_Q"] = Y, np.float32(q.value)
    np.savez_compressed(os.path.join(out_dir, "embedding.npz"), **emb)

    # --- the whole pipeline (src/ncvis.cpp:354-459)
    fit = {}
    Xf = rng.normal(size=(200, 5)).astype(np.float32)
    fit["X"] = Xf
    for dist in range(4):
        Y = np.empty((200, 2), np.float32)
        assert R.ref_fit_transform(Xf, 200, 5, 2, 1, 15, 42, 50, 20, A_DEFAULT, B_DEFAULT, 1.0,
                                   1.0, plan, dist, Y) == 0
        fit[f"Y_{dist}"] = Y
    np.savez_compressed(os.path.join(out_dir, "fit.npz"), **fit)
    for f in sorted(os.listdir(out_dir)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(out_dir, f)), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
