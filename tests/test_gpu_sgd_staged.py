"""K7 staged-noise optimizer on the GPU (ncvis_optimize_staged_device).

The staged form draws every noise sample of a round from a shared-memory
window of Y (segments of 256 rows at uniform starts) instead of from the
whole array; each sample is still uniform over the other N - 1 rows.

* One chain has a sequential counterpart: oracle/sgd_staged_oracle.py
  restates the same rounds, windows, Philox draws and updates in FP64.  After
  two epochs Y and Q agree to 1e-4 relative (|dY| <= 1e-4 * max(1, max|Y|));
  the GPU evaluates the weights with fast single-precision intrinsics.
* Many chains (the engine's default at N >= 65,536 for d <= 2) are checked
  end to end: trustworthiness at k = 15 within 0.01 of the unstaged
  optimizer's on the same graph and start.
"""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu

A, B = 0.76687364, 1.22256382


def _t(cuda, a, dtype):
    return cuda.tensor(np.ascontiguousarray(a).astype(dtype), device="cuda")


def _graph(N, n_src, per, rng):
    """Edges sorted by source: n_src sources with `per` edges each, one self
    edge and one repeated destination among them."""
    srcs = np.sort(rng.choice(N, n_src, replace=False))
    src = np.repeat(srcs, per)
    dst = rng.integers(0, N, size=src.size)
    dst[3] = src[3]        # a self edge
    dst[5] = dst[4]        # the same destination twice in a row
    dst[per] = src[0]      # a destination that was an earlier source
    return src.astype(np.int32), dst.astype(np.int32)


@pytest.mark.parametrize("d", [1, 2, 4])
def test_one_chain_matches_oracle(cuda, d):
    from ncvis_gb300 import stages
    from oracle.sgd_staged_oracle import optimize_staged_one_chain, window_rows
    rng = np.random.default_rng(11 + d)
    N = 16 * window_rows(d)
    Y0 = rng.normal(0.0, 1.0, size=(N, d)).astype(np.float32)
    src, dst = _graph(N, 30, 4, rng)
    plan = np.array([5, 3], np.uintp)
    alpha = 0.05
    dY = _t(cuda, Y0, np.float32)
    dQ = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    stages.optimize(dY, dQ, _t(cuda, src, np.int32), _t(cuda, dst, np.int32), 9, plan, A, B,
                    alpha=alpha, chains=1, staged=True, round_edges=8)
    Yo, Qo = optimize_staged_one_chain(Y0, 0.0, src, dst, 9, plan, A, B, alpha=alpha,
                                       round_edges=8)
    gy, gq = dY.cpu().numpy(), float(dQ.cpu()[0])
    moved = np.abs(Yo - Y0).max()
    assert moved > 1e-3  # the run changed Y
    err = np.abs(gy - Yo).max() / max(1.0, np.abs(Yo).max())
    assert err <= 1e-4, err
    assert abs(gq - Qo) <= 1e-4 * max(1.0, abs(Qo)), (gq, Qo)


def test_many_chains_quality_matches_unstaged(cuda):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality, stages
    N = 65536
    X, _ = gmm(N, 32, 20, 5.0, seed=3)
    Xd = _t(cuda, X, np.float32)
    inds, dists = stages.knn(Xd, 15, 0)
    rp, cols, _, src = stages.symmetrize(inds, dists)
    Y0 = stages.init_embedding(rp, cols, 2, 42, 20, np.float32(1 / 15))
    plan = ncvis.default_noise_plan(50)
    T = {}
    for staged in (False, True):
        Y = Y0.clone()
        Q = cuda.zeros(1, dtype=cuda.float32, device="cuda")
        stages.optimize(Y, Q, src, cols, 42, plan, A, B, staged=staged)
        assert bool(cuda.isfinite(Y).all())
        T[staged] = quality.trustworthiness_device(Xd, Y, 15, distance=0)
    assert abs(T[True] - T[False]) <= 0.01, T
    assert T[True] > 0.9, T


def test_fit_transform_uses_staged_noise_by_default(cuda):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality
    N = 65536
    X, _ = gmm(N, 32, 20, 5.0, seed=4)
    Xd = _t(cuda, X, np.float32)
    T = {}
    for mode in ("hogwild", "hogwild_unstaged"):
        Y = ncvis.NCVis(random_seed=42, sgd_mode=mode).fit_transform(Xd)
        assert Y.shape == (N, 2) and bool(cuda.isfinite(Y).all())
        T[mode] = quality.trustworthiness_device(Xd, Y, 15, distance=0)
    assert abs(T["hogwild"] - T["hogwild_unstaged"]) <= 0.01, T


def test_rejects_noise_plan_above_bound(cuda):
    """Both optimizer entries refuse a plan entry above 2^24 before any device
    work (the kernels keep sample numbers in 32-bit counters)."""
    from ncvis_gb300 import _lib, stages
    Y = cuda.zeros((70000, 2), dtype=cuda.float32, device="cuda")
    Q = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    src = cuda.zeros(4, dtype=cuda.int32, device="cuda")
    for staged in (False, True):
        with pytest.raises(_lib.NcvisError, match="n_noise entries must be at most"):
            stages.optimize(Y, Q, src, src, 1, np.array([3, (1 << 24) + 1], np.uintp), A, B,
                            staged=staged)


def test_rejects_small_problems_and_wide_embeddings(cuda):
    from ncvis_gb300 import _lib, stages
    for N, d in ((1000, 2), (65536, 5)):
        Y = cuda.zeros((N, d), dtype=cuda.float32, device="cuda")
        Q = cuda.zeros(1, dtype=cuda.float32, device="cuda")
        src = cuda.zeros(4, dtype=cuda.int32, device="cuda")
        with pytest.raises(_lib.NcvisError, match="optimize_staged"):
            stages.optimize(Y, Q, src, src, 1, np.array([1], np.uintp), A, B, staged=True)
