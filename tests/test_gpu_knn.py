"""kNN stage on the GPU (K1 preprocess + K3 FP32 selection + K4 rerank)
against the oracle's exact kNN with the reference's row contract
(src/ncvis.cpp:128-153): k+1 nearest by (distance, index), nearest dropped,
descending order.

Tolerances: index sets must agree with the FP64 oracle except where two
candidates' distances differ by less than FP32 rounding (recall >= 0.999 on
random data); the returned distances must equal the oracle's FP32 distance
of the same pair to 1e-5 relative (summation order differs)."""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu


def _run(cuda, X, k, dist):
    from ncvis_gb300 import stages
    inds, dists = stages.knn(cuda.tensor(X, device="cuda"), k, dist)
    return inds.cpu().numpy().astype(np.int64), dists.cpu().numpy()


def _exact_pair(oracle, Xp, i, j, dist):
    a, b = Xp[i].astype(np.float64), Xp[j].astype(np.float64)
    return ((a - b) ** 2).sum() if dist == 0 else 1.0 - (a * b).sum()


@pytest.mark.parametrize("dist", [0, 1, 2, 3])
def test_knn_matches_fp64_oracle(cuda, oracle, dist):
    X, _ = gmm(3000, 24, 6, 3.0, seed=dist)
    k = 15
    gi, gd = _run(cuda, X, k, dist)
    Xp = oracle.preprocess(X, dist)
    oi, od = oracle.knn(Xp, dist, k, use_f64=True)
    recall = np.mean([len(np.intersect1d(a, b)) / k for a, b in zip(gi, oi)])
    assert recall >= 0.999, recall
    assert np.all(np.diff(gd, axis=1) <= 0), "rows must be in descending distance order"
    for i in range(0, 3000, 97):
        for j in range(k):
            ref = _exact_pair(oracle, Xp, i, gi[i, j], dist)
            assert abs(gd[i, j] - ref) <= 1e-5 * max(1.0, abs(ref))
    # every index is a valid point and not repeated within a row
    assert gi.min() >= 0 and gi.max() < 3000
    assert all(len(np.unique(r)) == k for r in gi)


@pytest.mark.parametrize("N,D,k", [(2, 3, 1), (5, 3, 4), (17, 1, 15), (300, 300, 15), (1000, 7, 30)])
def test_knn_shapes(cuda, oracle, N, D, k):
    rng = np.random.default_rng(N * 31 + D)
    X = rng.normal(size=(N, D)).astype(np.float32)
    k = min(k, N - 1)
    gi, gd = _run(cuda, X, k, 0)
    oi, od = oracle.knn(oracle.preprocess(X, 0), 0, k, use_f64=True)
    recall = np.mean([len(np.intersect1d(a, b)) / k for a, b in zip(gi, oi)])
    assert recall >= 0.999
    np.testing.assert_allclose(gd, od, rtol=1e-5, atol=1e-5)


def test_knn_duplicates_tie_order(cuda, oracle):
    """Exact duplicates tie at distance 0: the pair order (distance, index)
    decides, as the reference's max-heap of (distance, label) does."""
    rng = np.random.default_rng(3)
    base = rng.normal(size=(50, 4)).astype(np.float32)
    X = np.concatenate([base, base, base[:10]])  # 110 points, many exact twins
    gi, gd = _run(cuda, X, 5, 0)
    oi, od = oracle.knn(oracle.preprocess(X, 0), 0, 5, use_f64=False)
    assert np.array_equal(gi, oi)
    np.testing.assert_allclose(gd, od, rtol=1e-6, atol=0)


def test_knn_rejects_nonfinite(cuda):
    from ncvis_gb300 import NcvisError
    X = np.ones((10, 3), np.float32)
    X[4, 1] = np.nan
    with pytest.raises(NcvisError, match="non-finite"):
        _run(cuda, X, 3, 0)
