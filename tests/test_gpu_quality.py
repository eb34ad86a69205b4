"""Full-size quality metric on the GPU (ncvis_trustworthiness_device) against
the FP64 brute-force trustworthiness of ncvis_gb300.quality (the definition
scikit-learn implements: ranks of each embedding neighbour among the other
points in X)."""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu


def _embed(X, seed):
    """A deterministic, imperfect 2-D embedding: a random projection plus noise."""
    rng = np.random.default_rng(seed)
    P = rng.normal(size=(X.shape[1], 2)).astype(np.float32)
    return (X @ P + rng.normal(0, 0.5, size=(X.shape[0], 2))).astype(np.float32)


@pytest.mark.parametrize("N,D,k", [(1500, 16, 15), (3001, 8, 10), (800, 3, 1)])
def test_trustworthiness_matches_fp64(cuda, N, D, k):
    from ncvis_gb300 import quality
    X, _ = gmm(N, D, 6, 4.0, seed=N)
    Y = _embed(X, N)
    t_gpu = quality.trustworthiness_device(X, Y, k, distance=0)
    t_ref = quality.trustworthiness(X, Y, k)
    assert 0.0 < t_ref < 1.0
    assert abs(t_gpu - t_ref) <= 1e-5, (t_gpu, t_ref)


def test_trustworthiness_cosine_ranks_are_euclidean_ranks_of_unit_vectors(cuda):
    from ncvis_gb300 import quality
    from ncvis_gb300.synthetic import vmf_mixture
    X, _ = vmf_mixture(2000, 24, n_comp=8, kappa=20.0, seed=3)
    Y = _embed(X, 3)
    t_gpu = quality.trustworthiness_device(X, Y, 15, distance=2)
    Xn = X / np.linalg.norm(X, axis=1, keepdims=True)
    t_ref = quality.trustworthiness(Xn, Y, 15)
    assert abs(t_gpu - t_ref) <= 2e-3, (t_gpu, t_ref)


def test_trustworthiness_of_the_data_itself_is_one(cuda):
    from ncvis_gb300 import quality
    rng = np.random.default_rng(0)
    X = rng.normal(size=(1200, 2)).astype(np.float32)
    assert quality.trustworthiness_device(X, X.copy(), 15, distance=0) == pytest.approx(1.0, abs=1e-12)


def test_trustworthiness_rejects_bad_arguments(cuda):
    from ncvis_gb300 import NcvisError, quality
    X = np.zeros((100, 4), np.float32)
    with pytest.raises(NcvisError, match="k must be in"):
        quality.trustworthiness_device(X, X[:, :2].copy(), 17)
    bad = X.copy()
    bad[3, 1] = np.nan
    with pytest.raises(NcvisError, match="non-finite"):
        quality.trustworthiness_device(bad, np.random.default_rng(1).normal(size=(100, 2)), 5)
