"""The trustworthiness used in the parity bars (ncvis_gb300.quality, which
the GPU metric is tested against) is scikit-learn's definition: equal to
sklearn.manifold.trustworthiness on random data (no distance ties), for
several k and embeddings of different quality.  CPU only; skipped where
scikit-learn is absent."""
import numpy as np
import pytest


@pytest.mark.parametrize("k", [1, 5, 15])
def test_trustworthiness_equals_sklearn(k):
    manifold = pytest.importorskip("sklearn.manifold")
    from ncvis_gb300 import quality
    rng = np.random.default_rng(k)
    X = rng.normal(size=(400, 12))
    for Y in (X[:, :2] + 0.01 * rng.normal(size=(400, 2)),  # a fair embedding
              rng.normal(size=(400, 2))):                      # an unrelated one
        ours = quality.trustworthiness(X, Y, k, device="cpu", block=128)
        ref = manifold.trustworthiness(X, Y, n_neighbors=k)
        assert abs(ours - ref) <= 1e-12, (k, ours, ref)
