"""K10 approximate kNN (inverted file on the tensor cores) + K4 exact rerank.

The search is approximate (as the reference's hnswlib search is), so the bars
are recall@15 against FP64 exact search and the row contract:
* 131,072 x 64 Gaussian mixture (64 components; squared L2), default cells
  (256) and probes (32): recall >= 0.99 on a 2000-query sample;
* 131,072 x 100 vMF (cosine; kappa = 50 in 100 dimensions leaves a point's
  nearest neighbours spread over many k-means cells): 64 of 256 cells probed
  (the most a cell lists) give recall >= 0.92, the value a CPU simulation of
  the same partition gives (0.936);
* all four distances on a 20,000 x 32 Gaussian mixture with 64 cells and 8
  probes: recall >= 0.95;
* probing every cell (or a single cell) searches every point, so the rows
  equal the exact BF16 path's (same BF16 selection, same exact rerank): this
  holds the work-list mechanics (query tiles spanning many items, candidate
  ranges masked at both ends, the row map back to original numbering) to the
  exact kernel;
* every returned distance equals its pair's FP32 distance to 1e-5 relative,
  rows descending, indices valid and distinct."""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu


def _ivf(cuda, X, k, dist, lists=0, probe=0, rf=0):
    from ncvis_gb300 import stages
    i, d = stages.knn_ivf(cuda.tensor(X, device="cuda"), k, dist, lists=lists, probe=probe,
                          rerank_factor=rf)
    return i.cpu().numpy().astype(np.int64), d.cpu().numpy()


def _exact_bf16(cuda, X, k, dist, rf=0):
    from ncvis_gb300 import stages
    i, d = stages.knn(cuda.tensor(X, device="cuda"), k, dist, precision=1, rerank_factor=rf)
    return i.cpu().numpy().astype(np.int64), d.cpu().numpy()


def _fp64_rows(Xp, queries, k, dist):
    Xd = Xp.astype(np.float64)
    out = []
    for s in range(0, len(queries), 512):
        q = queries[s:s + 512]
        if dist == 0:
            d = (Xd[q] ** 2).sum(1)[:, None] + (Xd ** 2).sum(1)[None, :] - 2 * Xd[q] @ Xd.T
        else:
            d = 1.0 - Xd[q] @ Xd.T
        part = np.argpartition(d, k + 1, axis=1)[:, :k + 2]
        for r in range(len(q)):
            c = part[r]
            order = np.lexsort((c, d[r, c]))[:k + 1]
            out.append(c[order][1:])
    return np.array(out)


def _recall(found, exact):
    return np.mean([len(np.intersect1d(a, b)) / len(b) for a, b in zip(found, exact)])


def _contract(Xp, gi, gd, dist, N, sample):
    assert gi.min() >= 0 and gi.max() < N
    assert all(len(np.unique(r)) == gi.shape[1] for r in gi[sample])
    assert np.all(np.diff(gd, axis=1) <= 0)
    for i in sample[::40]:
        for j in range(gi.shape[1]):
            a, b = Xp[i].astype(np.float64), Xp[gi[i, j]].astype(np.float64)
            ref = ((a - b) ** 2).sum() if dist == 0 else 1.0 - (a * b).sum()
            assert abs(gd[i, j] - ref) <= 1e-5 * max(1.0, abs(ref))


def test_gmm_131072_recall(cuda, oracle):
    N = 131072
    X, _ = gmm(N, 64, 64, 5.0, seed=7)
    gi, gd = _ivf(cuda, X, 15, 0)
    rng = np.random.default_rng(0)
    q = np.sort(rng.choice(N, 2000, replace=False))
    Xp = oracle.preprocess(X, 0)
    r = _recall(gi[q], _fp64_rows(Xp, q, 15, 0))
    print(f"recall@15 (IVF, 131072 x 64 Gaussian mixture, default cells/probes): {r:.5f}")
    assert r >= 0.99, r
    _contract(Xp, gi, gd, 0, N, q)


def test_vmf_131072_recall(cuda, oracle):
    from ncvis_gb300.synthetic import vmf_mixture
    N = 131072
    X, _ = vmf_mixture(N, 100, n_comp=32, kappa=50.0, seed=42)
    gi, gd = _ivf(cuda, X, 15, 2, lists=256, probe=64)
    rng = np.random.default_rng(0)
    q = np.sort(rng.choice(N, 2000, replace=False))
    Xp = oracle.preprocess(X, 2)
    r = _recall(gi[q], _fp64_rows(Xp, q, 15, 2))
    print(f"recall@15 (IVF, 131072 x 100 vMF, 256 cells, 64 probes): {r:.5f}")
    assert r >= 0.92, r
    _contract(Xp, gi, gd, 2, N, q)


@pytest.mark.parametrize("dist", [0, 1, 2, 3])
def test_distances(cuda, oracle, dist):
    N = 20000
    X, lab = gmm(N, 32, 24, 4.0, seed=50 + dist)
    rng = np.random.default_rng(60 + dist)
    X = (X * rng.uniform(0.5, 2.0, size=24)[lab][:, None] + 2.0).astype(np.float32)
    gi, gd = _ivf(cuda, X, 15, dist, lists=64, probe=8)
    q = np.sort(rng.choice(N, 1000, replace=False))
    Xp = oracle.preprocess(X, dist)
    r = _recall(gi[q], _fp64_rows(Xp, q, 15, dist))
    print(f"recall@15 (IVF, 64 cells, 8 probes, distance {dist}): {r:.5f}")
    assert r >= 0.95, r
    _contract(Xp, gi, gd, dist, N, q)


@pytest.mark.parametrize("N,D,dist,lists,probe,rf", [
    (5000, 24, 2, 16, 16, 2),    # every cell probed: many items per query tile
    (5000, 24, 0, 16, 16, 4),    # folded squared L2, 64 candidates
    (3001, 100, 2, 1, 1, 2),     # one cell
    (777, 7, 3, 5, 5, 2),        # small and ragged
])
def test_all_cells_equal_exact(cuda, N, D, dist, lists, probe, rf):
    rng = np.random.default_rng(N + D)
    X = rng.normal(size=(N, D)).astype(np.float32)
    gi, gd = _ivf(cuda, X, 15, dist, lists=lists, probe=probe, rf=rf)
    ei, ed = _exact_bf16(cuda, X, 15, dist, rf=rf)
    same = np.mean([np.array_equal(np.sort(a), np.sort(b)) for a, b in zip(gi, ei)])
    assert same >= 0.999, same
    assert np.allclose(gd, ed, rtol=1e-6, atol=1e-6)


def test_fit_transform_ivf(cuda):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality
    from ncvis_gb300.synthetic import vmf_mixture
    X, _ = vmf_mixture(65536, 64, n_comp=32, kappa=50.0, seed=5)
    Xd = cuda.tensor(X, device="cuda")
    T = {}
    for prec in ("bf16", "ivf"):
        Y = ncvis.NCVis(distance="cosine", knn_precision=prec, random_seed=42).fit_transform(Xd)
        assert bool(cuda.isfinite(Y).all())
        T[prec] = quality.trustworthiness_device(Xd, Y, 15, distance=2)
    print("trustworthiness", T)
    assert abs(T["ivf"] - T["bf16"]) <= 0.01, T


def test_rejects_unfolded_squared_l2(cuda):
    from ncvis_gb300 import _lib
    X = np.random.default_rng(3).normal(size=(600, 127)).astype(np.float32)
    with pytest.raises(_lib.NcvisError, match="ivf"):
        _ivf(cuda, X, 5, 0)


@pytest.mark.parametrize("N", [2, 5, 40, 300])
def test_tiny_inputs_equal_exact(cuda, N):
    """Tiny inputs: one or a few cells; every cell probed by default, so the
    rows equal the exact BF16 search's."""
    X = np.random.default_rng(N).normal(size=(N, 12)).astype(np.float32)
    k = min(15, N - 1)
    gi, gd = _ivf(cuda, X, k, 2)
    ei, ed = _exact_bf16(cuda, X, k, 2)
    assert all(np.array_equal(np.sort(a), np.sort(b)) for a, b in zip(gi, ei))
    assert np.allclose(gd, ed, rtol=1e-6, atol=1e-6)
