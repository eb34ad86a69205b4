"""End-to-end fit_transform through the drop-in APIs.

* The reference's own behaviour tests (recipe/test.py:7-111), unchanged in
  their assertions: all four distances give finite output on 5 points in 3-D;
  the 1-D two-cluster split holds for the default kernel and for a = b = 1;
  n_threads is accepted (the GPU ignores it).
* Parity on the 10k-point, 64-D, 10-component Gaussian mixture at the
  reference's defaults: trustworthiness and kNN preservation at k=15 of the
  GPU's embedding within 0.01 of the oracle's (the reference's algorithm on
  the CPU with one thread), with the oracle's own run-to-run spread over
  thread counts printed beside it.
* Host-buffer and device-buffer entry points, replay mode, error messages.
"""
import time

import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu


def _ncvis():
    import ncvis_gb300 as ncvis
    return ncvis


def test_distances(cuda):
    ncvis = _ncvis()
    np.random.seed(42)
    X = np.random.random((5, 3))
    for distance in ["euclidean", "cosine", "correlation", "inner_product"]:
        vis = ncvis.NCVis(n_neighbors=15, M=16, ef_construction=200, random_seed=42,
                          n_init_epochs=20, n_epochs=50, min_dist=0.4, n_threads=-1,
                          distance=distance)
        Y = vis.fit_transform(X)
        assert np.all(np.isfinite(Y)), "All entries must be finite"


def test_threads_accepted(cuda):
    ncvis = _ncvis()
    np.random.seed(42)
    X = np.random.random((5 * 10**3, 10))
    for distance in ["euclidean", "cosine", "correlation", "inner_product"]:
        for n_th in (1, 2):
            vis = ncvis.NCVis(n_neighbors=15, M=16, ef_construction=200, random_seed=42,
                              n_init_epochs=20, n_epochs=50, min_dist=0.4, n_threads=n_th,
                              distance=distance)
            t = time.time()
            Y = vis.fit_transform(X)
            assert np.isfinite(Y).all()
            print(f"{distance}: n_threads = {n_th}, time = {time.time() - t:.3f}s")


def _two_clusters():
    np.random.seed(42)
    n = 50
    return n, np.concatenate((np.random.normal(-1, 1.5, (n, 1)), np.random.normal(1, 1.5, (n, 1))))


def test_1d_clustering(cuda):
    ncvis = _ncvis()
    n, X = _two_clusters()
    vis = ncvis.NCVis(n_neighbors=15, M=16, ef_construction=200, d=1, n_init_epochs=20,
                      n_epochs=50, min_dist=0.4, n_threads=-1, distance="euclidean",
                      random_seed=42)
    Y = vis.fit_transform(X).ravel()
    n_pos = np.count_nonzero(Y - Y.mean() > 0)
    assert np.abs(n_pos - n) < 5, "Clustering quality is too poor"


def test_1d_tsne(cuda):
    ncvis = _ncvis()
    n, X = _two_clusters()
    vis = ncvis.NCVis(n_neighbors=15, M=16, ef_construction=200, d=1, n_init_epochs=20,
                      n_epochs=50, a=1, b=1, n_threads=-1, distance="euclidean", random_seed=42)
    Y = vis.fit_transform(X).ravel()
    n_pos = np.count_nonzero(Y - Y.mean() > 0)
    assert np.abs(n_pos - n) < 5, "Clustering quality is too poor"


def test_reference_errors(cuda):
    ncvis = _ncvis()
    vis = ncvis.NCVis()
    with pytest.raises(ncvis.NcvisError, match="at least one element"):
        vis.fit_transform(np.zeros((0, 3), np.float32))
    with pytest.raises(ncvis.NcvisError, match="at least two elements"):
        vis.fit_transform(np.zeros((1, 3), np.float32))


def test_quality_parity_10k(cuda, oracle):
    """Trustworthiness / kNN preservation at k=15 within 0.01 of the oracle."""
    ncvis = _ncvis()
    from ncvis_gb300 import quality
    X, _ = gmm(10000, 64, 10, 5.0, seed=42)
    a, b = ncvis.find_ab_params(1.0, 0.4)
    plan = ncvis.default_noise_plan(50)
    vis = ncvis.NCVis(random_seed=42)
    t = time.time()
    Yg = vis.fit_transform(X)
    t_gpu = time.time() - t
    times = vis.stage_times()
    Yo = oracle.fit_transform(X, d=2, n_neighbors=15, seed=42, n_epochs=50, n_init_epochs=20,
                              a=a, b=b, n_noise=plan, dist=0, n_threads=1)
    Yo8 = oracle.fit_transform(X, d=2, n_neighbors=15, seed=42, n_epochs=50, n_init_epochs=20,
                               a=a, b=b, n_noise=plan, dist=0, n_threads=8)
    tg, to, to8 = (quality.trustworthiness(X, Y, 15) for Y in (Yg, Yo, Yo8))
    pg, po, po8 = (quality.knn_preservation(X, Y, 15) for Y in (Yg, Yo, Yo8))
    print(f"trustworthiness gpu {tg:.4f} oracle(1t) {to:.4f} oracle(8t) {to8:.4f}; "
          f"kNN preservation gpu {pg:.4f} oracle(1t) {po:.4f} oracle(8t) {po8:.4f}; "
          f"gpu wall {t_gpu:.3f}s stages {times}")
    assert abs(tg - to) <= 0.01
    assert abs(pg - po) <= 0.01


def test_host_and_device_entry_points(cuda):
    ncvis = _ncvis()
    from ncvis_gb300 import quality
    X, _ = gmm(4000, 16, 5, 5.0, seed=3)
    vis = ncvis.NCVis(random_seed=3)
    Yh = vis.fit_transform(X)
    Yd = vis.fit_transform(cuda.tensor(X, device="cuda"))
    assert Yd.is_cuda and Yd.shape == (4000, 2)
    th = quality.trustworthiness(X, Yh, 15)
    td = quality.trustworthiness(X, Yd.cpu().numpy(), 15)
    assert abs(th - td) < 0.01
    t = vis.stage_times()
    assert t["n_edges"] > 4000 * 15 and t["k"] == 15 and t["total_ms"] > 0


def test_replay_mode_end_to_end(cuda, oracle):
    """fit_transform in replay mode consumes the one-thread noise stream of
    the same graph and is deterministic."""
    ncvis = _ncvis()
    X, _ = gmm(600, 8, 4, 6.0, seed=11)
    inds, dists = oracle.knn(oracle.preprocess(X, 0), 0, 15)
    rp, cols, _ = oracle.symmetrize(inds, dists)
    src = oracle.edges_from_csr(rp)
    plan = ncvis.default_noise_plan(50)
    stream = oracle.negative_stream(600, src, 42, plan)
    vis = ncvis.NCVis(random_seed=42, sgd_mode="replay", replay_stream=stream)
    Y1 = vis.fit_transform(X)
    Y2 = vis.fit_transform(X)
    assert vis.stage_times()["n_edges"] == src.size
    assert np.array_equal(Y1, Y2)
    assert np.isfinite(Y1).all()
