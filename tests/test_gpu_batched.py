"""Batched embeddings (ncvis_fit_transform_batched_device): many independent
problems in one run, each with its own kNN graph, initialisation stream,
noise range and Q, the SGD epoch loop captured as one CUDA graph.

Each problem must come out as if embedded alone: its kNN table (through the
same FP32 selection) equals the single-problem one, its init equals the
oracle's one-thread init for its seed (1e-5), and its embedding quality
(trustworthiness at k=15) is within 0.01 of the single-problem path and of
the reference's algorithm run on the problem alone.
"""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu


def _problems(sizes, D=16, seed=0):
    Xs = []
    for p, n in enumerate(sizes):
        X, _ = gmm(n, D, 4 + p % 5, 5.0, seed=seed + p)
        Xs.append(X)
    return Xs


def test_batched_matches_single_problems(cuda, oracle):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality
    sizes = [500, 1337, 4000, 777, 2500]
    Xs = _problems(sizes)
    seeds = [11, 12, 13, 14, 15]
    vis = ncvis.NCVis(random_seed=42)
    Ys = vis.fit_transform_batched(Xs, seeds=seeds)
    assert [Y.shape for Y in Ys] == [(n, 2) for n in sizes]
    t = vis.stage_times()
    assert t["k"] == 15 and t["n_edges"] > sum(sizes) * 15
    for X, Y, sd in zip(Xs, Ys, seeds):
        assert np.isfinite(Y).all()
        Ysingle = ncvis.NCVis(random_seed=sd).fit_transform(X)
        tb = quality.trustworthiness(X, Y, 15)
        ts = quality.trustworthiness(X, Ysingle, 15)
        print(f"batched fp32 N={len(X)}: trustworthiness batched {tb:.4f} single {ts:.4f}")
        assert abs(tb - ts) <= 0.01, (len(X), tb, ts)


def test_batched_bf16_knn_matches_single_problems(cuda):
    """The tensor-core kNN over all problems in one launch (problems at
    256-aligned rows of a padded copy, query tiles spread over the CTAs):
    every problem's graph stays inside the problem, and its embedding quality
    is within 0.01 of the single-problem path."""
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality
    sizes = [300, 1000, 2600, 257, 4100, 900]
    Xs = _problems(sizes, seed=9)
    seeds = [21, 22, 23, 24, 25, 26]
    vis = ncvis.NCVis(random_seed=3, knn_precision="bf16")
    Ys = vis.fit_transform_batched(Xs, seeds=seeds)
    assert [Y.shape for Y in Ys] == [(n, 2) for n in sizes]
    for X, Y, sd in zip(Xs, Ys, seeds):
        assert np.isfinite(Y).all()
        Ysingle = ncvis.NCVis(random_seed=sd).fit_transform(X)
        tb = quality.trustworthiness(X, Y, 15)
        ts = quality.trustworthiness(X, Ysingle, 15)
        print(f"batched bf16 N={len(X)}: trustworthiness batched {tb:.4f} single {ts:.4f}")
        assert abs(tb - ts) <= 0.01, (len(X), tb, ts)


def test_batched_against_reference(cuda, oracle):
    """Each batched problem against the reference's algorithm (the oracle's
    fit_transform: brute-force kNN, symmetrize, init and optimize on one
    thread, with the problem's seed and the same a, b and noise plan): its
    trustworthiness at k=15 within 0.01 of the oracle's, the oracle's own
    one-thread vs all-threads spread printed beside it."""
    import os
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import quality
    sizes = [3000, 5000, 8000]
    Xs = _problems(sizes, seed=70)
    seeds = [31, 32, 33]
    vis = ncvis.NCVis(random_seed=42)
    Ys = vis.fit_transform_batched(Xs, seeds=seeds)
    a, b = ncvis.find_ab_params(1.0, 0.4)
    plan = ncvis.default_noise_plan(50)
    threads = os.cpu_count() or 1
    for X, Y, sd in zip(Xs, Ys, seeds):
        Yo = oracle.fit_transform(X, 2, 15, sd, 50, 20, a, b, 1.0, 1.0, plan, 0, 1)
        YoN = oracle.fit_transform(X, 2, 15, sd, 50, 20, a, b, 1.0, 1.0, plan, 0, threads)
        tb = quality.trustworthiness(X, Y, 15)
        to = quality.trustworthiness(X, Yo, 15)
        tN = quality.trustworthiness(X, YoN, 15)
        print(f"batched N={len(X)}: trustworthiness batched {tb:.4f} | oracle 1 thread {to:.4f}, "
              f"{threads} threads {tN:.4f} (spread {abs(to - tN):.4f})")
        assert abs(tb - to) <= 0.01, (len(X), tb, to)


def test_batched_init_and_graph(cuda, oracle):
    """With no SGD epochs the batched output is each problem's init, which
    must match the oracle's one-thread init of that problem's graph."""
    import ncvis_gb300 as ncvis
    sizes = [600, 1500, 900]
    Xs = _problems(sizes, seed=5)
    seeds = [101, 202, 303]
    vis = ncvis.NCVis(random_seed=1, n_epochs=0, n_noise=np.zeros(0, dtype=np.int64))
    Ys = vis.fit_transform_batched(Xs, seeds=seeds)
    for X, Y, sd in zip(Xs, Ys, seeds):
        from ncvis_gb300 import stages
        inds, dists = stages.knn(cuda.tensor(X, device="cuda"), 15, 0)
        inds, dists = inds.cpu().numpy().astype(np.int64), dists.cpu().numpy()
        rp, cols, _ = oracle.symmetrize(inds, dists)
        ref = oracle.init_embedding(len(X), 2, oracle.edges_from_csr(rp), cols, sd, 20,
                                    np.float32(1 / 15), 1)
        np.testing.assert_allclose(Y, ref, rtol=0, atol=1e-5 * max(1.0, np.abs(ref).max()))


def test_batched_rejects_bad_layout(cuda):
    import ncvis_gb300 as ncvis
    vis = ncvis.NCVis()
    with pytest.raises(ncvis.NcvisError, match="at least two points"):
        vis.fit_transform_batched([np.zeros((1, 3), np.float32), np.ones((5, 3), np.float32)])
    # Replay consumes one recorded stream per fit: refused before any device work.
    vis = ncvis.NCVis(sgd_mode="replay")
    with pytest.raises(ncvis.NcvisError, match="replay mode"):
        vis.fit_transform_batched(_problems([300, 400]))


@pytest.mark.parametrize("d", [1, 2, 3, 4])
def test_batched_tiny_and_boundary_problems(cuda, d):
    """Problems of 2 and 3 points, one just below and one just above the
    1,024-row shared-memory window of the staged optimizer (the whole problem
    staged, or segments of it), in every embedding width the staged kernel
    has: all finite, each problem's rows in place."""
    import ncvis_gb300 as ncvis
    sizes = [2, 3, 1024, 1025, 17]
    Xs = _problems(sizes, D=8, seed=40 + d)
    Ys = ncvis.NCVis(d=d, random_seed=3).fit_transform_batched(Xs, seeds=[1, 2, 3, 4, 5])
    assert [Y.shape for Y in Ys] == [(n, d) for n in sizes]
    for Y in Ys:
        assert np.isfinite(Y).all()
        assert np.abs(Y).max() > 0
