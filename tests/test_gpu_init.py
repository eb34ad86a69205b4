"""K6 init_embedding on the GPU against the reference (golden fixtures) and
the oracle (src/ncvis.cpp:184-273).

The uniform start is the one-thread pcg64(seed) stream and must be
bit-exact.  After standardisation epochs the GPU's FP64 mean/variance
reductions and IEEE division differ from the reference's sequential FP32 sums
and reciprocal-based division in the last bits; tolerance: |dY| <= 1e-5 *
max(1, max|Y|)."""
import numpy as np
import pytest

from conftest import gmm, golden

pytestmark = pytest.mark.gpu


def _gpu_init(cuda, rp, cols, d, seed, n_init, alpha):
    from ncvis_gb300 import stages
    Y = stages.init_embedding(cuda.tensor(rp.astype(np.int64), device="cuda"),
                              cuda.tensor(cols.astype(np.int32), device="cuda"), d, seed, n_init,
                              alpha)
    return Y.cpu().numpy()


def test_uniform_start_bit_exact(cuda, oracle):
    g = golden("embedding.npz")
    rp, cols = g["rp"], g["cols"]
    N = rp.size - 1
    for d in (1, 2, 3):
        Y = _gpu_init(cuda, rp, cols, d, 42, 0, 1 / 15)
        ref = oracle.uniform_real(42, N * d).reshape(N, d)
        assert np.array_equal(Y.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("d,n_init", [(2, 20), (2, 1), (1, 20), (5, 3)])
def test_golden(cuda, d, n_init):
    g = golden("embedding.npz")
    ref = g[f"init_d{d}_e{n_init}"]
    Y = _gpu_init(cuda, g["rp"], g["cols"], d, 42, n_init, np.float32(1 / 15))
    np.testing.assert_allclose(Y, ref, rtol=0, atol=1e-5 * max(1.0, np.abs(ref).max()))


def test_large_graph(cuda, oracle):
    X, _ = gmm(20000, 16, 10, 5.0, seed=1)
    inds, dists = oracle.knn(oracle.preprocess(X, 0), 0, 15)
    rp, cols, _ = oracle.symmetrize(inds, dists)
    src = oracle.edges_from_csr(rp)
    ref = oracle.init_embedding(20000, 2, src, cols, 1234, 20, np.float32(1 / 15), 1)
    Y = _gpu_init(cuda, rp, cols, 2, 1234, 20, np.float32(1 / 15))
    np.testing.assert_allclose(Y, ref, rtol=0, atol=1e-5 * max(1.0, np.abs(ref).max()))


def test_sequential_statistics(cuda, oracle):
    """The statistics summed as the reference's one thread sums them (FP32,
    rows in order) track the oracle's init at 1e-6 (and the default FP64
    statistics the oracle's double sums)."""
    X, _ = gmm(30000, 16, 10, 5.0, seed=2)
    inds, dists = oracle.knn(oracle.preprocess(X, 0), 0, 15)
    rp, cols, _ = oracle.symmetrize(inds, dists)
    src = oracle.edges_from_csr(rp)
    alpha = np.float32(1 / 15)
    from ncvis_gb300 import stages
    t_rp = cuda.tensor(rp.astype(np.int64), device="cuda")
    t_cols = cuda.tensor(cols.astype(np.int32), device="cuda")
    for d in (1, 2, 5):
        ref = oracle.init_embedding(30000, d, src, cols, 7, 20, alpha, 1)
        ref64 = oracle.init_embedding(30000, d, src, cols, 7, 20, alpha, 1, stats64=True)
        Ys = stages.init_embedding(t_rp, t_cols, d, 7, 20, alpha, sequential_stats=True)
        Yd = stages.init_embedding(t_rp, t_cols, d, 7, 20, alpha)
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(Ys.cpu().numpy() - ref).max() <= 1e-6 * scale
        assert np.abs(Yd.cpu().numpy() - ref64).max() <= 1e-6 * scale
