"""K8: the differentiable NCE loss (ncvis_gb300.nce) against its FP64
restatement (oracle/nce_oracle.py), FP64 finite differences, and the
reference's own SGD update.

Tolerances: noise indices bit-exact; loss within 1e-5 relative of FP64;
gradient within 2e-4 * max|grad| of the FP64 analytic gradient (FP32
per-sample terms, FP32 atomics); analytic FP64 gradient within 1e-6 relative
of central differences; one reference SGD step with a small step size
(1e-4) moves Y and Q by -step * gradient to 1e-2 relative (first order).
"""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu

A, B = 0.76687364, 1.22256382


def _graph(oracle, N, D=16, seed=0):
    X, _ = gmm(N, D, 8, 5.0, seed=seed)
    inds, dists = oracle.knn(oracle.preprocess(X, 0), 0, 15)
    rp, cols, _ = oracle.symmetrize(inds, dists)
    return oracle.edges_from_csr(rp), cols


@pytest.fixture(scope="module")
def graph2k(oracle):
    return _graph(oracle, 2000)


def _t(cuda, a, dtype):
    return cuda.tensor(np.ascontiguousarray(a).astype(dtype), device="cuda")


def test_noise_indices_match(cuda, graph2k):
    from ncvis_gb300 import nce
    from oracle import nce_oracle
    src, _ = graph2k
    got = nce.noise_indices(_t(cuda, src, np.int32), 2000, 5, seed=123, tag=7,
                            edge_offset=1 << 33).cpu().numpy()
    ref = nce_oracle.noise_indices(src, 2000, 5, seed=123, tag=7, edge_offset=1 << 33)
    assert np.array_equal(got, ref)
    assert not np.any(got == src[:, None])


@pytest.mark.parametrize("d", [2, 16])
def test_loss_and_grad_vs_fp64(cuda, graph2k, d):
    from ncvis_gb300 import nce
    from oracle import nce_oracle
    src, dst = graph2k
    rng = np.random.default_rng(d)
    Y0 = rng.normal(0, 1.0, size=(2000, d)).astype(np.float32)
    Q0 = 1.0
    Y = _t(cuda, Y0, np.float32).requires_grad_(True)
    Q = cuda.tensor(Q0, dtype=cuda.float32, device="cuda", requires_grad=True)
    loss = nce.nce_loss(Y, Q, _t(cuda, src, np.int32), _t(cuda, dst, np.int32), n_noise=5, a=A,
                        b=B, seed=9, tag=0)
    loss.backward()
    noise = nce_oracle.noise_indices(src, 2000, 5, seed=9, tag=0)
    L, gY, gQ = nce_oracle.loss_and_grad(Y0, Q0, src, dst, noise, A, B)
    assert abs(loss.item() - L) <= 1e-5 * abs(L)
    got = Y.grad.cpu().numpy()
    assert np.abs(got - gY).max() <= 2e-4 * np.abs(gY).max()
    assert abs(Q.grad.item() - gQ) <= 1e-4 * max(1.0, abs(gQ))


def test_gpu_gradient_vs_finite_differences(cuda, graph2k):
    """GPU gradient against FP64 central differences of the loss itself."""
    from ncvis_gb300 import nce
    from oracle import nce_oracle
    src, dst = graph2k
    rng = np.random.default_rng(8)
    Y0 = rng.normal(0, 1e-2, size=(2000, 2)).astype(np.float32)
    Y = _t(cuda, Y0, np.float32).requires_grad_(True)
    Q = cuda.tensor(1.0, dtype=cuda.float32, device="cuda", requires_grad=True)
    nce.nce_loss(Y, Q, _t(cuda, src, np.int32), _t(cuda, dst, np.int32), seed=2).backward()
    noise = nce_oracle.noise_indices(src, 2000, 5, seed=2, tag=0)
    g = Y.grad.cpu().numpy()
    Yd = Y0.astype(np.float64)
    h = 1e-6
    for (r, c) in [(int(src[10]), 0), (int(dst[99]), 1), (500, 0)]:
        Yp, Ym = Yd.copy(), Yd.copy()
        Yp[r, c] += h
        Ym[r, c] -= h
        # only the edges that touch row r depend on it
        m = (src == r) | (dst == r) | (noise == r).any(1)
        fd = (nce_oracle.loss_only(Yp, 1.0, src[m], dst[m], noise[m], A, B) -
              nce_oracle.loss_only(Ym, 1.0, src[m], dst[m], noise[m], A, B)) / (2 * h)
        assert abs(fd - g[r, c]) <= 1e-3 * max(abs(fd), 1e-2 * np.abs(g).max())


def test_reference_sgd_step_is_gradient_step(cuda, graph2k, oracle):
    """One reference optimizer pass over a batch with a small step moves Y and
    Q by -step * dL/dY and -alpha_Q * dL/dQ to first order."""
    from ncvis_gb300 import nce
    from oracle import nce_oracle
    src, dst = graph2k
    src, dst = src[:200], dst[:200]
    rng = np.random.default_rng(3)
    Y0 = rng.normal(0, 1.0, size=(2000, 2)).astype(np.float32)
    noise = nce_oracle.noise_indices(src, 2000, 5, seed=5, tag=0)
    step = 1e-4
    Yn, Qn, _ = oracle.optimize_block(Y0, 1.0, src, dst, 0, 50, 5, 0, src.size,
                                      noise.astype(np.int32).ravel(), 0, A, B, alpha=step,
                                      alpha_Q=step)
    Y = _t(cuda, Y0, np.float32).requires_grad_(True)
    Q = cuda.tensor(1.0, dtype=cuda.float32, device="cuda", requires_grad=True)
    nce.nce_loss(Y, Q, _t(cuda, src, np.int32), _t(cuda, dst, np.int32), seed=5).backward()
    dY_ref = (Yn - Y0).astype(np.float64)
    dY_grad = -step * Y.grad.cpu().numpy().astype(np.float64)
    moved = np.abs(dY_grad) > 1e-3 * np.abs(dY_grad).max()
    rel = np.abs(dY_ref[moved] - dY_grad[moved]).max() / np.abs(dY_grad).max()
    assert rel < 1e-2, rel
    assert abs((Qn - 1.0) - (-step * Q.grad.item())) <= 1e-2 * abs(step * Q.grad.item())


def test_torch_optimizer_drives_objective(cuda, oracle):
    """Adam on (Y, Q) over edge batches lowers the loss (the objective can
    drive torch optimizers)."""
    from ncvis_gb300 import nce
    src, dst = _graph(oracle, 5000, seed=1)
    s, t = _t(cuda, src, np.int32), _t(cuda, dst, np.int32)
    gen = cuda.Generator(device="cuda").manual_seed(0)
    Y = (1e-2 * cuda.randn((5000, 2), device="cuda", generator=gen)).requires_grad_(True)
    Q = cuda.tensor(1.0, device="cuda", requires_grad=True)
    opt = cuda.optim.Adam([Y, Q], lr=0.05)
    first = None
    for it in range(60):
        opt.zero_grad()
        loss = nce.nce_loss(Y, Q, s, t, seed=it) / src.size
        loss.backward()
        opt.step()
        first = first if first is not None else loss.item()
    assert loss.item() < 0.8 * first
