"""K7 SGD on the GPU (src/ncvis.cpp:275-352).

Replay mode is held to the reference's one-thread optimizer step by step: a
step is a block of at most 1024 consecutive edges of one epoch (every
positive sample and its noise samples), started from the oracle's Y and
running Q copy; after the step Y and Q must agree to 1e-5 relative
(|dY| <= 1e-5 * max(1, max|Y|), |dQ| <= 1e-5 * max(1, |Q|)).  The only
arithmetic difference left is the power/exponential, evaluated in double and
rounded once on the GPU but by glibc's powf/expf in the reference.

Hogwild mode has no sample-by-sample counterpart (neither has the
reference's multi-thread run); it is checked for invariants here and for
embedding quality end to end in test_gpu_fit_transform.py."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

A, B = 0.76687364, 1.22256382


def _t(cuda, a, dtype):
    return cuda.tensor(np.ascontiguousarray(a).astype(dtype), device="cuda")


def test_replay_steps_match_oracle(cuda, oracle):
    from ncvis_gb300 import stages
    g = golden("embedding.npz")
    rp, cols, plan = g["rp"], g["cols"], g["plan"]
    N = rp.size - 1
    src = oracle.edges_from_csr(rp)
    E = src.size
    stream = oracle.negative_stream(N, src, 42, plan)
    d_src, d_dst = _t(cuda, src, np.int32), _t(cuda, cols, np.int32)
    d_stream = _t(cuda, stream, np.int32)
    Y, Q = g["init_d2_e20"].copy(), 0.0
    pos = 0
    block = 1024
    worst_y = worst_q = 0.0
    for ep in range(plan.size):
        nu = int(plan[ep])
        Qc = Q
        for e0 in range(0, E, block):
            e1 = min(E, e0 + block)
            Yn, Qn, pos_n = oracle.optimize_block(Y, Qc, src, cols, ep, plan.size, nu, e0, e1,
                                                  stream, pos, A, B)
            dY = _t(cuda, Y, np.float32)
            dQ = cuda.tensor([Qc], dtype=cuda.float32, device="cuda")
            stages.optimize_replay(dY, dQ, d_src, d_dst, d_stream, pos, ep, plan.size, nu, A, B,
                                   edge_begin=e0, edge_end=e1)
            gy, gq = dY.cpu().numpy(), float(dQ.cpu()[0])
            ey = np.abs(gy - Yn).max() / max(1.0, np.abs(Yn).max())
            eq = abs(gq - Qn) / max(1.0, abs(Qn))
            worst_y, worst_q = max(worst_y, ey), max(worst_q, eq)
            assert ey <= 1e-5, (ep, e0, ey)
            assert eq <= 1e-5, (ep, e0, eq)
            Y, Qc, pos = Yn, Qn, pos_n
        Q = Qc  # one chain: the epoch average is its own copy
    print(f"replay worst step error: Y {worst_y:.2e}, Q {worst_q:.2e}")


def test_replay_full_epochs_run(cuda, oracle):
    """Whole epochs chained on the GPU stay finite and close in scale to the
    reference (the chaotic dynamics make late epochs diverge bitwise)."""
    from ncvis_gb300 import stages
    g = golden("embedding.npz")
    rp, cols, plan = g["rp"], g["cols"], g["plan"]
    N = rp.size - 1
    src = oracle.edges_from_csr(rp)
    stream = oracle.negative_stream(N, src, 42, plan)
    dY = _t(cuda, g["init_d2_e20"], np.float32)
    dQ = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    d_src, d_dst, d_stream = _t(cuda, src, np.int32), _t(cuda, cols, np.int32), _t(cuda, stream, np.int32)
    pos = 0
    for ep in range(plan.size):
        stages.optimize_replay(dY, dQ, d_src, d_dst, d_stream, pos, ep, plan.size, int(plan[ep]), A, B)
        pos += src.size * int(plan[ep])
    Y = dY.cpu().numpy()
    ref = g["opt_d2_Y"]
    assert np.isfinite(Y).all()
    assert 0.5 < np.std(Y) / np.std(ref) < 2.0
    assert abs(float(dQ.cpu()[0]) - float(g["opt_d2_Q"])) < 1.0


def test_replay_rejects_bad_stream(cuda, oracle):
    from ncvis_gb300 import NcvisError, stages
    g = golden("embedding.npz")
    rp, cols = g["rp"], g["cols"]
    N = rp.size - 1
    src = oracle.edges_from_csr(rp)
    stream = np.full(src.size * 2, N + 5, np.int32)  # out of range
    dY = _t(cuda, g["init_d2_e20"], np.float32)
    before = dY.clone()
    dQ = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    with pytest.raises(NcvisError, match="outside"):
        stages.optimize_replay(dY, dQ, _t(cuda, src, np.int32), _t(cuda, cols, np.int32),
                               _t(cuda, stream, np.int32), 0, 0, 1, 2, A, B)
    # the first edge's positive sample ran, the bad noise index stopped the chain
    assert np.isfinite(dY.cpu().numpy()).all()
    assert not cuda.isnan(before).any()


@pytest.mark.parametrize("d", [1, 2, 3, 5])
def test_hogwild_invariants(cuda, oracle, d):
    from ncvis_gb300 import stages
    g = golden("embedding.npz")
    rp, cols, plan = g["rp"], g["cols"], g["plan"]
    N = rp.size - 1
    src = oracle.edges_from_csr(rp)
    Y0 = oracle.init_embedding(N, d, src, cols, 42, 20, np.float32(1 / 15), 1)
    dY = _t(cuda, Y0, np.float32)
    dQ = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    stages.optimize(dY, dQ, _t(cuda, src, np.int32), _t(cuda, cols, np.int32), 42, plan, A, B,
                    chains=8)
    Y = dY.cpu().numpy()
    assert np.isfinite(Y).all() and np.isfinite(float(dQ.cpu()[0]))
    # The reference (8 threads = 8 chains) settles Q near the same value.
    Yr, Qr = oracle.optimize(Y0, 0.0, src, cols, 42, plan, A, B, n_threads=8)
    assert abs(float(dQ.cpu()[0]) - Qr) < 1.5
    # Embedding spreads like the reference's.
    assert 0.5 < np.std(Y) / np.std(Yr) < 2.0


@pytest.mark.parametrize("d", [1, 2, 3, 4])
def test_grouped_chain_matches_sequential_chain(cuda, d):
    """One chain, so the result is deterministic: the kernel for d <= 4, which
    gathers the rows of a group of samples before applying them, keeps y_i in
    registers across a run of equal sources and applies y_o -= dx as an L2
    reduction, must give bit-identical Y and Q to the plain kernel for d > 4,
    which reads and stores every row when it is used; the latter runs on the
    same embedding padded with zero columns to d = 5 (zero columns add exact
    zeros to every distance and never move).  Small N and up to 20 noise
    samples per edge make samples of one group hit the same row all the time;
    runs of 1-5 equal sources and self edges cover the write-back of y_i."""
    from ncvis_gb300 import stages
    rng = np.random.default_rng(d)
    N = 24
    runs = rng.integers(1, 6, size=60)
    src = np.repeat(rng.integers(0, N, size=runs.size), runs).astype(np.int32)
    dst = rng.integers(0, N, size=src.size).astype(np.int32)
    self_edges = rng.random(src.size) < 0.05
    dst[self_edges] = src[self_edges]
    plan = np.array([0, 1, 2, 3, 7, 20], dtype=np.uint64)
    Y0 = rng.normal(0, 1, size=(N, d)).astype(np.float32)
    Y5 = np.zeros((N, 5), np.float32)
    Y5[:, :d] = Y0
    out = []
    for Y in (Y0, Y5):
        dY = _t(cuda, Y, np.float32)
        dQ = cuda.zeros(1, dtype=cuda.float32, device="cuda")
        stages.optimize(dY, dQ, _t(cuda, src, np.int32), _t(cuda, dst, np.int32), 7, plan, A, B,
                        chains=1)
        out.append((dY.cpu().numpy(), float(dQ.cpu()[0])))
    (Yw, Qw), (Ys, Qs) = out
    assert np.isfinite(Yw).all()
    assert not np.array_equal(Yw, Y0)
    assert np.array_equal(Ys[:, d:], np.zeros((N, 5 - d), np.float32))
    assert np.array_equal(Yw.view(np.uint32), Ys[:, :d].copy().view(np.uint32))
    assert np.float32(Qw).view(np.uint32) == np.float32(Qs).view(np.uint32)


def test_hogwild_rejects_bad_edges(cuda):
    from ncvis_gb300 import NcvisError, stages
    dY = cuda.zeros((10, 2), dtype=cuda.float32, device="cuda")
    dQ = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    src = cuda.tensor([0, 1, 2], dtype=cuda.int32, device="cuda")
    dst = cuda.tensor([1, 2, 10], dtype=cuda.int32, device="cuda")
    with pytest.raises(NcvisError, match="outside"):
        stages.optimize(dY, dQ, src, dst, 1, np.array([1], np.uintp), A, B)


def test_update_rate_diagnostic(cuda):
    """The optimizer's ceiling probe: random row gathers and random gathers
    plus reductions over a 2^20-row array both report positive rates, the
    update rate is not above the gather rate, and unsupported row widths are
    refused."""
    import ctypes as C
    from ncvis_gb300 import _lib
    L = _lib.lib()
    g, u = C.c_double(0), C.c_double(0)
    assert L.ncvis_measure_update_rate(1 << 20, 2, C.byref(g), C.byref(u), None) == 0
    assert 1e8 < u.value <= 1.1 * g.value
    assert L.ncvis_measure_update_rate(1 << 20, 3, C.byref(g), C.byref(u), None) == 3
    assert b"d must be 1, 2 or 4" in L.ncvis_get_last_error()
