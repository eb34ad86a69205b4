"""K5 symmetrization on the GPU is bit-exact with the reference's one-thread
KNNTable::symmetrize (src/knntable.cpp:24-99) + build_edges
(src/ncvis.cpp:155-173): same row_ptr, same column indices in the same order,
bitwise-equal distances.  Checked against the golden fixtures (the
reference's own code) and against the oracle on larger generated tables,
including tie-heavy rows and hub rows longer than the shared-memory path."""
import numpy as np
import pytest

from conftest import gmm, golden

pytestmark = pytest.mark.gpu


def _gpu_sym(cuda, inds, dists):
    from ncvis_gb300 import stages
    rp, cols, vals, src = stages.symmetrize(cuda.tensor(inds.astype(np.int32), device="cuda"),
                                            cuda.tensor(dists.astype(np.float32), device="cuda"))
    return (rp.cpu().numpy(), cols.cpu().numpy().astype(np.int64), vals.cpu().numpy(),
            src.cpu().numpy().astype(np.int64))


def _assert_same(got, rp, cols, vals):
    g_rp, g_cols, g_vals, g_src = got
    assert np.array_equal(g_rp, rp)
    assert np.array_equal(g_cols, cols)
    assert np.array_equal(g_vals.view(np.uint32), vals.view(np.uint32))
    assert np.array_equal(g_src, np.repeat(np.arange(rp.size - 1), np.diff(rp)))


@pytest.mark.parametrize("case", ["0", "1", "2", "3", "ties", "hub", "tiny2", "tiny5"])
def test_golden(cuda, case):
    g = golden("symmetrize.npz")
    if case.isdigit():
        inds, dists = g[f"knn_inds_{case}"], g[f"knn_dists_{case}"]
        rp, cols, vals = g[f"sym_rp_{case}"], g[f"sym_cols_{case}"], g[f"sym_vals_{case}"]
    else:
        inds, dists = g[f"{case}_inds"], g[f"{case}_dists"]
        rp, cols, vals = g[f"{case}_rp"], g[f"{case}_cols"], g[f"{case}_vals"]
    _assert_same(_gpu_sym(cuda, inds, dists), rp, cols, vals)


def test_gpu_knn_table(cuda, oracle):
    """The table the engine itself produces (10k-point mixture, k=15)."""
    from ncvis_gb300 import stages
    X, _ = gmm(10000, 32, 10, 5.0, seed=42)
    inds, dists = stages.knn(cuda.tensor(X, device="cuda"), 15, 0)
    inds, dists = inds.cpu().numpy().astype(np.int64), dists.cpu().numpy()
    _assert_same(_gpu_sym(cuda, inds, dists), *oracle.symmetrize(inds, dists))


@pytest.mark.parametrize("seed,N,k,levels", [(1, 20000, 15, 3), (2, 5000, 7, 1), (3, 3000, 31, 16)])
def test_tie_heavy(cuda, oracle, seed, N, k, levels):
    """Quantised distances: most sort keys tie, so the emulated introsort's tie
    order decides the rows."""
    rng = np.random.default_rng(seed)
    inds = rng.integers(0, N - 1, size=(N, k))
    inds = inds + (inds >= np.arange(N)[:, None])  # no self entries
    dists = (rng.integers(0, levels, size=(N, k)) / max(levels, 1)).astype(np.float32)
    dists = -np.sort(-dists, axis=1)
    _assert_same(_gpu_sym(cuda, inds, dists), *oracle.symmetrize(inds, dists))


def test_hubs_long_rows(cuda, oracle):
    """Rows with over a thousand entries (hubs)."""
    rng = np.random.default_rng(7)
    N, k = 6000, 15
    hubs = rng.integers(0, N, size=20)
    inds = np.where(rng.random((N, k)) < 0.3, hubs[rng.integers(0, 20, size=(N, k))],
                    rng.integers(0, N, size=(N, k)))
    dists = np.round(rng.random((N, k)) * 64).astype(np.float32) / 64
    dists = -np.sort(-dists, axis=1)
    rp, cols, vals = oracle.symmetrize(inds, dists)
    assert np.diff(rp).max() > 200
    _assert_same(_gpu_sym(cuda, inds, dists), rp, cols, vals)


def test_rows_across_merge_tiers(cuda, oracle):
    """Row lengths k + in-degree in every merge tier of the GPU path (up to 48
    items one thread per row; 128, 1,024 and 8,192 items one warp per row;
    longer on the global scratch), with tied distances."""
    rng = np.random.default_rng(11)
    N, k = 30000, 15
    inds = rng.integers(0, N - 1, size=(N, k))
    inds = inds + (inds >= np.arange(N)[:, None])  # no self entries
    flat = inds.reshape(-1)
    owner = np.repeat(np.arange(N), k)
    # Hub targets with ~60, ~500, ~3,000 and ~9,000 incoming entries.
    hubs = rng.choice(N, size=34, replace=False)
    want = [60] * 20 + [500] * 10 + [3000] * 3 + [9000]
    slots = rng.permutation(flat.size)
    at = 0
    for h, m in zip(hubs, want):
        take = slots[at:at + m]
        at += m
        take = take[owner[take] != h]
        flat[take] = h
    dists = (rng.integers(0, 8, size=(N, k)) / 8).astype(np.float32)
    dists = -np.sort(-dists, axis=1)
    rp, cols, vals = oracle.symmetrize(inds, dists)
    lens = k + np.bincount(inds.reshape(-1), minlength=N)
    for lo, hi in [(48, 128), (128, 1024), (1024, 8192), (8192, 1 << 30)]:
        assert ((lens > lo) & (lens <= hi)).any(), (lo, hi)
    _assert_same(_gpu_sym(cuda, inds, dists), rp, cols, vals)


def test_rejects_out_of_range(cuda):
    from ncvis_gb300 import NcvisError
    inds = np.array([[1], [2], [3]], np.int64)  # 3 is outside [0, 3)
    dists = np.ones((3, 1), np.float32)
    with pytest.raises(NcvisError, match="outside"):
        _gpu_sym(cuda, inds, dists)
