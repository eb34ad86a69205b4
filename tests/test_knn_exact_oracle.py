"""The FP64 exact kNN oracle (oracle/knn_exact.py) against a full sort per
row by (distance, index), on both backends, with duplicated points (ties at
distance 0 broken by index), all four distance kinds' two formulas, and the
recall helper."""
import numpy as np
import pytest

from oracle.knn_exact import exact_rows, recall


def _full_sort_rows(X, q, k, dist):
    X = X.astype(np.float64)
    out = []
    for i in q:
        if dist == 0:
            d = ((X - X[i]) ** 2).sum(1)
        else:
            d = 1.0 - X @ X[i]
        order = np.lexsort((np.arange(len(X)), d))
        out.append(order[1:k + 1])
    return np.array(out)


@pytest.mark.parametrize("dist", [0, 2])
@pytest.mark.parametrize("device", [None, "cpu"])
def test_matches_full_sort(dist, device):
    if device:
        pytest.importorskip("torch")
    rng = np.random.default_rng(7 + dist)
    X = rng.normal(size=(700, 9)).astype(np.float32)
    if dist:
        X /= np.linalg.norm(X, axis=1, keepdims=True)
    q = np.arange(0, 700, 3)
    got = exact_rows(X, q, 15, dist, device=device, block=64)
    ref = _full_sort_rows(X, q, 15, dist)
    # Squared L2 by the |x|^2 + |y|^2 - 2<x, y> form can reorder pairs whose
    # distances differ by rounding only; none do in this draw.
    assert np.array_equal(got, ref)


def test_duplicates_break_ties_by_index():
    rng = np.random.default_rng(3)
    X = np.repeat(rng.normal(size=(50, 4)).astype(np.float32), 4, axis=0)
    q = np.arange(200)
    for device in (None, "cpu"):
        got = exact_rows(X, q, 3, 0, device=device)
        # the k + 1 = 4 nearest are the four copies; the lowest index is dropped
        base = (q // 4) * 4
        assert np.array_equal(got, base[:, None] + np.arange(1, 4)[None, :])


def test_recall():
    exact = np.array([[1, 2, 3], [4, 5, 6]])
    assert recall(exact, exact) == 1.0
    assert recall(np.array([[3, 2, 9], [7, 8, 9]]), exact) == pytest.approx(2 / 6)
