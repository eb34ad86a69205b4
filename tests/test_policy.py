"""Host-side parameter policy of the Python API (wrapper/ncvis.pyx:7-24,
103-143): a/b curve fit, noise schedule, distance names and the ValueErrors
the reference raises.  No GPU: the errors are raised before the engine is
created."""
import numpy as np
import pytest

import ncvis_gb300 as ncvis
from ncvis_gb300.api import default_noise_plan, find_ab_params


def test_ab_defaults():
    # spread=1, min_dist=0.4 (the Python defaults of the reference)
    a, b = find_ab_params(1.0, 0.4)
    assert abs(a - 0.76687364) < 1e-6 and abs(b - 1.22256382) < 1e-6


def test_ab_function_default_min_dist():
    a, b = find_ab_params()  # min_dist=0.1, the function's own default
    assert a > 0 and b > 0 and abs(b - 0.8950608781603216) < 1e-3


def test_noise_plan_50():
    plan = default_noise_plan(50)
    expect = [1] * 21 + [2] * 4 + [3] * 3 + [4] * 3 + [5, 5, 6, 7, 7, 8, 8, 9, 10, 11, 11, 12, 13,
                                                       14, 15, 16, 17, 18, 20]
    assert plan.tolist() == expect
    assert plan.sum() == 262 and (plan + 1).sum() == 312
    assert plan.dtype == np.uintp


def test_noise_plan_small():
    # One epoch: the reference's 0 / 0 would cast NaN (2^63 on x86-64).
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        assert default_noise_plan(1).tolist() == [1]
        assert default_noise_plan(0).tolist() == []
    assert default_noise_plan(3).min() >= 1


def test_n_noise_errors():
    with pytest.raises(ValueError, match="exactly one dimension"):
        ncvis.NCVis(n_noise=np.ones((2, 2), dtype=int))
    with pytest.raises(ValueError, match="at least 1"):
        ncvis.NCVis(n_noise=0)
    with pytest.raises(ValueError, match="unsupported type"):
        ncvis.NCVis(n_noise=1.5)
    # A negative entry would wrap to 2^64 - 1 in the uintp plan.
    with pytest.raises(ValueError, match="should be in"):
        ncvis.NCVis(n_noise=np.array([3, -1, 3]))
    with pytest.raises(ValueError, match="should be in"):
        ncvis.NCVis(n_noise=np.array([3, (1 << 24) + 1]))
    with pytest.raises(ValueError, match="at most"):
        ncvis.NCVis(n_noise=(1 << 24) + 1)
    assert ncvis.NCVis(n_noise=np.array([0, 1 << 24])).noise_plan.tolist() == [0, 1 << 24]


def test_distance_error():
    with pytest.raises(ValueError, match="Unsupported distance"):
        ncvis.NCVis(distance="manhattan")


def test_ab_pair_error():
    with pytest.raises(ValueError):
        ncvis.NCVis(a=1.0, b=None)
    with pytest.raises(ValueError):
        ncvis.NCVis(a=None, b=1.0)


def test_mode_errors():
    with pytest.raises(ValueError):
        ncvis.NCVis(knn_precision="fp8")
    with pytest.raises(ValueError):
        ncvis.NCVis(sgd_mode="async")
    with pytest.raises(ValueError, match="non-negative"):
        ncvis.NCVis(rerank_factor=-1)
    with pytest.raises(ValueError, match="non-negative"):
        ncvis.NCVis(sgd_chains=-1)


def test_distance_enum_matches_reference_order():
    # ncvis::Distance {squared_L2, inner_product, cosine_similarity, correlation}
    assert ncvis.DISTANCES == {"euclidean": 0, "inner_product": 1, "cosine": 2, "correlation": 3}
