"""Failure detection without a GPU fault.

* A bounded device wait that runs out: the tensor-core kNN kernel is made to
  wait on a barrier that nothing completes (the `inject_stall` diagnostic,
  with a short `wait_limit_cycles`).  The kernel stops, drains its copies and
  MMAs, frees its tensor memory and returns; fit_transform reports
  NCVIS_DEVICE_TIMEOUT; the next call on the same handle, with the stall off,
  succeeds and gives the same embedding quality as a fresh engine.
* An allocation failure injected on the host: with `arena_limit` below what
  the fit needs, fit_transform fails as a failed cudaMalloc would
  (NCVIS_CUDA_ERROR, "out of memory"), touching no device memory; with the
  limit lifted the same handle fits.
* The reference's own error paths (src/ncvis.cpp:364-369, :90) are covered in
  test_gpu_fit_transform.py and test_abi.py.
"""
import numpy as np
import pytest

from conftest import gmm

pytestmark = pytest.mark.gpu


def test_knn_wait_runs_out_then_recovers(cuda):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import _lib, quality
    X, _ = gmm(6000, 32, 6, 5.0, seed=5)
    Xd = cuda.tensor(X, device="cuda")
    vis = ncvis.NCVis(random_seed=5, knn_precision="bf16")
    vis.set_options(inject_stall=1, wait_limit_cycles=200_000)
    with pytest.raises(ncvis.NcvisError) as info:
        vis.fit_transform(Xd)
    assert info.value.code == _lib.NCVIS_DEVICE_TIMEOUT, str(info.value)
    assert "timed out" in str(info.value)
    # The same handle, stall off: a normal fit.
    vis.set_options(inject_stall=0, wait_limit_cycles=0)
    Y = vis.fit_transform(Xd)
    cuda.cuda.synchronize()
    assert bool(cuda.isfinite(Y).all())
    fresh = ncvis.NCVis(random_seed=5, knn_precision="bf16").fit_transform(Xd)
    t_after = quality.trustworthiness_device(Xd, Y, 15, distance=0)
    t_fresh = quality.trustworthiness_device(Xd, fresh, 15, distance=0)
    assert abs(t_after - t_fresh) <= 0.01, (t_after, t_fresh)


def test_knn_wait_runs_out_in_a_batched_fit(cuda):
    """The batched path checks the same flag."""
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import _lib
    Xs = [cuda.tensor(gmm(n, 16, 3, 5.0, seed=n)[0], device="cuda") for n in (700, 1300)]
    vis = ncvis.NCVis(random_seed=1, knn_precision="bf16")
    vis.set_options(inject_stall=1, wait_limit_cycles=200_000)
    with pytest.raises(ncvis.NcvisError) as info:
        vis.fit_transform_batched(Xs)
    assert info.value.code == _lib.NCVIS_DEVICE_TIMEOUT
    vis.set_options(inject_stall=0, wait_limit_cycles=0)
    Ys = vis.fit_transform_batched(Xs)
    assert all(bool(cuda.isfinite(Y).all()) for Y in Ys)


def test_allocation_failure_is_reported_and_recovers(cuda):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import _lib
    X, _ = gmm(4000, 16, 4, 5.0, seed=9)
    vis = ncvis.NCVis(random_seed=9, arena_limit=1 << 20)
    with pytest.raises(ncvis.NcvisError) as info:
        vis.fit_transform(X)
    assert info.value.code == _lib.NCVIS_CUDA_ERROR
    assert "out of memory" in str(info.value)
    vis.set_options(arena_limit=0)
    Y = vis.fit_transform(X)
    assert Y.shape == (4000, 2) and np.isfinite(Y).all()
    # A limit above the need changes nothing.
    vis.set_options(arena_limit=1 << 34)
    assert np.isfinite(vis.fit_transform(X)).all()


def test_options_refuse_negative_wait_limit(cuda):
    import ncvis_gb300 as ncvis
    from ncvis_gb300 import _lib
    vis = ncvis.NCVis()
    with pytest.raises(ncvis.NcvisError) as info:
        vis.set_options(wait_limit_cycles=-1)
    assert info.value.code == _lib.NCVIS_INVALID_ARGUMENT
