"""The allocation-free NCE loss entry point (ncvis_nce_loss_device_noalloc)
against the allocating one (ncvis_nce_loss_device), through the C ABI.

Callers that cannot allocate device memory when they need the loss use the
no-allocation variant; it must give the same loss (tolerance of the loss
tests: 1e-5 relative) on consecutive calls, whose shared scratch array keeps
the previous call's contents, and reject batches above its 2^20-edge limit.
Runs alone in a fresh process or after the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A, B = 0.76687364, 1.22256382


def _loss(torch, fn, N, d, src, dst, Y, Q, seed, tag):
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    rc = fn(N, d, src.shape[0], src.data_ptr(), dst.data_ptr(), Y.data_ptr(), Q.data_ptr(), 5, A,
            B, seed, tag, 0, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return rc, out


def test_noalloc_loss_matches_allocating_entry():
    import torch
    from ncvis_gb300 import _lib
    L = _lib.lib()
    g = torch.Generator(device="cuda").manual_seed(1)
    N, d, E = 20000, 2, 300000
    src = torch.randint(0, N, (E,), device="cuda", dtype=torch.int32, generator=g)
    dst = torch.randint(0, N, (E,), device="cuda", dtype=torch.int32, generator=g)
    Q = torch.tensor([0.7], device="cuda", dtype=torch.float32)
    for call in range(2):  # second call reuses the scratch left by the first
        Y = torch.randn((N, d), device="cuda", dtype=torch.float32, generator=g)
        rc_a, ref = _loss(torch, L.ncvis_nce_loss_device, N, d, src, dst, Y, Q, 3 + call, call)
        rc_b, got = _loss(torch, L.ncvis_nce_loss_device_noalloc, N, d, src, dst, Y, Q, 3 + call,
                          call)
        assert rc_a == 0 and rc_b == 0, L.ncvis_get_last_error()
        a, b = ref.item(), got.item()
        assert np.isfinite(b) and abs(a - b) <= 1e-5 * abs(a), (call, a, b)


def test_noalloc_rejects_oversized_batch():
    import torch
    from ncvis_gb300 import _lib
    L = _lib.lib()
    N, E = 1000, (1 << 20) + 1
    src = torch.zeros(E, device="cuda", dtype=torch.int32)
    dst = torch.ones(E, device="cuda", dtype=torch.int32)
    Y = torch.zeros((N, 2), device="cuda", dtype=torch.float32)
    Q = torch.zeros(1, device="cuda", dtype=torch.float32)
    rc, _ = _loss(torch, L.ncvis_nce_loss_device_noalloc, N, 2, src, dst, Y, Q, 1, 0)
    assert rc == _lib.NCVIS_INVALID_ARGUMENT
    assert b"2^20" in L.ncvis_get_last_error()
