"""The allocation-free NCE loss entry point (ncvis_nce_loss_device_noalloc)
against the allocating one (ncvis_nce_loss_device), through the C ABI.

Callers that cannot allocate device memory when they need the loss (a pool
that already holds all free memory, a loop that must not take the
allocator's synchronisation, a framework that forbids outside allocations)
use the no-allocation variant.  It must give the same loss (tolerance of the
loss tests: 1e-5 relative) on consecutive calls, whose shared scratch array
keeps the previous call's contents; leave the device's stream-ordered memory
pool and its free memory untouched (read through the driver, which sees the
library's allocations whatever runtime copy made them); refuse batches above
its 2^20-edge limit and edges outside [0, N); and give 0 for an empty batch.
Runs alone in a fresh process or after the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A, B = 0.76687364, 1.22256382
USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8  # CUmemPool_attribute


class DriverMemory:
    """The default memory pool of device 0 and the context's free memory,
    through libcuda (cuDeviceGetDefaultMemPool, cuMemPoolGet/SetAttribute,
    cuMemGetInfo)."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        dev = C.c_int(0)
        assert self.cu.cuDeviceGet(C.byref(dev), 0) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def pool_attr(self, attr):
        v = C.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, USED_MEM_HIGH, C.byref(zero)) == 0

    def free_bytes(self):
        free, total = C.c_size_t(0), C.c_size_t(0)
        assert self.cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
        return free.value


def _loss(torch, fn, N, d, src, dst, Y, Q, seed, tag, out=None, E=None):
    if out is None:
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    E = src.shape[0] if E is None else E
    rc = fn(N, d, E, src.data_ptr(), dst.data_ptr(), Y.data_ptr(), Q.data_ptr(), 5, A, B, seed,
            tag, 0, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
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


def test_noalloc_allocates_nothing():
    """After a warm-up call, two calls move neither the default pool's
    high-water mark (which the allocating entry does move: the check is
    live) nor the device's free memory."""
    import torch
    from ncvis_gb300 import _lib
    L = _lib.lib()
    mem = DriverMemory()
    g = torch.Generator(device="cuda").manual_seed(2)
    N, d, E = 50000, 2, 1 << 20
    src = torch.randint(0, N, (E,), device="cuda", dtype=torch.int32, generator=g)
    dst = torch.randint(0, N, (E,), device="cuda", dtype=torch.int32, generator=g)
    Y = torch.randn((N, d), device="cuda", dtype=torch.float32, generator=g)
    Q = torch.tensor([0.2], device="cuda", dtype=torch.float32)
    outs = [torch.zeros(1, dtype=torch.float64, device="cuda") for _ in range(3)]
    torch.cuda.synchronize()
    mem.reset_high()
    rc, _ = _loss(torch, L.ncvis_nce_loss_device, N, d, src, dst, Y, Q, 9, 0, outs[1])
    assert rc == 0, L.ncvis_get_last_error()
    torch.cuda.synchronize()
    assert mem.pool_attr(USED_MEM_HIGH) > 0, "the allocating entry should show in the pool"
    # Warm-up call (set-up on this device), then the measured calls.
    rc, _ = _loss(torch, L.ncvis_nce_loss_device_noalloc, N, d, src, dst, Y, Q, 9, 0, outs[0])
    assert rc == 0, L.ncvis_get_last_error()
    torch.cuda.synchronize()

    used0 = mem.pool_attr(USED_MEM_CURRENT)
    free0 = mem.free_bytes()
    mem.reset_high()
    for call in range(2):
        rc, _ = _loss(torch, L.ncvis_nce_loss_device_noalloc, N, d, src, dst, Y, Q, 9, 0,
                      outs[2])
        assert rc == 0, L.ncvis_get_last_error()
    torch.cuda.synchronize()
    assert mem.pool_attr(USED_MEM_HIGH) == 0
    assert mem.pool_attr(USED_MEM_CURRENT) == used0
    assert mem.free_bytes() == free0
    a, b = outs[1].item(), outs[2].item()
    assert abs(a - b) <= 1e-5 * abs(a), (a, b)


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


def test_noalloc_rejects_bad_endpoint_and_takes_empty_batch():
    import torch
    from ncvis_gb300 import _lib
    L = _lib.lib()
    N = 1000
    Y = torch.randn((N, 2), device="cuda", dtype=torch.float32)
    Q = torch.zeros(1, device="cuda", dtype=torch.float32)
    src = torch.arange(64, device="cuda", dtype=torch.int32)
    dst = src.clone()
    dst[37] = N  # one endpoint outside [0, N)
    rc, _ = _loss(torch, L.ncvis_nce_loss_device_noalloc, N, 2, src, dst, Y, Q, 1, 0)
    assert rc == _lib.NCVIS_INVALID_ARGUMENT
    assert b"outside" in L.ncvis_get_last_error()
    # An empty batch (E = 0): loss 0, as the allocating entry gives.
    rc_a, ref = _loss(torch, L.ncvis_nce_loss_device, N, 2, src, src, Y, Q, 1, 0, E=0)
    rc_b, got = _loss(torch, L.ncvis_nce_loss_device_noalloc, N, 2, src, src, Y, Q, 1, 0, E=0)
    assert rc_a == 0 and rc_b == 0, L.ncvis_get_last_error()
    assert ref.item() == 0.0 and got.item() == 0.0
