"""The NCVis objective as a differentiable torch function.

``nce_loss(Y, Q, src, dst, ...)`` is the noise-contrastive loss whose
per-sample gradient the reference's optimizer follows (src/ncvis.cpp:304-323):
for each edge (i, j) one positive term softplus(log nu + Q - log Ph(d2_ij))
and nu noise terms softplus(log Ph(d2_io) - Q - log nu), Ph(d2) = 1/(1 + a
d2^b).  Forward and backward are CUDA kernels of libncvis_gb300.so (K8);
noise samples come from a counter-based stream keyed by (seed, tag) and
counted by the global edge index, so a batch's backward sees its forward's
samples, and batches of one edge list (``edge_offset``) see disjoint
streams.  The loss is a sum over the batch; dL/dQ and the loss are reduced
in FP64 on the device.  With it, torch optimizers can drive the NCVis
objective (e.g. Adam on Y and Q over edge batches).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


def _stream():
    return torch.cuda.current_stream().cuda_stream


class NCELoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, Y, Q, src, dst, n_noise, a, b, seed, tag, edge_offset):
        assert Y.is_cuda and Y.dtype == torch.float32 and Y.dim() == 2
        Y = Y.contiguous()
        Q = Q.reshape(1).to(torch.float32).contiguous()
        src = src.to(torch.int32).contiguous()
        dst = dst.to(torch.int32).contiguous()
        N, d = Y.shape
        loss = torch.empty(1, dtype=torch.float64, device=Y.device)
        _lib.check(_lib.lib().ncvis_nce_loss_device(
            N, d, src.shape[0], src.data_ptr(), dst.data_ptr(), Y.data_ptr(), Q.data_ptr(),
            int(n_noise), float(a), float(b), int(seed), int(tag), int(edge_offset),
            loss.data_ptr(), _stream()))
        ctx.save_for_backward(Y, Q, src, dst)
        ctx.args = (int(n_noise), float(a), float(b), int(seed), int(tag), int(edge_offset))
        return loss.reshape(()).to(torch.float32)

    @staticmethod
    def backward(ctx, grad):
        Y, Q, src, dst = ctx.saved_tensors
        n_noise, a, b, seed, tag, edge_offset = ctx.args
        N, d = Y.shape
        scale = grad.reshape(1).to(torch.float32).contiguous()
        gY = torch.zeros_like(Y)
        gQ = torch.empty(1, dtype=torch.float64, device=Y.device)
        _lib.check(_lib.lib().ncvis_nce_grad_device(
            N, d, src.shape[0], src.data_ptr(), dst.data_ptr(), Y.data_ptr(), Q.data_ptr(),
            n_noise, a, b, seed, tag, edge_offset, scale.data_ptr(), gY.data_ptr(),
            gQ.data_ptr(), _stream()))
        return gY, gQ.to(torch.float32).reshape(()), None, None, None, None, None, None, None, None


def nce_loss(Y, Q, src, dst, n_noise: int = 5, a: float = 0.76687364, b: float = 1.22256382,
             seed: int = 0, tag: int = 0, edge_offset: int = 0):
    """Summed NCE loss of the edges (src[e], dst[e]) with n_noise noise
    samples each; differentiable in Y (float32 [N, d], CUDA) and Q (scalar)."""
    return NCELoss.apply(Y, Q, src, dst, n_noise, a, b, seed, tag, edge_offset)


def noise_indices(src, N: int, n_noise: int, seed: int = 0, tag: int = 0, edge_offset: int = 0):
    """The noise samples nce_loss uses for these edges: int32 [E, n_noise]."""
    src = src.to(torch.int32).contiguous()
    out = torch.empty((src.shape[0], n_noise), dtype=torch.int32, device=src.device)
    _lib.check(_lib.lib().ncvis_nce_noise_device(N, src.shape[0], src.data_ptr(), n_noise, seed,
                                                 tag, edge_offset, out.data_ptr(), _stream()))
    return out
