"""Differentiable fixed-skeleton interpolative decomposition (FP32 kernels).

With the skeleton ``S`` held fixed, ``C = A[:, S]``, ``B = A[:, rd]`` and
``T = C^+ B`` (the interpolation matrix that RBRP returns for that skeleton),

    loss(A) = ||B - C T||_F^2 + ||T w||^2,

where ``w`` holds one weight per column of A (the entries at S are ignored).
:class:`FixedSkeletonIDLoss` is a ``torch.autograd.Function``: its forward runs
the fixed-skeleton ID (``rbrp_fixed_id_f32``: the RBRP panels, swaps and
updates with the sampler replaced by the given skeleton) and the loss kernels;
its backward runs the hand-written adjoint kernels of
``rbrp_fixed_id_adjoint_f32`` on the forward's factorisation, which stays in the
handle (R, T and the permutation of the last run) unless the handle did other
work in between or the backward runs on another stream; then it runs the
fixed-skeleton ID again first:

    dL/dB = 2 E + 2 (C z) w^T,   dL/dC = -2 E T^T - 2 (C z) u^T + 2 (E w) z^T,
    E = B - C T,  u = T w,  z = (C^T C)^{-1} u = R11^{-1} R11^{-T} u.

A gradient with respect to anything A is built from (a kernel lengthscale,
point coordinates) follows from torch's autograd through that construction.
The reference has no differentiable ID; the skeleton of a forward adaptive
RBRP (``Handle.column_id``) is the intended ``S``.
"""
import ctypes

import torch

from . import _lib
from ._lib import Result, check
from .rbrp import Handle, _colmajor, _ld


def _as_f32_colmajor(A):
    if A.dtype != torch.float32:
        raise TypeError("the fixed-skeleton adjoint takes an FP32 matrix")
    A = _colmajor(A)
    if A.stride(0) != 1:
        A = A.t().contiguous().t()
    return A


def fixed_skeleton_id(handle, A, S, b=64):
    """Run the fixed-skeleton ID of the FP32 CUDA matrix ``A`` on skeleton ``S``.

    Returns the permutation (``perm[:k]`` = S in panel-pivot order) and the
    :class:`~robust_blockwise_random_pivoting_gb300._lib.Result`; T stays in
    the handle (``handle.T()``).
    """
    A = _as_f32_colmajor(A)
    m, n = A.shape
    S = S.to(device=A.device, dtype=torch.int32).contiguous()
    perm = torch.empty(n, dtype=torch.int32, device=A.device)
    r = Result()
    handle._bind_stream(torch.cuda.current_stream(A.device))
    check(handle.lib.rbrp_fixed_id_f32(handle.h, m, n, ctypes.c_void_p(A.data_ptr()), _ld(A),
                                       ctypes.c_void_p(S.data_ptr()), int(S.numel()), int(b),
                                       ctypes.c_void_p(perm.data_ptr()), ctypes.byref(r)), handle.h)
    handle.n_last = n
    return perm, r


def fixed_skeleton_loss_and_grad(handle, A, S, w, b=64, grad=True, scale=1.0, reuse_epoch=None):
    """Loss (float) and, if ``grad``, ``scale * dloss/dA`` (FP32, column major) for skeleton ``S``.

    With ``reuse_epoch`` equal to ``handle.epoch`` (read right after a call for the same A, S
    and b) the handle's factorisation is taken as it stands instead of being recomputed."""
    A = _as_f32_colmajor(A)
    m, n = A.shape
    w = w.to(device=A.device, dtype=torch.float32).contiguous()
    if w.numel() != n:
        raise ValueError("w needs one entry per column of A")
    if reuse_epoch is None or reuse_epoch != handle.epoch:
        fixed_skeleton_id(handle, A, S, b)
    G = torch.empty((n, m), dtype=torch.float32, device=A.device).t() if grad else None
    loss = ctypes.c_double()
    check(handle.lib.rbrp_fixed_id_adjoint_f32(handle.h, m, n, ctypes.c_void_p(A.data_ptr()), _ld(A),
                                               ctypes.c_void_p(w.data_ptr()), ctypes.c_float(scale),
                                               ctypes.c_void_p(G.data_ptr()) if grad else None, m,
                                               ctypes.byref(loss)), handle.h)
    return loss.value, G


class FixedSkeletonIDLoss(torch.autograd.Function):
    """``loss = ||A[:, rd] - A[:, S] T||_F^2 + ||T w[rd]||^2`` with ``T = A[:, S]^+ A[:, rd]``."""

    @staticmethod
    def forward(ctx, A, S, w, b=64, handle=None):
        h = handle or Handle(A.device.index)
        loss, _ = fixed_skeleton_loss_and_grad(h, A.detach(), S, w, b, grad=False)
        ctx.save_for_backward(A.detach(), S, w)
        ctx.b, ctx.handle = b, h
        ctx.epoch, ctx.stream = h.epoch, torch.cuda.current_stream(A.device).cuda_stream
        return torch.tensor(loss, dtype=torch.float64, device=A.device)

    @staticmethod
    def backward(ctx, g):
        A, S, w = ctx.saved_tensors
        same_stream = torch.cuda.current_stream(A.device).cuda_stream == ctx.stream
        _, G = fixed_skeleton_loss_and_grad(ctx.handle, A, S, w, ctx.b, grad=True, scale=float(g),
                                            reuse_epoch=ctx.epoch if same_stream else None)
        return G, None, None, None, None


def fixed_skeleton_id_loss(A, S, w, b=64, handle=None):
    """Differentiable loss of the fixed-skeleton ID (see :class:`FixedSkeletonIDLoss`)."""
    return FixedSkeletonIDLoss.apply(A, S, w, b, handle)


def gaussian_kernel_matrix(points, lengthscale):
    """``exp(-|x_i - x_j|^2 / (2 l^2))`` built with torch ops (differentiable in both arguments)."""
    sq = (points * points).sum(1)
    d2 = (sq[:, None] + sq[None, :] - 2.0 * points @ points.t()).clamp_min(0.0)
    return torch.exp(-d2 / (2.0 * lengthscale * lengthscale))
