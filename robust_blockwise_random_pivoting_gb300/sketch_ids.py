"""Comparison IDs of the reference, on the library's kernels.

* :func:`cpqr_id` - the deterministic column-pivoted QR ID
  (``gpu/id_cpqr.cu:30-172``, ``matlab/driver.m:102-171``): greedy block
  pivoting with b = 1 takes, at every step, the column of largest residual
  norm (LAPACK ``dgeqp3``'s rule, first index on ties), so the skeleton is
  CPQR's and T = R11^{-1} R12.
* :func:`rand_cpqr_os` - ``RandCPQR_OS`` (``gpu/randCPQR_OS.cu:20-111``): a
  Gaussian sketch Y = G A with 2r rows (G ~ N(0, 1/m)), the skeleton from the
  column-pivoted QR of the first r rows of Y, and T = R11^{-1} R12 of the QR of
  the column-permuted sketch, i.e. T = Y(:, S)^+ Y(:, rd).
* :func:`interpolation` - the notebook's ``interpolation`` modes
  (``python/RBRP.ipynb`` cell 7 lines 1-37) for a given skeleton: ``'sid'``
  (least squares on A) and ``'fsid'`` (least squares on an oversampled sketch
  of A), both through the fixed-skeleton ID.
* :func:`rand_lupp_os` - ``RandLUPP_OS`` (``gpu/randLUPP_OS.cu:14-119``): the
  same sketch with 2k rows, the skeleton from the partial-pivoted LU of
  Y(1:k, :)^T (:func:`lupp_pivots`), and T = Y(:, S)^+ Y(:, rd).
* :func:`gaussian_sketch` - ``Y = G A`` with Philox Gaussian G
  (``rbrp_sketch_gaussian_f32``).
"""
import ctypes
import math

import torch

from . import _lib
from ._lib import Result, check
from .rbrp import Handle, _colmajor, _ld


def _cm(A, dtype):
    A = _colmajor(A.to(dtype))
    return A if A.stride(0) == 1 else A.t().contiguous().t()


def gaussian_sketch(A, l, seed=0, scale=None, handle=None):
    """``Y = G A`` (``l x n``, FP32, column major) with ``G = scale * N(0, 1)``, ``scale`` default ``1/sqrt(m)``."""
    h = handle or Handle(A.device.index)
    A = _cm(A, torch.float32)
    m, n = A.shape
    scale = 1.0 / math.sqrt(m) if scale is None else float(scale)
    Y = torch.empty((n, l), dtype=torch.float32, device=A.device).t()
    h._bind_stream(torch.cuda.current_stream(A.device))
    check(h.lib.rbrp_sketch_gaussian_f32(h.h, int(l), m, n, ctypes.c_void_p(A.data_ptr()), _ld(A), int(seed),
                                         ctypes.c_float(scale), ctypes.c_void_p(Y.data_ptr()), int(l)), h.h)
    return Y


def fixed_skeleton(handle, A, S, b=64):
    """Fixed-skeleton ID of ``A`` (FP64 or FP32) on ``S``: returns ``(perm, T)`` in the run's own order."""
    dtype = torch.float64 if A.dtype == torch.float64 else torch.float32
    A = _cm(A, dtype)
    m, n = A.shape
    S = S.to(device=A.device, dtype=torch.int32).contiguous()
    perm = torch.empty(n, dtype=torch.int32, device=A.device)
    r = Result()
    handle._bind_stream(torch.cuda.current_stream(A.device))
    fn = handle.lib.rbrp_fixed_id_f64 if dtype == torch.float64 else handle.lib.rbrp_fixed_id_f32
    check(fn(handle.h, m, n, ctypes.c_void_p(A.data_ptr()), _ld(A), ctypes.c_void_p(S.data_ptr()), int(S.numel()),
             int(b), ctypes.c_void_p(perm.data_ptr()), ctypes.byref(r)), handle.h)
    handle.n_last = n
    return perm, handle.T()


def _reorder(perm_run, T_run, S, rd):
    """T of a run (rows perm_run[:k], columns perm_run[k:]) with rows in S order and columns in rd order."""
    n = perm_run.numel()
    k = S.numel()
    pos = torch.empty(n, dtype=torch.long, device=perm_run.device)
    pos[perm_run.long()] = torch.arange(n, device=perm_run.device)
    rows = pos[S.long()]
    cols = pos[rd.long()] - k
    return T_run[rows][:, cols]


def cpqr_id(A, k, handle=None):
    """Deterministic CPQR ID of rank ``k`` (FP64): returns ``(sk, rd, T)``, T = R11^{-1} R12."""
    h = handle or Handle(A.device.index)
    A = _cm(A, torch.float64)
    r = h.column_id(A, b=1, tol=None, kmax=k, sampler="greedy", compute_T=True)
    return r.perm[: r.k], r.perm[r.k:], r.T


def rand_cpqr_os(A, r, seed=0, handle=None):
    """``RandCPQR_OS`` (``gpu/randCPQR_OS.cu:20-111``): returns ``(sk, rd, T)`` with T r x (n - r)."""
    h = handle or Handle(A.device.index)
    Y = gaussian_sketch(A, 2 * r, seed=seed, handle=h)
    piv = h.column_id(_cm(Y[:r], torch.float64), b=1, tol=None, kmax=r, sampler="greedy", compute_T=False)
    S = piv.perm[: piv.k].clone()
    rd = piv.perm[piv.k:].clone()
    perm_run, T_run = fixed_skeleton(h, _cm(Y, torch.float64), S, b=min(64, max(1, S.numel())))
    return S, rd, _reorder(perm_run, T_run, S, rd)


def lupp_pivots(W, handle=None, return_ipiv=False):
    """Column permutation of ``W`` (k x n) from the partial-pivoted LU of ``W^T`` (``rbrp_lupp_pivots_f64``).

    ``perm[:k]`` are the pivot columns in pivot order; with ``return_ipiv`` also
    LAPACK's 1-based ``ipiv`` (k,).  Computed in FP64.
    """
    h = handle or Handle(W.device.index)
    W = _cm(W, torch.float64)
    k, n = W.shape
    perm = torch.empty(n, dtype=torch.int32, device=W.device)
    ipiv = torch.empty(k, dtype=torch.int32, device=W.device) if return_ipiv else None
    h._bind_stream(torch.cuda.current_stream(W.device))
    check(h.lib.rbrp_lupp_pivots_f64(h.h, k, n, ctypes.c_void_p(W.data_ptr()), _ld(W),
                                     ctypes.c_void_p(perm.data_ptr()),
                                     ctypes.c_void_p(ipiv.data_ptr() if ipiv is not None else None)), h.h)
    return (perm, ipiv) if return_ipiv else perm


def rand_lupp_os(A, k, seed=0, handle=None):
    """``RandLUPP_OS`` (``gpu/randLUPP_OS.cu:14-119``): returns ``(sk, rd, T)`` with T k x (n - k)."""
    h = handle or Handle(A.device.index)
    Y = _cm(gaussian_sketch(A, 2 * k, seed=seed, handle=h), torch.float64)
    perm = lupp_pivots(Y[:k], handle=h)
    S = perm[:k].clone()
    rd = perm[k:].clone()
    perm_run, T_run = fixed_skeleton(h, Y, S, b=min(64, k))
    return S, rd, _reorder(perm_run, T_run, S, rd)


def interpolation(A, perm, k, mode="sid", oversampling=1.0, seed=0, handle=None):
    """Interpolation matrix for the skeleton ``perm[:k]`` (rows in that order, columns in ``perm[k:]`` order).

    ``mode='sid'``: T = A(:, S)^+ A(:, rd) (least squares on A).  ``mode='fsid'``:
    the same on a Gaussian sketch of A with ceil(k * oversampling) rows.
    """
    h = handle or Handle(A.device.index)
    perm = perm.to(A.device)
    S, rd = perm[:k], perm[k:]
    if mode == "sid":
        B = A if A.dtype == torch.float64 else A.float()
    elif mode == "fsid":
        B = gaussian_sketch(A, int(math.ceil(k * oversampling)), seed=seed, handle=h).double()
    else:
        raise ValueError(f"mode {mode!r}: 'sid' or 'fsid' (the RBRP run's own T is 'id')")
    perm_run, T_run = fixed_skeleton(h, B, S, b=64)
    return _reorder(perm_run, T_run, S, rd)


def matdivide(A, B, tol=1e-12, handle=None):
    """``A * pinv(B)`` with the singular values of B above ``tol`` kept: the notebook's
    ``matdivide(A, B, tol=TOL_FP)`` (``python/RBRP.ipynb`` cell 2 lines 111-126) on CUDA
    tensors, A (m x n), B (k x n), result (m x k) FP64.  Returns ``(X, rank)``.  The SVD
    is the library's FP64 one-sided Jacobi (``rbrp_matdivide_f64`` on B^T and A^T)."""
    h = handle or Handle(A.device.index)
    Bt = _cm(B.t(), torch.float64)          # (n x k): the matrix whose pseudo-inverse is taken
    At = _cm(A.t(), torch.float64)          # (n x m)
    n, k = Bt.shape
    m = At.shape[1]
    if At.shape[0] != n:
        raise ValueError("A and B need the same number of columns")
    X = torch.empty((m, k), dtype=torch.float64, device=A.device).t()   # (k x m) column major
    rank = ctypes.c_int()
    h._bind_stream(torch.cuda.current_stream(A.device))
    check(h.lib.rbrp_matdivide_f64(h.h, n, k, m, ctypes.c_void_p(Bt.data_ptr()), _ld(Bt),
                                   ctypes.c_void_p(At.data_ptr()), _ld(At), float(tol),
                                   ctypes.c_void_p(X.data_ptr()), _ld(X), ctypes.byref(rank)), h.h)
    return X.t(), rank.value
