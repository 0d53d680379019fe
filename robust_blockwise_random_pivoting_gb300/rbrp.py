"""Python host API of the GB300 RBRP column ID (over the C ABI).

Mirrors the reference's entry points:

* :func:`RBRP` - ``RBRP(m, n, A, blk, ranks, error, t_ranks, t_rbrp, flops)``
  (``gpu/rbrp.hpp:6-8``): runs to rank min(m, n) and returns the per-block
  trace.
* :func:`rand_adap_rbrp` - ``RandAdapLUPP``'s contract (``gpu/rid.hpp:5-7``)
  with RBRP pivoting: tolerance and block size in; skeleton ``sk``, redundant
  set ``rd``, interpolation matrix ``T`` and rank out.
* :func:`blocked_rpid` - the notebook's ``blocked_rpid(X, k, b, tol, mode,
  ortho=1, tol_loc)`` (``python/RBRP.ipynb`` cell 11 lines 76-173): rows of
  ``X`` are the items (``X = A.T``), ``tol`` bounds the squared residual.
* :class:`Handle` - the reusable handle (workspace, stream, last result).
* :class:`Batch` / :func:`batched_column_id` - thousands of independent FP32
  column IDs of uneven shape in one persistent launch (no reference
  counterpart: the reference solves one matrix per ``RBRP`` call).

Device memory and streams come from PyTorch; all arithmetic runs in the
sm_103a kernels of ``librbrp_gb300.so``.
"""
import ctypes
from collections.abc import Sequence
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import Params, Result, check


def _colmajor(A):
    """A column-major (Fortran-ordered) view of a 2-D tensor, copying if needed."""
    if A.dim() != 2:
        raise ValueError("A must be 2-D")
    m, n = A.shape
    if (A.stride(0) == 1 or m == 1) and (A.stride(1) >= max(1, m) or n == 1):
        return A
    return A.t().contiguous().t()


def _ld(A):
    """Leading dimension of a column-major tensor (size-1 dimensions carry arbitrary strides)."""
    m, n = A.shape
    return max(1, m) if n == 1 else max(1, m, A.stride(1)) if m == 1 else A.stride(1)


@dataclass
class IDResult:
    perm: torch.Tensor            # (n,) int32: S = perm[:k], rd = perm[k:]
    k: int
    ranks: np.ndarray             # cumulative rank after each block
    residuals: np.ndarray         # squared relative residual estimate after each block
    t_ms: np.ndarray              # cumulative device time after each block, ms
    res0: float
    err_est: float
    draws: int
    ms_total: float
    ms_loop: float
    ms_T: float
    nblocks: int
    T: torch.Tensor = field(default=None)  # (k, n-k) FP64, column major, or None

    @property
    def S(self):
        return self.perm[: self.k]

    @property
    def rd(self):
        return self.perm[self.k:]


class Handle:
    """Owns a library handle (device workspace, CUDA stream, last result)."""

    def __init__(self, device=None):
        self.lib = _lib.load()
        if device is None:
            device = torch.cuda.current_device()
        self.device = int(device)
        h = ctypes.c_void_p()
        check(self.lib.rbrp_create(ctypes.byref(h), self.device))
        self.h = h
        self.n_last = None
        # work counter: advanced by every call that launches work or changes the last run's
        # results, so a caller can tell whether those results are still the ones it made
        self.epoch = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.rbrp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _params(self, b, tol, kmax, seed, sampler, tol_loc, compute_T, precision, recompute):
        p = Params()
        self.lib.rbrp_params_default(ctypes.byref(p))
        p.b = int(b)
        p.tol = 0.0 if tol is None else float(tol)
        p.kmax = int(kmax or 0)
        p.seed = int(seed)
        p.sampler = _lib.SAMPLERS[sampler]
        p.tol_loc = 0.0 if tol_loc is None else float(tol_loc)
        p.compute_T = int(bool(compute_T))
        p.precision = _lib.PRECISIONS[precision]
        p.recompute = int(bool(recompute))
        return p

    def _bind_stream(self, stream, work=True):
        check(self.lib.rbrp_set_stream(self.h, ctypes.c_void_p(stream.cuda_stream)), self.h)
        if work:
            self.epoch += 1

    def column_id(self, A, b=64, tol=1e-12, kmax=None, seed=0, sampler="np", tol_loc=None,
                  compute_T=True, recompute=True, stream=None):
        """Adaptive RBRP column ID of the CUDA matrix ``A`` (m x n, FP64 or FP32).

        FP64 runs the plain form, FP32 the mixed-precision form.  ``tol``
        bounds the squared relative residual.  Returns an :class:`IDResult`.
        """
        if not A.is_cuda:
            raise ValueError("A must be a CUDA tensor (use column_id_host for host arrays)")
        if A.dtype not in (torch.float64, torch.float32):
            raise TypeError("A must be float64 or float32")
        A = _colmajor(A)
        m, n = A.shape
        prec = "f64" if A.dtype == torch.float64 else "f32_mixed"
        p = self._params(b, tol, kmax, seed, sampler, tol_loc, compute_T, prec, recompute)
        self._bind_stream(torch.cuda.current_stream(A.device) if stream is None else stream)
        perm = torch.empty(n, dtype=torch.int32, device=A.device)
        r = Result()
        fn = self.lib.rbrp_id_f64 if A.dtype == torch.float64 else self.lib.rbrp_id_f32
        check(fn(self.h, m, n, ctypes.c_void_p(A.data_ptr()), _ld(A), ctypes.byref(p),
                 ctypes.c_void_p(perm.data_ptr()), ctypes.byref(r)), self.h)
        self.n_last = n
        res = self._result(r, perm)
        if compute_T:
            res.T = self.T()
        return res

    def _result(self, r, perm):
        nb = ctypes.c_int()
        check(self.lib.rbrp_get_trace(self.h, None, None, None, 0, ctypes.byref(nb)), self.h)
        ranks = np.zeros(nb.value, np.int32)
        errs = np.zeros(nb.value, np.float64)
        tms = np.zeros(nb.value, np.float64)
        check(self.lib.rbrp_get_trace(self.h, ranks.ctypes.data_as(ctypes.c_void_p),
                                      errs.ctypes.data_as(ctypes.c_void_p),
                                      tms.ctypes.data_as(ctypes.c_void_p), nb.value, ctypes.byref(nb)), self.h)
        return IDResult(perm=perm, k=r.k, ranks=ranks, residuals=errs, t_ms=tms, res0=r.res0,
                        err_est=r.err_est, draws=int(r.draws), ms_total=r.ms_total, ms_loop=r.ms_loop,
                        ms_T=r.ms_T, nblocks=r.nblocks)

    def T(self):
        """T of the last run as a (k, n-k) column-major FP64 CUDA tensor (a copy)."""
        ptr, ld = ctypes.c_void_p(), ctypes.c_int()
        check(self.lib.rbrp_T_device(self.h, ctypes.byref(ptr), ctypes.byref(ld)), self.h)
        k, nc = ld.value, self.n_last - ld.value
        out = torch.empty((nc, k), dtype=torch.float64, device=f"cuda:{self.device}").t()
        if k > 0 and nc > 0:
            check(self.lib.rbrp_copy_T(self.h, ctypes.c_void_p(out.data_ptr()), k), self.h)
        return out

    def L(self):
        """The notebook's L = A^T Q of the last run (python/RBRP.ipynb cell 11): an (n, k) FP64
        CUDA tensor, row j for column j of A, column a for basis vector a; zero where the column
        was chosen before basis vector a.  Basis vectors follow a positive-diagonal panel factor,
        so a column may have the opposite sign of the notebook's (LAPACK) one; the interpolation
        matrix derived from L does not depend on those signs."""
        ptr, ld = ctypes.c_void_p(), ctypes.c_int()
        check(self.lib.rbrp_T_device(self.h, ctypes.byref(ptr), ctypes.byref(ld)), self.h)
        k, n = ld.value, self.n_last
        out = torch.empty((k, n), dtype=torch.float64, device=f"cuda:{self.device}").t()
        if k > 0 and n > 0:
            check(self.lib.rbrp_copy_L(self.h, ctypes.c_void_p(out.data_ptr()), n), self.h)
        return out

    def T_matdivide(self, tol=1e-12):
        """T of the last run as pinv_tol(R11) R12 (the notebook's ``matdivide``, python/RBRP.ipynb
        cell 2 lines 111-126): returns ``(T, rank)``, T a (k, n-k) column-major FP64 CUDA tensor
        and rank the number of singular values of R11 above ``tol``.  Later ``T()`` calls
        return the same matrix until the next run."""
        rank = ctypes.c_int()
        self.epoch += 1
        check(self.lib.rbrp_T_matdivide(self.h, float(tol), ctypes.byref(rank)), self.h)
        return self.T(), rank.value

    def refine_T(self, A, steps=1, tol=0.0):
        """FP64 iterative refinement of the last run's T against ``A`` (the CUDA matrix the run
        used): each step adds pinv(A_S) (A_rd - A_S T), computed in FP64 on A's exact values.
        Returns |dT|_F / |T|_F of the last step; ``T()`` then returns the refined T."""
        A = _colmajor(A)
        m, n = A.shape
        ch = ctypes.c_double()
        fn = self.lib.rbrp_refine_T_f64 if A.dtype == torch.float64 else self.lib.rbrp_refine_T_f32
        self.epoch += 1
        check(fn(self.h, m, n, ctypes.c_void_p(A.data_ptr()), _ld(A), int(steps), float(tol), ctypes.byref(ch)),
              self.h)
        return ch.value

    def set_profiling(self, on=True):
        """Bracket every phase with CUDA events (accumulated until reset)."""
        check(self.lib.rbrp_set_profiling(self.h, int(bool(on))), self.h)

    def set_variant(self, variant):
        """Projection and update kernels of the FP32 form: 0 = tcgen05 (default), 1 = CUDA-core FFMA."""
        check(self.lib.rbrp_set_variant(self.h, int(variant)), self.h)

    def set_tsolve_fp64(self, on=True):
        """T solve on the FP64 pipe (True) or in double-float on the FP32 pipe (False, default)."""
        check(self.lib.rbrp_set_tsolve_fp64(self.h, int(bool(on))), self.h)

    def set_wait_budget(self, cycles=0):
        """Limit (SM clock cycles) of the bounded device-side waits launched through this
        handle (the LU grid barrier, the tcgen05 projection's mbarriers); 0 = default (~2 s).
        A few cycles makes them run out: calls then raise status 7 (device wait timed out)."""
        check(self.lib.rbrp_set_wait_budget(self.h, int(cycles)), self.h)

    def reset_phase_stats(self):
        check(self.lib.rbrp_reset_phase_stats(self.h), self.h)

    def phase_stats(self):
        """{phase: dict(ms, bytes, flops, launches)} accumulated since the last reset."""
        st = _lib.PhaseStats()
        check(self.lib.rbrp_get_phase_stats(self.h, ctypes.byref(st)), self.h)
        return {name: dict(ms=st.ms[q], bytes=st.bytes[q], flops=st.flops[q], launches=st.launches[q])
                for q, name in enumerate(_lib.PHASES)}

    def id_error(self, A):
        """Squared relative ID error of the last run, recomputed in FP64 on the device."""
        A = _colmajor(A)
        m, n = A.shape
        e = ctypes.c_double()
        fn = self.lib.rbrp_id_error_f64 if A.dtype == torch.float64 else self.lib.rbrp_id_error_f32
        check(fn(self.h, m, n, ctypes.c_void_p(A.data_ptr()), _ld(A), ctypes.byref(e)), self.h)
        return e.value

    def column_id_host(self, A, b=64, tol=1e-12, kmax=None, seed=0, sampler="np", tol_loc=None,
                       compute_T=True, recompute=True, perm_out=None, T_out=None):
        """Host-buffer form: ``A`` is a host CPU tensor or numpy array (FP64 or FP32).

        The host-to-device copy of A and the device-to-host copies of perm
        and T happen inside the call (pinned buffers make them fast).
        ``T_out`` needs room for ``min(m, n) * n`` FP64 values; T is written
        column major with leading dimension ``min(m, n)``.  Returns
        ``(k, perm_out, T, result)`` where ``T`` is a (k, n-k) view of ``T_out``.
        """
        if isinstance(A, torch.Tensor):
            if A.is_cuda:
                raise ValueError("column_id_host takes host memory")
            A = _colmajor(A)
            ptr, (m, n), lda, is64 = A.data_ptr(), A.shape, _ld(A), A.dtype == torch.float64
        else:
            A = np.asfortranarray(A)
            if A.dtype not in (np.float64, np.float32):
                raise TypeError("A must be float64 or float32")
            ptr, (m, n), lda, is64 = A.ctypes.data, A.shape, A.shape[0], A.dtype == np.float64
        prec = "f64" if is64 else "f32_mixed"
        p = self._params(b, tol, kmax, seed, sampler, tol_loc, compute_T, prec, recompute)
        self._bind_stream(torch.cuda.current_stream(self.device))
        kcap = min(m, n)
        if perm_out is None:
            perm_out = np.empty(n, np.int32)
        if T_out is None and compute_T:
            T_out = np.empty(kcap * n, np.float64)
        _ptr = lambda x: 0 if x is None else (x.data_ptr() if isinstance(x, torch.Tensor) else x.ctypes.data)
        _len = lambda x: 0 if x is None else (x.numel() if isinstance(x, torch.Tensor) else x.size)
        r = Result()
        fn = self.lib.rbrp_id_f64_host if is64 else self.lib.rbrp_id_f32_host
        check(fn(self.h, m, n, ctypes.c_void_p(ptr), lda, ctypes.byref(p), ctypes.c_void_p(_ptr(perm_out)),
                 ctypes.c_void_p(_ptr(T_out)) if compute_T else None, kcap, _len(T_out), ctypes.byref(r)), self.h)
        self.n_last = n
        T = None
        if compute_T and T_out is not None:
            k, nc = r.k, n - r.k
            T = T_out[: kcap * nc].reshape(nc, kcap).T[:k] if nc > 0 else T_out[:0]
        return r.k, perm_out, T, r


@dataclass
class BatchIDResult:
    """Per-problem outputs of a batched run (arrays indexed by problem)."""
    k: np.ndarray
    nblocks: np.ndarray
    status: np.ndarray
    attempts: np.ndarray
    res0: np.ndarray
    err_est: np.ndarray
    draws: np.ndarray
    alg_bytes: np.ndarray  # algorithmic HBM bytes per problem (minimum traffic)
    alg_flops: np.ndarray  # algorithmic flops per problem
    perms: Sequence      # (n_q,) int32 CUDA views: S = perm[:k], rd = perm[k:]
    Ts: Sequence         # (k_q, n_q - k_q) FP64 column-major CUDA views, or None
    ms: float            # device time of the run (CUDA events), ms


class Batch:
    """A planned batch of independent column IDs run in one persistent launch.

    ``As`` is a sequence of FP32 matrices of any shapes, either all CUDA
    tensors on one device or all column-major views of pinned host memory
    (``pin_memory``).  Host-resident matrices are read in place by the kernel,
    each once over the host link, while other problems compute; their perm
    and T buffers are then pinned host memory too, so a run moves no data
    through separate copies.  ``b <= 0`` lets the library's autotuner pick the
    block size on this batch.  ``tol`` bounds the squared relative residual of
    every problem; problem q uses the Philox key ``seed + q``.  T of problem q
    gets room for ``min(kcap_q, t_rank_cap)`` rows (kcap_q = min(m_q, n_q,
    kmax)); a larger rank reports status 6.
    """

    def __init__(self, handle, As, b=0, tol=1e-8, kmax=None, seed=0, sampler="np", tol_loc=None,
                 compute_T=True, t_rank_cap=None):
        self.h = handle
        lib = handle.lib
        As = list(As)
        if not As:
            raise ValueError("empty batch")
        self.host = not As[0].is_cuda
        if self.host:
            for A in As:
                if A.is_cuda or A.dtype != torch.float32 or not A.is_pinned():
                    raise TypeError("host-resident batches take FP32 views of pinned host memory")
                if _colmajor(A) is not A:
                    raise ValueError("host-resident matrices must be column-major views (no copies are made)")
            dev = torch.device("cuda", handle.device)
            out = dict(device="cpu", pin_memory=True)
        else:
            As = [_colmajor(A) for A in As]
            dev = As[0].device
            for A in As:
                if not A.is_cuda or A.dtype != torch.float32 or A.device != dev:
                    raise TypeError("the batched form takes FP32 CUDA matrices on one device")
            out = dict(device=dev)
        self.As = As
        self.device = dev
        shapes = [tuple(A.shape) for A in self.As]
        self.shapes = shapes
        ns = np.array([n for _, n in shapes], np.int64)
        self.perm_off = np.concatenate([[0], np.cumsum(ns)])
        self.perm_buf = torch.empty(int(self.perm_off[-1]), dtype=torch.int32, **out)
        kc = [min(m, n, kmax or min(m, n)) for m, n in shapes]
        if t_rank_cap is not None:
            kc = [min(k, int(t_rank_cap)) for k in kc]
        tcap = np.array([k * n for k, (_, n) in zip(kc, shapes)], np.int64) if compute_T else np.zeros(len(shapes),
                                                                                                       np.int64)
        self.t_off = np.concatenate([[0], np.cumsum(tcap)])
        self.T_buf = torch.empty(max(1, int(self.t_off[-1])), dtype=torch.float64, **out)
        n_prob = len(self.As)
        self.probs = (_lib.BatchProblem * n_prob)()
        for q, A in enumerate(self.As):
            pr = self.probs[q]
            pr.m, pr.n = shapes[q]
            pr.lda = _ld(A)
            pr.A = A.data_ptr()
            pr.perm = self.perm_buf.data_ptr() + 4 * int(self.perm_off[q])
            pr.T = (self.T_buf.data_ptr() + 8 * int(self.t_off[q])) if compute_T and tcap[q] > 0 else None
            pr.T_cap = int(tcap[q])
        self.compute_T = compute_T
        p = handle._params(b if b and b > 0 else 0, tol, kmax, seed, sampler, tol_loc, compute_T, "f32_mixed", True)
        handle._bind_stream(torch.cuda.current_stream(dev))
        check(lib.rbrp_batch_plan(handle.h, n_prob, self.probs, ctypes.byref(p)), handle.h)
        self.n_prob = n_prob
        # a handle holds one plan: a later Batch on the same handle replaces this one
        self._token = object()
        handle._batch_token = self._token

    def _check_plan(self):
        if getattr(self.h, "_batch_token", None) is not self._token:
            raise RuntimeError("another Batch was planned on this handle since: use one handle per live Batch")

    def info(self):
        self._check_plan()
        inf = _lib.BatchInfo()
        check(self.h.lib.rbrp_batch_get_info(self.h.h, ctypes.byref(inf)), self.h.h)
        return dict(b=inf.b, panel_cols=inf.panel_cols, ctas=inf.ctas, ctas_per_sm=inf.ctas_per_sm,
                    ms_last=inf.ms_last, ms_autotune=inf.ms_autotune, workspace_bytes=inf.workspace_bytes)

    def set_order(self, order):
        """Queue order of the persistent CTAs (problem indices, each once); results do not
        depend on it.  The plan's default is largest m*n first."""
        self._check_plan()
        arr = (ctypes.c_int * self.n_prob)(*[int(q) for q in order])
        check(self.h.lib.rbrp_batch_set_order(self.h.h, arr, len(order)), self.h.h)

    def set_profiling(self, on=True):
        """In-kernel phase cycle counters (reset when switched on)."""
        self._check_plan()
        check(self.h.lib.rbrp_batch_set_profiling(self.h.h, int(bool(on))), self.h.h)

    def phase_cycles(self):
        """{phase: SM cycles summed over CTAs} accumulated since profiling was switched on."""
        self._check_plan()
        n = len(_lib.BATCH_PHASES)
        buf = (ctypes.c_double * n)()
        check(self.h.lib.rbrp_batch_get_phase_cycles(self.h.h, buf, n), self.h.h)
        return dict(zip(_lib.BATCH_PHASES, list(buf)))

    def run(self, stream=None):
        """Enqueue the batch (one CUDA graph launch) on the current torch stream."""
        self._check_plan()
        self.h._bind_stream(torch.cuda.current_stream(self.device) if stream is None else stream)
        check(self.h.lib.rbrp_batch_run(self.h.h), self.h.h)

    def _perm_view(self, q):
        return self.perm_buf[int(self.perm_off[q]): int(self.perm_off[q + 1])]

    def _T_view(self, q, kq, status):
        if not self.compute_T or status != 0:
            return None
        n = self.shapes[q][1]
        if 0 < kq < n:
            return self.T_buf[int(self.t_off[q]): int(self.t_off[q]) + kq * (n - kq)].view(n - kq, kq).t()
        return torch.empty((kq, n - kq), dtype=torch.float64, device=self.T_buf.device,
                           pin_memory=self.host)

    def results(self):
        """Wait for the last run and return a :class:`BatchIDResult`.

        The per-problem fields are numpy arrays read in one pass; ``perms`` and
        ``Ts`` are sequences whose views (CUDA, or pinned CPU for a host-resident
        batch) are made when indexed.
        """
        self._check_plan()
        out = (_lib.BatchResult * self.n_prob)()
        check(self.h.lib.rbrp_batch_results(self.h.h, out, self.n_prob), self.h.h)
        arr = np.ctypeslib.as_array(out)
        k = arr["k"].astype(np.int64)
        status = arr["status"].astype(np.int64)
        perms = _Views(self.n_prob, self._perm_view)
        Ts = _Views(self.n_prob, lambda q: self._T_view(q, int(k[q]), int(status[q])))
        return BatchIDResult(k=k, nblocks=arr["nblocks"].astype(np.int64), status=status,
                             attempts=arr["attempts"].astype(np.int64), res0=arr["res0"].astype(np.float64),
                             err_est=arr["err_est"].astype(np.float64), draws=arr["draws"].astype(np.uint64),
                             alg_bytes=arr["alg_bytes"].astype(np.float64),
                             alg_flops=arr["alg_flops"].astype(np.float64), perms=perms, Ts=Ts,
                             ms=self.info()["ms_last"])


class _Views(Sequence):
    """Read-only sequence of per-problem views, each made on first access."""

    def __init__(self, n, make):
        self._n, self._make, self._cache = n, make, {}

    def __len__(self):
        return self._n

    def __getitem__(self, q):
        if isinstance(q, slice):
            return [self[x] for x in range(*q.indices(self._n))]
        q = int(q)
        if q < 0:
            q += self._n
        if not 0 <= q < self._n:
            raise IndexError(q)
        if q not in self._cache:
            self._cache[q] = self._make(q)
        return self._cache[q]


def packed_offsets(shapes):
    """Float offsets of matrices packed back to back, each column major and starting on a
    16-byte boundary (offsets rounded up to 4 floats): the layout :class:`HostBatch` reads.
    Aligned starts let the batched kernel load the first block with 16-byte vectors."""
    sizes = np.array([int(m) * int(n) for m, n in shapes], np.int64)
    padded = (sizes + 3) // 4 * 4
    return np.concatenate([[0], np.cumsum(padded)]), sizes


class HostBatch:
    """Batched column IDs of FP32 matrices held in pinned host memory, with the
    host-to-device copies overlapped with the IDs.

    ``host_pack`` is one pinned FP32 CPU tensor holding the matrices back to
    back (each column major, ``shapes[q] = (m_q, n_q)``, starting at
    ``packed_offsets(shapes)[0][q]``).  The problems are cut
    into ``parts`` consecutive groups of about equal size; each group has its
    own handle, device buffer and plan.  :meth:`run` enqueues every group's
    host-to-device copy on one copy stream and, on one compute stream, each
    group's graph launch (after its copy's event) and the copies of its perm
    and T back to pinned host buffers: group g + 1's copy runs while group g
    computes, and the groups' persistent kernels never run at the same time
    (concurrent ones take SMs from each other's largest problems).  A group
    still balances its load over fewer problems than one launch over all of
    them, so more groups hide more of the copy but lengthen the compute.
    Problem q keeps the Philox key
    ``seed + q`` and every group uses the block size the first group's autotuner
    chose, so the results are those of one batch over all problems with that b.
    """

    def __init__(self, host_pack, shapes, parts=2, b=0, tol=1e-8, kmax=None, seed=0, sampler="np", tol_loc=None,
                 compute_T=True, t_rank_cap=None, device=None):
        if host_pack.is_cuda or host_pack.dtype != torch.float32 or not host_pack.is_pinned():
            raise TypeError("host_pack must be a pinned FP32 CPU tensor")
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else int(device))
        offs, sizes = packed_offsets(shapes)
        if offs[-1] != host_pack.numel():
            raise ValueError("host_pack does not hold the listed shapes in the packed_offsets layout")
        parts = max(1, min(int(parts), len(shapes)))
        cuts = [0] + [int(np.searchsorted(offs, g * offs[-1] / parts)) for g in range(1, parts)] + [len(shapes)]
        cuts = sorted(set(min(max(c, 0), len(shapes)) for c in cuts))
        self.compute_T = compute_T
        self.groups = []
        b_used = b if b and b > 0 else 0
        for q0, q1 in zip(cuts[:-1], cuts[1:]):
            if q1 <= q0:
                continue
            base = int(offs[q0])
            dpack = torch.empty(int(offs[q1]) - base, dtype=torch.float32, device=dev)
            views = [dpack[int(offs[q]) - base: int(offs[q]) - base + int(sizes[q])]
                     .view(int(shapes[q][1]), int(shapes[q][0])).t() for q in range(q0, q1)]
            h = Handle(dev.index)
            bt = Batch(h, views, b=b_used, tol=tol, kmax=kmax, seed=seed + q0, sampler=sampler, tol_loc=tol_loc,
                       compute_T=compute_T, t_rank_cap=t_rank_cap)
            if b_used <= 0:
                b_used = bt.info()["b"]
            self.groups.append(dict(
                q0=q0, q1=q1, dpack=dpack, handle=h, batch=bt, host=host_pack[base: int(offs[q1])],
                perm_h=torch.empty(bt.perm_buf.numel(), dtype=torch.int32, pin_memory=True),
                T_h=torch.empty(bt.T_buf.numel() if compute_T else 0, dtype=torch.float64, pin_memory=True)))
        self.b = b_used
        self.copy_stream = torch.cuda.Stream(dev)
        self.compute_stream = torch.cuda.Stream(dev)
        self.streams = [self.copy_stream, self.compute_stream]
        self.h2d_bytes = int(host_pack.numel() * 4)
        self.d2h_bytes = int(sum(G["perm_h"].numel() * 4 + G["T_h"].numel() * 8 for G in self.groups))

    def run(self):
        """Enqueue every group: copy in, graph launch, perm and T out (no host wait)."""
        cs, ks = self.copy_stream, self.compute_stream
        # the copy stream must not overwrite a group's buffer before the previous run's
        # graph has read it: start behind the compute stream's last work
        cs.wait_stream(ks)
        arrived = []
        for G in self.groups:
            with torch.cuda.stream(cs):
                G["dpack"].copy_(G["host"], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                arrived.append(ev)
        for G, ev in zip(self.groups, arrived):
            ks.wait_event(ev)
            with torch.cuda.stream(ks):
                G["batch"].run(ks)
                G["perm_h"].copy_(G["batch"].perm_buf, non_blocking=True)
                if self.compute_T:
                    G["T_h"].copy_(G["batch"].T_buf, non_blocking=True)

    def results(self):
        """Wait for the last run; per group ``(first problem, BatchIDResult)`` with host perm and T buffers done."""
        out = []
        for G in self.groups:
            out.append((G["q0"], G["batch"].results()))
        for s in self.streams:
            s.synchronize()
        return out

    def host_perm(self, q):
        """perm of problem q from the pinned host buffer of the last run."""
        for G in self.groups:
            if G["q0"] <= q < G["q1"]:
                bt = G["batch"]
                j = q - G["q0"]
                return G["perm_h"][int(bt.perm_off[j]): int(bt.perm_off[j + 1])]
        raise IndexError(q)

    def close(self):
        for G in self.groups:
            G["handle"].close()


def batched_column_id(As, b=0, tol=1e-8, kmax=None, seed=0, sampler="np", tol_loc=None, compute_T=True,
                      t_rank_cap=None, handle=None):
    """Column IDs of many FP32 matrices (CUDA tensors, or column-major views of pinned host
    memory) in one persistent launch (plan, run, results)."""
    h = handle or Handle(As[0].device.index)
    bt = Batch(h, As, b=b, tol=tol, kmax=kmax, seed=seed, sampler=sampler, tol_loc=tol_loc, compute_T=compute_T,
               t_rank_cap=t_rank_cap)
    bt.run()
    return bt.results()


_rt = None


def _cudart():
    """The CUDA runtime already loaded by the library (for raw device copies)."""
    global _rt
    if _rt is None:
        _lib.load()
        _rt = ctypes.CDLL("libcudart.so.13")
        _rt.cudaMemcpy.restype = ctypes.c_int
        _rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return _rt


def _copy_device(src_ptr, dst, nbytes):
    if nbytes > 0 and src_ptr:
        rc = _cudart().cudaMemcpy(ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src_ptr), nbytes, 3)
        if rc != 0:
            raise _lib.RBRPError(2, f"cudaMemcpy failed ({rc})")


def _fp64_colmajor(A):
    A = _colmajor(A)
    if A.dtype != torch.float64 or A.stride(1) != A.shape[0]:
        A = A.to(torch.float64).t().contiguous().t()
    return A


def RBRP(A, blk):
    """``RBRP(m, n, A, blk, ...)`` of ``gpu/rbrp.hpp:6-8`` on a CUDA matrix (FP64, ld = m).

    Returns ``(ranks, error, t_ranks, t_rbrp, flops)``: cumulative ranks,
    squared relative residual per block, cumulative seconds per block, total
    seconds and the algorithmic flop count.
    """
    lib = _lib.load()
    A = _fp64_colmajor(A)
    m, n = A.shape
    cap = min(m, n)
    ranks = np.zeros(cap, np.int32)
    err = np.zeros(cap, np.float64)
    tr = np.zeros(cap, np.float64)
    nb, t, f = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
    with torch.cuda.device(A.device):
        check(lib.rbrp_RBRP(m, n, ctypes.c_void_p(A.data_ptr()), int(blk), ranks.ctypes.data_as(ctypes.c_void_p),
                            err.ctypes.data_as(ctypes.c_void_p), tr.ctypes.data_as(ctypes.c_void_p), cap,
                            ctypes.byref(nb), ctypes.byref(t), ctypes.byref(f)))
    k = nb.value
    return ranks[:k], err[:k], tr[:k], t.value, f.value


def rand_adap_rbrp(A, tol=1e-8, blk=16):
    """``RandAdapLUPP(A, m, n, sk, rd, T, rank, flops, tol, blk)`` (``gpu/rid.hpp:5-7``) with RBRP pivoting.

    Returns ``(sk, rd, T, rank, flops)`` as CUDA tensors (sk, rd int32; T FP64
    rank x (n - rank), column major).  ``tol`` bounds the squared residual.
    """
    lib = _lib.load()
    A = _fp64_colmajor(A)
    m, n = A.shape
    sk, rd, T = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    rank, flops = ctypes.c_int(), ctypes.c_double()
    with torch.cuda.device(A.device):
        check(lib.rbrp_RandAdapRBRP(ctypes.c_void_p(A.data_ptr()), m, n, ctypes.byref(sk), ctypes.byref(rd),
                                    ctypes.byref(T), ctypes.byref(rank), ctypes.byref(flops), float(tol), int(blk)))
        k = rank.value
        try:
            sk_t = torch.empty(k, dtype=torch.int32, device=A.device)
            rd_t = torch.empty(n - k, dtype=torch.int32, device=A.device)
            T_t = torch.empty((n - k, k), dtype=torch.float64, device=A.device).t()
            torch.cuda.synchronize(A.device)
            _copy_device(sk.value, sk_t, 4 * k)
            _copy_device(rd.value, rd_t, 4 * (n - k))
            _copy_device(T.value, T_t, 8 * k * (n - k))
        finally:
            lib.rbrp_free(sk)
            lib.rbrp_free(rd)
            lib.rbrp_free(T)
    return sk_t, rd_t, T_t, k, flops.value


def blocked_rpid(X, k, b=20, tol=None, mode="rp", ortho=1, tol_loc=None, seed=0, handle=None, return_L=False):
    """The notebook's ``blocked_rpid`` contract on the GPU (rows of ``X`` are the items).

    ``X`` is an (n, d) CUDA tensor; the ID is the column ID of ``A = X.T``.
    Only ``ortho=1`` (RBRP) exists.  Returns ``(row_perm, T, residuals,
    time_pivot, ranks)``: the interpolation matrix ``T`` (k x (n-k)) that the
    notebook derives from its ``L``.  With ``return_L=True`` the second entry is
    the notebook's own ``L = X Q`` ((n, k), :meth:`Handle.L`) instead, so the
    notebook's ``get_rpid_error`` / ``interpolation`` take the tuple unchanged.
    """
    if ortho != 1:
        raise ValueError("only ortho=1 (RBRP) is implemented")
    sampler = {"rp": "np", "gp": "greedy"}[mode]
    A = X.t()
    h = handle or Handle(A.device.index)
    r = h.column_id(A, b=b, tol=tol, kmax=k, seed=seed, sampler=sampler, tol_loc=tol_loc)
    return (r.perm.cpu().numpy().astype(np.int64), h.L() if return_L else r.T, r.residuals, r.t_ms * 1e-3,
            r.ranks.astype(np.int64))
