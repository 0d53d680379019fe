"""CPU oracle: adaptive RBRP column interpolative decomposition (numpy/scipy, FP64).

TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
against; nothing in the product path imports it.

It restates the reference's Python RBRP, ``blocked_rpid`` with ``ortho=1`` and
``mode='rp'`` (``python/RBRP.ipynb`` cell 11 lines 76-173), transposed from the
notebook's row convention (``X`` is n x d, rows are items) to a column ID of
``A`` (m x n, columns are items; ``A = X.T``).  Two corrections are applied,
both following ``matlab/RBRP.m``:

1. The block swap.  The notebook's ``aux = row_perm[i:i+block_size]`` is a numpy
   *view* (cell 11 lines 126-128), so the swap duplicates the sampled entries
   and drops the displaced ones whenever a sampled position lies outside
   ``[i, i+bs)``.  The oracle uses the ``setdiff(...,'stable')`` swap of
   ``matlab/RBRP.m:81-99``: positions of the block not selected (ascending)
   are paired with selected positions outside the block (in pivot order).
2. The zero-residual stop.  The notebook tests ``diags[row_perm[i+1:]]``
   (cell 11 line 164), skipping position ``i``; the oracle tests every remaining
   position, as ``matlab/RBRP.m:113-116`` does.

One extension, for termination: if the robust filter keeps no column (the
sampled panel is numerically zero) the sampled columns' weights are zeroed
and the loop continues; the notebook and MATLAB loop forever in that case.

Everything else is the notebook's arithmetic: squared column norms, weights
``diags / sum(diags)``, ``Generator.choice(replace=False, p=...)`` semantics,
one classical Gram-Schmidt pass against the previous basis, LAPACK pivoted QR
(``scipy.linalg.qr(pivoting=True)`` = dgeqp3) of the panel, the local clip
``_block_size_local_clip`` with ``tol_loc = 1/b``, the projection
``L = A^T Q_blk`` with FP64 norm downdate and clip at zero, and the squared
residual stopping rule ``residual < residual_0 * tol``.
"""
import numpy as np
import scipy.linalg as spla

from .philox import PhiloxStream, es_uniforms


# --------------------------------------------------------------------------
# block sampler: numpy Generator.choice(replace=False, p=w/sum(w))
# --------------------------------------------------------------------------
def np_compat_choice(weights, size, random):
    """Weighted sampling without replacement, numpy ``Generator.choice`` semantics.

    Follows ``python/RBRP.ipynb`` cell 11 line 108, whose ``rng.choice(n-i,
    size=b, p=diags/sum(diags), replace=False)`` runs numpy's published
    rejection scheme: draw ``size - found`` uniforms; zero the weights of the
    indices already found; build ``cdf = cumsum(p) / cdf[-1]``; map each uniform
    with ``searchsorted(side='right')``; keep first occurrences in draw order;
    repeat until ``size`` distinct indices are found.  ``random(n)`` supplies
    the uniforms.  ``size`` is capped at the number of positive weights (the
    caller already caps it; numpy would raise instead).
    """
    w = np.asarray(weights, dtype=np.float64)
    total = sum(w)  # the notebook normalises with Python's sequential sum
    p = w / total
    size = int(min(size, np.count_nonzero(p > 0)))
    found = np.zeros(size, dtype=np.int64)
    n_uniq = 0
    while n_uniq < size:
        x = random(size - n_uniq)
        if n_uniq > 0:
            p[found[:n_uniq]] = 0
        cdf = np.cumsum(p)
        cdf /= cdf[-1]
        new = cdf.searchsorted(x, side="right")
        _, first = np.unique(new, return_index=True)
        first.sort()
        new = new.take(first)
        found[n_uniq:n_uniq + new.size] = new
        n_uniq += new.size
    return found


def es_topb(weights, size, u):
    """Exponential-key (Efraimidis-Spirakis) weighted sampling without replacement.

    Key of item j is ``-log(1 - u_j) / w_j`` (an Exp(w_j) variate); the sample
    is the ``size`` smallest keys, returned in ascending key order, which is
    the order a sequential without-replacement draw would produce.  Items
    with zero weight are never chosen; ties break toward the lower index.
    """
    w = np.asarray(weights, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    pos = w > 0
    size = int(min(size, np.count_nonzero(pos)))
    keys = np.full(w.shape, np.inf)
    keys[pos] = -np.log(1.0 - u[pos]) / w[pos]
    order = np.lexsort((np.arange(w.size), keys))
    return order[:size].astype(np.int64)


# --------------------------------------------------------------------------
# robust block filter
# --------------------------------------------------------------------------
def local_clip(R, tol):
    """Number of leading pivots kept by the robust filter.

    Restates ``_block_size_local_clip`` (``python/RBRP.ipynb`` cell 11 lines
    69-73): reverse cumulative sums of the squared row norms of the panel's R,
    relative to the total; keep every row if the last relative sum is at least
    ``tol``, else keep the rows before the first relative sum below ``tol``.
    A zero panel keeps nothing.
    """
    rn = spla.norm(R, ord=2, axis=1) ** 2
    rncs = np.flip(np.flip(rn).cumsum())
    if not rncs.size or rncs[0] == 0.0:
        return 0
    rel = rncs / rncs[0]
    return int(R.shape[0] if rel[-1] >= tol else np.argmax(rel < tol))


# --------------------------------------------------------------------------
# block swap (matlab/RBRP.m:81-99)
# --------------------------------------------------------------------------
def corrected_swap(perm, i, kept):
    """Move the kept positions ``kept`` (pivot order) to ``[i, i+len(kept))`` in place.

    ``K1`` = block positions not kept (ascending), ``K2`` = kept positions
    outside the block (pivot order); ``perm[K2] = perm[K1]`` and
    ``perm[i:i+bs] = perm[kept]``, as ``matlab/RBRP.m:81-89``.
    """
    kept = np.asarray(kept, dtype=np.int64)
    bs = kept.size
    in_block = (kept >= i) & (kept < i + bs)
    kset = set(kept.tolist())
    K1 = np.array([p for p in range(i, i + bs) if p not in kset], dtype=np.int64)
    K2 = kept[~in_block]
    T = perm[kept].copy()
    perm[K2] = perm[K1]
    perm[i:i + bs] = T
    return perm


# --------------------------------------------------------------------------
# RBRP column ID
# --------------------------------------------------------------------------
def rbrp_column_id(A, b, tol=None, kmax=None, seed=0, sampler="np", mode="rp",
                   tol_loc=None, rng=None, sampler_impl="restated"):
    """Adaptive RBRP column ID of ``A`` (m x n, FP64).

    ``tol`` bounds the *squared* relative residual, as in the notebook (cell 11
    line 164).  ``sampler``: ``'np'`` (numpy-choice semantics over the
    ``PhiloxStream(seed)`` uniforms, or over ``rng`` when given) or ``'es'``
    (exponential keys over ``es_uniforms``).  ``mode``: ``'rp'`` (random) or
    ``'gp'`` (greedy top-b, cell 11 line 112).  ``sampler_impl='numpy'`` calls
    ``rng.choice`` itself instead of the restatement.

    The per-block trace ``blocks`` holds, for each sampled panel, its positions
    ``js``, the LAPACK pivots ``piv``, the kept count ``bs`` and ``cols_piv``, the
    panel's original columns in pivot order.

    Returns a dict with ``perm`` (position -> original column), ``k``, ``ranks``
    (cumulative per block), ``residuals`` (relative squared residual per
    block), ``Q`` (m x k), ``R`` (k x n, indexed by original column, with the
    panel R on the diagonal blocks as ``matlab/RBRP.m:78``), ``L`` (n x k,
    the notebook's ``A^T Q`` for the columns remaining at each block), the
    per-block trace ``blocks`` and ``draws`` (uniforms consumed).
    """
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    p = min(m, n)
    kmax = p if kmax is None else int(min(kmax, p))
    tol_loc = 1.0 / b if tol_loc is None else tol_loc
    stream = None
    if sampler == "np" and mode == "rp":
        if rng is None:
            stream = PhiloxStream(seed)
            draw = stream.random
        else:
            draw = rng.random

    perm = np.arange(n, dtype=np.int64)
    diags = spla.norm(A, ord=2, axis=0).astype(np.float64) ** 2
    residual = sum(diags)
    res0 = residual
    Q = np.zeros((m, kmax))
    L = np.zeros((n, kmax))
    R = np.zeros((kmax, n))
    residuals, ranks, blocks = [], [], []
    i = 0
    t = 0
    while i < kmax:
        rem = perm[i:]
        w = diags[rem]
        bs = int(min(kmax - i, b, np.count_nonzero(w)))
        if bs == 0:
            break
        if mode == "gp":
            rel = np.argsort(-w, kind="stable")[:bs]
        elif sampler == "np":
            if sampler_impl == "numpy":
                rel = rng.choice(n - i, size=bs, p=w / sum(w), replace=False)
            else:
                rel = np_compat_choice(w, bs, draw)
        elif sampler == "es":
            u = es_uniforms(seed, t, n)[rem]
            rel = es_topb(w, bs, u)
        else:
            raise ValueError(f"sampler {sampler!r}")
        js = i + np.asarray(rel, dtype=np.int64)
        bs_sampled = js.size

        AJ = A[:, perm[js]]
        if i == 0:
            V = AJ.copy()
        else:
            V = AJ - Q[:, :i] @ (Q[:, :i].T @ AJ)
        QV, RV, pV = spla.qr(V, mode="economic", pivoting=True)
        bs = local_clip(RV, tol_loc)
        blocks.append(dict(i=i, js=js.copy(), bs_sampled=bs_sampled, piv=pV.copy(), bs=bs,
                           cols_piv=perm[js[pV]].copy()))
        t += 1
        if bs == 0:
            # numerically zero panel: these columns carry no residual
            diags[perm[js]] = 0.0
            if np.count_nonzero(diags[perm[i:]]) < 1:
                break
            continue
        kept = js[pV[:bs]]
        corrected_swap(perm, i, kept)
        Q[:, i:i + bs] = QV[:, :bs]
        W = A[:, perm[i:]].T @ Q[:, i:i + bs]          # (n - i, bs)
        L[perm[i:], i:i + bs] = W
        R[i:i + bs, perm[i:]] = W.T
        R[i:i + bs, perm[i:i + bs]] = np.triu(RV[:bs, :bs])
        diags[perm[i + bs:]] -= np.sum(W[bs:] ** 2, axis=1)
        diags = diags.clip(min=0)
        residual = sum(diags[perm[i + bs:]])
        i += bs
        residuals.append(residual)
        ranks.append(i)
        if (tol is not None and residual < res0 * tol) or np.count_nonzero(diags[perm[i:]]) < 1:
            break

    k = i
    return dict(
        perm=perm, k=k, ranks=np.array(ranks, dtype=np.int64),
        residuals=np.array(residuals) / res0 if res0 > 0 else np.array(residuals),
        res0=res0, Q=Q[:, :k], L=L[:, :k], R=R[:k], blocks=blocks,
        diags=diags, draws=(stream.draws if stream is not None else None),
    )


# --------------------------------------------------------------------------
# interpolation matrix and ID error
# --------------------------------------------------------------------------
def interp_sid(A, perm, k):
    """T (k x (n-k)) by the stable ID of ``python/RBRP.ipynb`` cell 7 lines 19-22.

    ``Q, R = qr(A[:, S])``; ``T = R^{-1} Q^T A[:, rd]`` with ``S = perm[:k]`` and
    ``rd = perm[k:]`` (the notebook's ``W_perm_sub`` is ``T.T``).
    """
    A = np.asarray(A, dtype=np.float64)
    S, rd = perm[:k], perm[k:]
    Qs, Rs = spla.qr(A[:, S], mode="economic")
    return spla.solve_triangular(Rs, Qs.T @ A[:, rd])


def interp_r11(R, perm, k):
    """T = R11^{-1} R12 from the RBRP factor, as ``matlab/driver.m:86``.

    ``R`` is indexed by original column (k x n); ``R11 = R[:, S]`` is upper
    triangular, ``R12 = R[:, rd]``.
    """
    S, rd = perm[:k], perm[k:]
    return spla.solve_triangular(np.triu(R[:k, S]), R[:k, rd])


def id_error(A, perm, T, relative=True):
    """Squared Frobenius ID error ``||A[:, rd] - A[:, S] T||_F^2`` (cell 7 lines 40-53).

    Relative to ``||A||_F^2`` when ``relative``.
    """
    A = np.asarray(A, dtype=np.float64)
    k = T.shape[0]
    S, rd = perm[:k], perm[k:]
    e = spla.norm(A[:, rd] - A[:, S] @ T, ord="fro") ** 2
    if relative:
        e /= spla.norm(A, ord="fro") ** 2
    return e


def error_at_rank(A, k, b, tol=None, seed=0, sampler="np", mode="rp", run=None):
    """The oracle's squared relative ID error at rank ``k`` (SID interpolation).

    Used to compare another implementation's ID of rank ``k`` with the
    reference's "at the same rank".  The adaptive run (``rbrp_column_id`` with
    ``tol``, or ``run`` when given) fixes the skeleton at every block
    boundary: later block swaps never move positions below the current rank, so
    its final ``perm[:k_t]`` is the skeleton after the block that reached
    ``k_t``.  When ``k`` is such a boundary (or the final rank), the error is
    that skeleton's ("boundary").  When ``k`` falls inside a block's sampled
    panel (``k_t < k <= k_t + sampled``), which is where a robust-filter
    decision near its threshold keeps one pivot more or fewer, the skeleton is
    ``perm[:k_t]`` plus the panel's first ``k - k_t`` pivots ("panel").
    Otherwise the run is repeated with ``kmax = k``, whose last block samples
    only the columns still missing ("capped").

    Returns ``(error, how)`` with ``how`` in ``{"boundary", "panel", "capped"}``.
    """
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[1]
    if run is None:
        run = rbrp_column_id(A, b, tol=tol, seed=seed, sampler=sampler, mode=mode)
    if k <= 0:
        return 1.0, "boundary"
    if k >= n:
        return 0.0, "boundary"
    bounds = set(int(x) for x in run["ranks"]) | {int(run["k"])}
    if k in bounds:
        return id_error(A, run["perm"], interp_sid(A, run["perm"], k)), "boundary"
    # the block that started at the largest boundary below k (the one in progress at rank k)
    starts = [blk for blk in run["blocks"] if int(blk["i"]) < k]
    if starts:
        blk = max(starts, key=lambda x: int(x["i"]))
        i0, cols = int(blk["i"]), blk["cols_piv"]
        if k <= i0 + len(cols):
            S = np.concatenate([run["perm"][:i0], cols[: k - i0]])
            perm = np.concatenate([S, np.setdiff1d(np.arange(n), S)])
            return id_error(A, perm, interp_sid(A, perm, k)), "panel"
    perm = rbrp_column_id(A, b, tol=None, kmax=k, seed=seed, sampler=sampler, mode=mode)["perm"]
    return id_error(A, perm, interp_sid(A, perm, k)), "capped"


def matdivide(A, B, tol=1e-12):
    """``A * pinv(B)`` from the SVD of B, keeping singular values above the absolute
    cutoff ``tol``: restates ``matdivide`` (``python/RBRP.ipynb`` cell 2 lines
    111-126; ``TOL_FP = 1e-12``, cell 0 line 26).  A (m x n), B (k x n); returns
    ``(X, r)`` with X (m x k) and r the number of singular values kept."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    U, s, Vh = spla.svd(B, full_matrices=False)
    r = int(np.count_nonzero(s > tol))
    aux = (A @ Vh[:r].T) / s[:r].reshape(1, -1)
    return aux @ U[:, :r].T, r
