"""Seeded synthetic input matrices for RBRP column ID.

These stand in for the reference's own test-matrix generators
(``python/RBRP.ipynb`` cell 5 lines 49-107, ``matlab/Matrix_*.m``,
``gpu/driver.cpp:23-111``); no dataset is downloaded.  All random numbers come
from ``numpy.random.Philox`` with key ``seed + 2**64`` (key word 1 = 1), which
keeps them independent of the sampler's uniform stream (key word 1 = 0).

Every generator returns a column-major (Fortran-ordered) ``numpy`` array: the
ID selects *columns*.
"""
import math

import numpy as np

GEN_KEY_HI = 1


def _gen(seed, stream=0):
    """Generator for workload ``stream`` of ``seed`` (independent of the sampler's stream)."""
    return np.random.Generator(np.random.Philox(key=int(seed) + (GEN_KEY_HI << 64),
                                                counter=[0, 0, 0, int(stream)]))


def haar(rng, n):
    """Haar-distributed orthogonal n x n matrix: QR of N(0,1) with the sign of diag(R) fixed."""
    Z = rng.standard_normal((n, n))
    Qm, Rm = np.linalg.qr(Z)
    d = np.sign(np.diag(Rm))
    d[d == 0] = 1.0
    return Qm * d


def gaussian_exp(m=1000, n=1000, decay=20.0, seed=0):
    """A = U diag(s) V^T, U and V Haar, ``s_i = exp(-i/decay)`` for i = 0..min(m,n)-1.

    The plain FP64 single-matrix workload (1000 x 1000, b = 40).  Follows the
    notebook's Gaussian targets (cell 5 lines 71-93) with an exponential spectrum.
    """
    rng = _gen(seed, 0)
    r = min(m, n)
    U = haar(rng, m)[:, :r]
    V = haar(rng, n)[:, :r]
    s = np.exp(-np.arange(r) / decay)
    return np.asfortranarray((U * s) @ V.T)


def snn_factors(m, n, r=2000, r1=100, amp=10.0, density=0.02, seed=0):
    """Factors of the sparse non-negative matrix ``A = X diag(w) Y^T``.

    ``w_j = amp/j`` for j <= r1 and ``1/j`` for r1 < j <= r (1-based);
    ``X`` (m x r) and ``Y`` (n x r) have i.i.d. entries that are nonzero with
    probability ``density`` and Uniform[0, 1] when nonzero.  Follows
    ``generate_sparse_nonnegative_target`` (cell 5 lines 95-107).
    """
    r = min(r, m, n)
    rng = _gen(seed, 1)
    j = np.arange(1, r + 1, dtype=np.float64)
    w = np.where(j <= r1, amp / j, 1.0 / j)
    X = np.where(rng.random((m, r)) < density, rng.random((m, r)), 0.0)
    Y = np.where(rng.random((n, r)) < density, rng.random((n, r)), 0.0)
    return X, w, Y


def snn(m=1024, n=1024, r=2000, r1=100, amp=10.0, density=0.02, seed=0):
    """Dense FP64 sparse-non-negative low-rank-plus-tail matrix (host product)."""
    X, w, Y = snn_factors(m, n, r, r1, amp, density, seed)
    return np.asfortranarray((X * w) @ Y.T)


def gmm(d=1024, npts=65536, nclusters=20, seed=0):
    """Imbalanced Gaussian mixture; columns are points (A is d x npts).

    Means ~ N(0, 4 I), isotropic cluster std ~ U[0.1, 1], cluster sizes
    proportional to ``2**-c`` with at least one point per cluster (cluster 0
    takes the remainder).  Returns ``(A, labels)``.  Follows
    ``genenrate_gmm_target`` (cell 5 lines 49-68) with the imbalanced weights.
    """
    rng = _gen(seed, 2)
    wts = 2.0 ** -np.arange(nclusters)
    sizes = np.maximum(1, np.round(npts * wts / wts.sum()).astype(np.int64))
    sizes[0] = npts - sizes[1:].sum()
    means = 2.0 * rng.standard_normal((d, nclusters))
    sig = rng.uniform(0.1, 1.0, nclusters)
    labels = np.repeat(np.arange(nclusters), sizes)
    A = means[:, labels] + rng.standard_normal((d, npts)) * sig[labels]
    return np.asfortranarray(A), labels


def driver_gmm(npts=1000, d=1000, nclusters=100, seed=0):
    """The Gaussian-mixture test matrix of ``gpu/driver.cpp:94-109``, d x npts.

    i.i.d. N(0, 1) entries; point i belongs to cluster c = i // (npts // nclusters)
    and has 10 (c + 1) added to coordinate c.
    """
    per = npts // nclusters
    if d < 1 or per < 1 or (npts - 1) // per >= d:
        raise ValueError("need npts >= nclusters and d above the cluster count")
    A = _gen(seed, 5).standard_normal((d, npts))
    c = np.arange(npts) // per
    A[c, np.arange(npts)] += 10.0 * (c + 1)
    return np.asfortranarray(A)


def kernel_block_shapes(nblocks=4096, lo=64, hi=2048, seed=0):
    """(m, n) of each off-diagonal kernel block, log-uniform in [lo, hi]."""
    rng = _gen(seed, 3)
    lm = rng.uniform(math.log(lo), math.log(hi), (nblocks, 2))
    return np.clip(np.round(np.exp(lm)).astype(np.int64), lo, hi)


def kernel_block_points(m, n, index, seed=0):
    """The two point clusters of kernel block ``index``: x (m x 3) in the unit
    cube and y (n x 3) in a unit cube whose centre is 2 to 8 away."""
    rng = _gen(seed, 4 + int(index))
    x = rng.random((m, 3))
    direction = rng.standard_normal(3)
    direction /= np.linalg.norm(direction)
    y = rng.random((n, 3)) + rng.uniform(2.0, 8.0) * direction
    return x, y


def kernel_block(m, n, index, lengthscale=0.5, seed=0):
    """Gaussian-kernel block between two clusters of 3-D points in unit cubes.

    Cube centres are 2 to 8 apart; ``A_ij = exp(-|x_i - y_j|^2 / (2 l^2))``.
    """
    x, y = kernel_block_points(m, n, index, seed)
    d2 = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    return np.asfortranarray(np.exp(-d2 / (2.0 * lengthscale ** 2)))


def kernel_block_scaled(m, n, index, lengthscale=0.5, seed=0, dtype=np.float32):
    """``kernel_block / max(kernel_block)``, evaluated without underflow.

    The entries of far-apart blocks lie far below FP32's range (down to
    ~1e-80), so FP32 storage keeps each block scaled by its largest entry:
    ``exp(-(d2 - min d2) / (2 l^2))``.  A column ID is invariant under a
    uniform scale (same S, same T, same relative error).
    """
    x, y = kernel_block_points(m, n, index, seed)
    d2 = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    return np.asfortranarray(np.exp(-(d2 - d2.min()) / (2.0 * lengthscale ** 2)).astype(dtype))


def gaussian_kernel_points(npts=8192, dim=8, seed=0):
    """Points ~ N(0, I_dim) for the differentiable fixed-skeleton workload."""
    return _gen(seed, 5).standard_normal((npts, dim))


def gaussian_kernel(points, lengthscale=1.5):
    """Dense Gaussian kernel matrix of ``points`` (FP64)."""
    sq = (points ** 2).sum(1)
    d2 = np.maximum(sq[:, None] + sq[None, :] - 2.0 * points @ points.T, 0.0)
    return np.asfortranarray(np.exp(-d2 / (2.0 * lengthscale ** 2)))


def zero_prefixed(B, z):
    """``[0_{m x z} | B]``: z zero columns in front of B.

    Zero columns are never sampled, so the block targets ``[i, i+bs)`` are never
    sampled either while ``i + bs <= z``; on such inputs the notebook's own swap
    (with its view bug removed) agrees with the corrected swap, which is what
    lets the reference's unmodified arithmetic pin the oracle.
    """
    m = B.shape[0]
    return np.asfortranarray(np.concatenate([np.zeros((m, z)), B], axis=1))


def kernel_blocks_device(nblocks=4096, lo=64, hi=2048, lengthscale=0.5, seed=0, device="cuda", fp64=False):
    """The batched workload on the device: ``nblocks`` scaled kernel blocks.

    Shapes from :func:`kernel_block_shapes`, points from
    :func:`kernel_block_points` (host, small), entries evaluated on the device
    as in :func:`kernel_block_scaled`.  Returns a list of column-major CUDA
    tensors (FP32, or FP64 with ``fp64=True``).
    """
    import torch
    out = []
    for q, (m, n) in enumerate(kernel_block_shapes(nblocks, lo, hi, seed)):
        x, y = kernel_block_points(int(m), int(n), q, seed)
        xd = torch.from_numpy(x).to(device)
        yd = torch.from_numpy(y).to(device)
        d2 = ((xd[:, None, :] - yd[None, :, :]) ** 2).sum(-1)
        A = torch.exp(-(d2 - d2.min()) / (2.0 * lengthscale ** 2))
        A = A if fp64 else A.to(torch.float32)
        out.append(A.t().contiguous().t())
    return out
