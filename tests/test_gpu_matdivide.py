"""GPU: the truncated-SVD interpolation (the notebook's ``matdivide``).

``rbrp_matdivide_f64`` computes pinv_tol(B) C with a one-sided Jacobi SVD in
FP64; the oracle restates ``matdivide`` (python/RBRP.ipynb cell 2 lines
111-126) with LAPACK's SVD.  Inputs have a clear gap in their singular values
around the cutoff, so both keep the same rank and the pseudo-inverse solutions
agree to rounding (relative Frobenius ~kappa^2 eps); an exactly dependent
column must be cut.  ``rbrp_T_matdivide`` on an RBRP run whose R11 spans seven orders of
magnitude must equal the notebook's ``matdivide`` on the oracle's factor of
the same skeleton, and equal R11^{-1} R12 when nothing is cut.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import matdivide, rbrp_column_id  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle(rbrp_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    h = Handle(0)
    yield h
    h.close()


def with_spectrum(p, q, s, seed):
    """p x q with singular values s (len <= min(p, q)), random singular vectors."""
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((p, len(s))))
    V, _ = np.linalg.qr(rng.standard_normal((q, len(s))))
    return (U * np.asarray(s)) @ V.T


def rel(X, Y):
    return np.linalg.norm(X - Y) / np.linalg.norm(Y)


@pytest.mark.parametrize("m,k,n,seed", [(5, 3, 7, 1), (40, 24, 60, 2), (130, 97, 300, 3)])
def test_matdivide_matches_notebook(handle, m, k, n, seed):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import matdivide as dev_matdivide
    r_true = max(1, (2 * k) // 3)
    s = np.concatenate([np.logspace(0, -4, r_true), np.full(k - r_true, 1e-15)])
    B = with_spectrum(k, n, s, seed)                       # k x n, numerical rank r_true
    A = np.random.default_rng(seed + 10).standard_normal((m, n))
    X_ref, r_ref = matdivide(A, B, tol=1e-12)
    X, r = dev_matdivide(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), tol=1e-12, handle=handle)
    assert r == r_ref == r_true
    # kappa of the kept part is 1e4: two FP64 pseudo-inverses agree to ~kappa^2 eps
    assert rel(X.cpu().numpy(), X_ref) <= 1e-7


def test_matdivide_cuts_an_exactly_dependent_column(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import matdivide as dev_matdivide
    rng = np.random.default_rng(7)
    B = rng.standard_normal((8, 50))
    B[5] = B[2]                                             # rank 7
    A = rng.standard_normal((20, 50))
    X_ref, r_ref = matdivide(A, B)
    X, r = dev_matdivide(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), handle=handle)
    assert r == r_ref == 7
    assert rel(X.cpu().numpy(), X_ref) <= 1e-9


def test_T_matdivide_on_an_rbrp_run(handle):
    """An RBRP run to squared tol 1e-14 on a spectrum with a gap (20 singular values in
    [1e-2, 1], 20 near 1e-5; every weight stays far above FP64 rounding, so the FP64
    form's skeleton is bit-exact with the oracle's): k = 40 and R11 has 20 singular
    values in [4e-3, 0.5] and 20 in [4e-7, 5e-6].  With cutoff 1e-4 the truncated T is
    the notebook's matdivide applied to the oracle's factor of the same skeleton (R11 =
    triu R(:, S), R12 = R(:, rd)); with a cutoff below every singular value it is
    R11^{-1} R12."""
    s = np.concatenate([np.logspace(0, -2, 20), np.logspace(-5, -5.5, 20)])
    A = with_spectrum(120, 160, s, 11)
    Ad = torch.from_numpy(np.asfortranarray(A)).cuda()
    r = handle.column_id(Ad, b=8, tol=1e-14, seed=0)
    k = r.k
    o = rbrp_column_id(A, 8, tol=1e-14, seed=0)
    assert k == o["k"] == 40 and np.array_equal(r.perm.cpu().numpy(), o["perm"])
    T_tri = r.T.cpu().numpy()
    S, rd = o["perm"][:k], o["perm"][k:]
    R11, R12 = np.triu(o["R"][:k, S]), o["R"][:k, rd]
    T_md, rank = handle.T_matdivide(1e-4)
    W, rank_ref = matdivide(R12.T, R11.T, tol=1e-4)
    assert rank == rank_ref == 20
    assert rel(T_md.cpu().numpy(), W.T) <= 1e-7
    assert np.array_equal(handle.T().cpu().numpy(), T_md.cpu().numpy())
    T_full, rank = handle.T_matdivide(1e-12)
    assert rank == k
    assert rel(T_full.cpu().numpy(), T_tri) <= 1e-6   # kappa(R11) ~ 1e6: both are FP64-level solves
