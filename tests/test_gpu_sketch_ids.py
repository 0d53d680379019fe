"""GPU: the comparison IDs (CPQR ID, RandCPQR_OS, SID interpolation modes) and the sketch.

The CPQR skeleton must equal LAPACK dgeqp3's (scipy ``qr(pivoting=True)``)
pivot for pivot on inputs without near-ties, with T = R11^{-1} R12 to 1e-8.
RandCPQR_OS must equal the same construction done by numpy/scipy on the
library's own sketch.  The sketch must be the linear map G A with G of the
requested scale.
"""
import numpy as np
import pytest
import scipy.linalg as sla

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle(rbrp_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    h = Handle(0)
    yield h
    h.close()


def decaying(m, n, seed, rate=40.0):
    rng = np.random.default_rng(seed)
    U = np.linalg.qr(rng.standard_normal((m, min(m, n))))[0]
    V = np.linalg.qr(rng.standard_normal((n, min(m, n))))[0]
    s = np.exp(-np.arange(min(m, n)) / rate)
    return (U * s) @ V.T


def test_sketch_is_linear_map_with_scale(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import gaussian_sketch
    m, l = 700, 96
    rng = np.random.default_rng(0)
    B = rng.standard_normal((m, 150)).astype(np.float32)
    A = np.concatenate([np.eye(m, dtype=np.float32), B], axis=1)
    At = torch.from_numpy(A).cuda()
    Y = gaussian_sketch(At, l, seed=5, scale=0.5, handle=handle).double().cpu().numpy()
    G = Y[:, :m]
    assert abs(G.mean()) < 0.02 and abs(G.std() - 0.5) < 0.02
    np.testing.assert_allclose(Y[:, m:], G @ B, rtol=0, atol=1e-4 * np.abs(G @ B).max())
    Y2 = gaussian_sketch(At, l, seed=5, scale=0.5, handle=handle).double().cpu().numpy()
    assert np.array_equal(Y, Y2)
    Y3 = gaussian_sketch(At, l, seed=6, scale=0.5, handle=handle).double().cpu().numpy()
    assert not np.array_equal(Y, Y3)


def test_tensor_core_sketch_matches_cuda_core_and_fp64(handle):
    """A with a 16-byte leading dimension takes the tcgen05 3xTF32 GEMM, any other the CUDA-core one: on the same
    seed both equal the FP64 product G B to FP32 accuracy (G read back through an identity block)."""
    from robust_blockwise_random_pivoting_gb300.sketch_ids import gaussian_sketch
    m, l, nb = 1500, 200, 700          # several tiles in every dimension, partial last tiles
    rng = np.random.default_rng(7)
    B = rng.standard_normal((m, nb)).astype(np.float32)
    A = np.concatenate([np.eye(m, dtype=np.float32), B], axis=1)
    n = A.shape[1]
    At = torch.from_numpy(A).cuda().t().contiguous().t()             # ld m = 1500: tensor cores
    Au = torch.zeros((n, m + 1), dtype=torch.float32, device="cuda").t()[:m, :]
    Au.copy_(At)                                                      # ld 1501: CUDA cores
    Yt = gaussian_sketch(At, l, seed=9, handle=handle).double().cpu().numpy()
    Yu = gaussian_sketch(Au, l, seed=9, handle=handle).double().cpu().numpy()
    G = Yu[:, :m]                      # FP32 FMA against the identity is exact
    ref = G @ B.astype(np.float64)
    tol = 2e-5 * np.abs(ref).max()
    np.testing.assert_allclose(Yu[:, m:], ref, rtol=0, atol=tol)
    np.testing.assert_allclose(Yt[:, m:], ref, rtol=0, atol=tol)
    np.testing.assert_allclose(Yt[:, :m], G, rtol=0, atol=1e-6 * np.abs(G).max())
    assert np.array_equal(Yt, gaussian_sketch(At, l, seed=9, handle=handle).double().cpu().numpy())


def test_cpqr_id_matches_lapack_pivots(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import cpqr_id
    A = decaying(300, 220, seed=1)
    k = 60
    sk, rd, T = cpqr_id(torch.from_numpy(A).cuda(), k, handle=handle)
    _, R, piv = sla.qr(A, mode="economic", pivoting=True)
    assert np.array_equal(sk.cpu().numpy(), piv[:k])
    # T columns follow rd (the library's remaining order); LAPACK's R12 follows piv[k:]
    Tref = sla.solve_triangular(R[:k, :k], R[:k, k:])
    order = {c: j for j, c in enumerate(piv[k:])}
    cols = np.array([order[c] for c in rd.cpu().numpy()])
    np.testing.assert_allclose(T.cpu().numpy(), Tref[:, cols], rtol=0, atol=1e-8 * np.abs(Tref).max())


def test_rand_cpqr_os_matches_numpy_on_same_sketch(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import gaussian_sketch, rand_cpqr_os
    A = decaying(500, 400, seed=2, rate=25.0)
    At = torch.from_numpy(A).cuda()
    r = 40
    sk, rd, T = rand_cpqr_os(At, r, seed=9, handle=handle)
    Y = gaussian_sketch(At, 2 * r, seed=9, handle=handle).double().cpu().numpy()
    _, _, piv = sla.qr(Y[:r], mode="economic", pivoting=True)
    assert np.array_equal(sk.cpu().numpy(), piv[:r])
    S, R_ = sk.cpu().numpy(), rd.cpu().numpy()
    Tref = np.linalg.lstsq(Y[:, S], Y[:, R_], rcond=None)[0]
    np.testing.assert_allclose(T.cpu().numpy(), Tref, rtol=0, atol=1e-7 * np.abs(Tref).max())
    # the sketched ID is a good ID of A itself
    err = np.linalg.norm(A[:, R_] - A[:, S] @ T.cpu().numpy()) / np.linalg.norm(A)
    s = np.linalg.svd(A, compute_uv=False)
    opt = np.sqrt((s[r:] ** 2).sum() / (s ** 2).sum())
    assert err < 30 * opt, (err, opt)


def test_interpolation_sid_and_fsid(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import interpolation
    A = decaying(400, 300, seed=3, rate=30.0)
    At = torch.from_numpy(A).cuda()
    r = handle.column_id(At, b=16, tol=1e-8, seed=0)
    k, perm = r.k, r.perm
    p = perm.cpu().numpy()
    T_sid = interpolation(At, perm, k, mode="sid", handle=handle).cpu().numpy()
    Tref = np.linalg.lstsq(A[:, p[:k]], A[:, p[k:]], rcond=None)[0]
    np.testing.assert_allclose(T_sid, Tref, rtol=0, atol=1e-7 * np.abs(Tref).max())
    T_f = interpolation(At, perm, k, mode="fsid", oversampling=2.0, seed=4, handle=handle).cpu().numpy()
    e_sid = np.linalg.norm(A[:, p[k:]] - A[:, p[:k]] @ T_sid)
    e_f = np.linalg.norm(A[:, p[k:]] - A[:, p[:k]] @ T_f)
    assert e_f < 10 * e_sid, (e_f, e_sid)


def test_workspaces_survive_growth_of_other_buffers(rbrp_lib):
    """A fixed-skeleton run that grows the skeleton-order buffer leaves the sketch workspace intact."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    from robust_blockwise_random_pivoting_gb300.sketch_ids import fixed_skeleton, gaussian_sketch
    h = Handle(0)
    try:
        A = torch.from_numpy(decaying(120, 90, seed=5)).cuda()
        Y1 = gaussian_sketch(A, 32, seed=1, handle=h).cpu()
        W = torch.from_numpy(decaying(150, 400, seed=6)).cuda()   # wider than any earlier run
        fixed_skeleton(h, W, torch.arange(0, 400, 10, dtype=torch.int32), b=16)
        Y2 = gaussian_sketch(A, 32, seed=1, handle=h).cpu()
        assert torch.equal(Y1, Y2)
    finally:
        h.close()


def _lapack_lupp(W):
    """Column permutation of W (k x n) from scipy's dgetrf on W^T, applied as sequential swaps."""
    k, n = W.shape
    _, piv = sla.lu_factor(W.T, check_finite=False)
    P = np.arange(n)
    for j in range(k):
        P[[j, piv[j]]] = P[[piv[j], j]]
    return P, piv + 1


@pytest.mark.parametrize("k,n", [(1, 1), (1, 37), (7, 7), (48, 700), (130, 3000)])
def test_lupp_pivots_match_lapack(handle, k, n):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import lupp_pivots
    rng = np.random.default_rng(k * 1000 + n)
    W = rng.standard_normal((k, n))
    perm, ipiv = lupp_pivots(torch.from_numpy(W).cuda(), handle=handle, return_ipiv=True)
    P, piv = _lapack_lupp(W)
    assert np.array_equal(perm.cpu().numpy(), P)
    assert np.array_equal(ipiv.cpu().numpy(), piv)


def test_lupp_ties_go_to_the_first_position(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import lupp_pivots
    rng = np.random.default_rng(11)
    W = np.round(rng.standard_normal((6, 90)) * 2)   # small integers: many exact ties in |value|
    W[0, 3] = W[0, 7] = -9.0                          # first step: columns 3 and 7 tie; LAPACK takes 3
    W[0, 40] = 9.0
    perm = lupp_pivots(torch.from_numpy(W).cuda(), handle=handle).cpu().numpy()
    P, _ = _lapack_lupp(W)
    assert perm[0] == 3
    assert np.array_equal(perm, P)


def test_lupp_errors(handle):
    from robust_blockwise_random_pivoting_gb300._lib import RBRPError
    from robust_blockwise_random_pivoting_gb300.sketch_ids import lupp_pivots
    rng = np.random.default_rng(2)
    W = rng.standard_normal((5, 50))
    Wz = W.copy()
    Wz[4] = 0.0                      # rank 4 < k = 5: step 5 meets an exact zero pivot (dgetrf info = 5)
    with pytest.raises(RBRPError, match="zero pivot"):
        lupp_pivots(torch.from_numpy(Wz).cuda(), handle=handle)
    Wn = W.copy()
    Wn[1, 20] = np.nan
    with pytest.raises(RBRPError, match="non-finite"):
        lupp_pivots(torch.from_numpy(Wn).cuda(), handle=handle)
    with pytest.raises(RBRPError):
        lupp_pivots(torch.from_numpy(W[:, :2].copy()).cuda(), handle=handle)   # k = 5 > n = 2
    # the handle stays usable
    perm = lupp_pivots(torch.from_numpy(W).cuda(), handle=handle).cpu().numpy()
    assert np.array_equal(perm, _lapack_lupp(W)[0])


def test_rand_lupp_os_matches_numpy_on_same_sketch(handle):
    from robust_blockwise_random_pivoting_gb300.sketch_ids import gaussian_sketch, rand_lupp_os
    A = decaying(500, 400, seed=7, rate=25.0)
    At = torch.from_numpy(A).cuda()
    k = 40
    sk, rd, T = rand_lupp_os(At, k, seed=3, handle=handle)
    Y = gaussian_sketch(At, 2 * k, seed=3, handle=handle).double().cpu().numpy()
    P, _ = _lapack_lupp(Y[:k])
    assert np.array_equal(sk.cpu().numpy(), P[:k])
    assert np.array_equal(rd.cpu().numpy(), P[k:])
    S, R_ = sk.cpu().numpy(), rd.cpu().numpy()
    Tref = np.linalg.lstsq(Y[:, S], Y[:, R_], rcond=None)[0]
    np.testing.assert_allclose(T.cpu().numpy(), Tref, rtol=0, atol=1e-7 * np.abs(Tref).max())
    err = np.linalg.norm(A[:, R_] - A[:, S] @ T.cpu().numpy()) / np.linalg.norm(A)
    s = np.linalg.svd(A, compute_uv=False)
    opt = np.sqrt((s[k:] ** 2).sum() / (s ** 2).sum())
    assert err < 30 * opt, (err, opt)


class _DeviceArray:
    """A raw device pointer seen by torch (``__cuda_array_interface__``)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3}


def test_c_abi_comparison_ids_equal_the_python_ones(handle, rbrp_lib):
    """rbrp_RandLUPP_OS / rbrp_RandCPQR_OS / rbrp_CPQR (the gpu/rid.hpp and gpu/id_cpqr.hpp
    signatures) return what the Python comparison IDs return on the same sketch seed."""
    import ctypes
    from robust_blockwise_random_pivoting_gb300.sketch_ids import rand_cpqr_os, rand_lupp_os
    m, n, k, seed = 300, 250, 30, 5
    A = decaying(m, n, seed=12, rate=20.0)
    At = torch.from_numpy(A).cuda().t().contiguous().t()
    lib = rbrp_lib
    dA = ctypes.c_void_p(At.data_ptr())
    sk, rd, T, fl = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_double()
    assert lib.rbrp_RandLUPP_OS(dA, m, n, k, ctypes.byref(sk), ctypes.byref(rd), ctypes.byref(T), ctypes.byref(fl),
                                seed) == 0
    try:
        sk_t = torch.as_tensor(_DeviceArray(sk.value, (k,), "<i4"), device="cuda").clone()
        rd_t = torch.as_tensor(_DeviceArray(rd.value, (n - k,), "<i4"), device="cuda").clone()
        T_t = torch.as_tensor(_DeviceArray(T.value, (n - k, k), "<f8"), device="cuda").t().clone()
    finally:
        for p in (sk, rd, T):
            lib.rbrp_free(p)
    S_py, rd_py, T_py = rand_lupp_os(At, k, seed=seed, handle=handle)
    assert torch.equal(sk_t, S_py) and torch.equal(rd_t, rd_py)
    assert torch.equal(T_t, T_py)
    assert fl.value > 0

    h_sk = (ctypes.c_int * k)()
    h_rd = (ctypes.c_int * (n - k))()
    T = ctypes.c_void_p()
    assert lib.rbrp_RandCPQR_OS(dA, m, n, k, h_sk, h_rd, ctypes.byref(T), ctypes.byref(fl), seed) == 0
    try:
        T_c = torch.as_tensor(_DeviceArray(T.value, (n - k, k), "<f8"), device="cuda").t().clone()
    finally:
        lib.rbrp_free(T)
    S_py, rd_py, T_py = rand_cpqr_os(At, k, seed=seed, handle=handle)
    assert list(h_sk) == S_py.cpu().tolist() and list(h_rd) == rd_py.cpu().tolist()
    assert torch.equal(T_c, T_py)

    ranks = (ctypes.c_int * 3)(5, 20, 40)
    err, tr = (ctypes.c_double * 3)(), (ctypes.c_double * 3)()
    tc, fl2 = ctypes.c_double(), ctypes.c_double()
    assert lib.rbrp_CPQR(m, n, dA, ranks, 3, err, tr, ctypes.byref(tc), ctypes.byref(fl2)) == 0
    r = handle.column_id(At, b=1, tol=None, kmax=40, sampler="greedy", compute_T=False)
    for q, kq in enumerate((5, 20, 40)):
        np.testing.assert_allclose(err[q], r.residuals[kq - 1], rtol=1e-12)
    assert err[0] > err[1] > err[2] > 0 and tr[0] <= tr[1] <= tr[2] <= tc.value
