"""GPU: parity of the sm_103a RBRP path (through the C ABI) with the CPU oracle.

Tolerances: skeleton indices, ranks, the permutation and the number of
uniforms consumed are compared bit for bit; squared residual estimates to
rtol 1e-6 + atol 1e-14 (the FP64 downdate carries ~1e-16 absolute noise per
block); squared relative ID errors to within 1.05x of the oracle's (the
acceptance bound) plus an absolute floor of 1e-20: T = R11^{-1} R12 of the
RBRP factor (matlab/driver.m:86) bottoms out near 1e-10 un-squared where the
least-squares interpolation of the oracle (python/RBRP.ipynb cell 7) reaches
1e-15, which only shows at exact rank or full rank.  T itself is compared
through the reconstruction A(:, S) T to 1e-8 relative on well-conditioned runs.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import error_at_rank, id_error, interp_sid, rbrp_column_id  # noqa: E402
from robust_blockwise_random_pivoting_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
ERR_FLOOR = 1e-20


@pytest.fixture(scope="module")
def handle(rbrp_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    h = Handle(0)
    yield h
    h.close()


def dev(A, dtype=torch.float64):
    return torch.from_numpy(np.asfortranarray(A)).to(dtype).cuda().t().contiguous().t()


def check_against_oracle(h, A, b, tol, sampler="np", mode="rp", seed=0, kmax=None, exact_T=True,
                         check_draws=True):
    o = rbrp_column_id(A, b, tol=tol, seed=seed, sampler=sampler, mode=mode, kmax=kmax)
    r = h.column_id(dev(A), b=b, tol=tol, seed=seed, sampler="greedy" if mode == "gp" else sampler, kmax=kmax)
    perm = r.perm.cpu().numpy()
    assert r.k == o["k"]
    assert np.array_equal(r.ranks, o["ranks"])
    assert np.array_equal(perm[: r.k], o["perm"][: o["k"]])
    assert np.array_equal(perm, o["perm"])
    np.testing.assert_allclose(r.residuals, o["residuals"], rtol=1e-6, atol=1e-14)
    if sampler == "np" and mode == "rp" and check_draws:
        assert r.draws == o["draws"]
    k = r.k
    if 0 < k < A.shape[1]:
        T = r.T.cpu().numpy()
        e_gpu = id_error(A, perm, T)
        To = interp_sid(A, o["perm"], k)
        e_ref = id_error(A, o["perm"], To)
        assert e_gpu <= 1.05 * e_ref + ERR_FLOOR, (e_gpu, e_ref)
        if exact_T and e_ref > 1e-16:
            S = o["perm"][:k]
            rec, rec_o = A[:, S] @ T, A[:, S] @ To
            assert np.linalg.norm(rec - rec_o) <= 1e-8 * np.linalg.norm(rec_o) + 1e-12
        e_dev = h.id_error(dev(A))
        np.testing.assert_allclose(e_dev, e_gpu, rtol=1e-6, atol=1e-26)
    return r, o


def _notebook_T_from_L(L, perm, k):
    """The interpolation matrix the notebook derives from L (T^T = L_rd L_S^{-1})."""
    LS, Lrd = L[perm[:k]], L[perm[k:]]
    return np.linalg.solve(LS.T, Lrd.T)


@pytest.mark.parametrize("fp32", [False, True])
def test_notebook_L_matches_oracle(handle, fp32):
    """Handle.L() / blocked_rpid(return_L=True) is the notebook's L = A^T Q: equal to the oracle's
    column by column up to each basis vector's sign (FP64 form to 1e-8 of |L|, the mixed form to
    1e-5) over the positions where the two runs pick the same columns, zero where a column was
    chosen before the basis vector, and the notebook's T from it is the library's T.  The squared
    tolerance 1e-6 keeps the skeleton's condition number near 1e3: deeper, the notebook's single
    Gram-Schmidt pass loses orthogonality at ~eps cond^2 and the two bases part by more than
    rounding (1e-4 of a column at k = 165 here), with the same T."""
    from robust_blockwise_random_pivoting_gb300.rbrp import blocked_rpid
    A = W.gaussian_exp(300, 420, decay=12.0, seed=5)
    b, tol = 24, 1e-6
    o = rbrp_column_id(A.astype(np.float32).astype(np.float64) if fp32 else A, b, tol=tol, seed=0)
    X = dev(A, torch.float32 if fp32 else torch.float64).t()
    row_perm, L, _, _, ranks = blocked_rpid(X, 300, b=b, tol=tol, seed=0, handle=handle, return_L=True)
    k = int(ranks[-1])
    L = L.cpu().numpy()
    assert L.shape == (420, k)
    if not fp32:
        assert k == o["k"] and np.array_equal(row_perm, o["perm"])
    kk = min(k, o["k"])
    diff = np.nonzero(row_perm[:kk] != o["perm"][:kk])[0]
    same = int(diff[0]) if diff.size else kk
    assert same >= 10
    Lo = o["L"][:, :same]
    sign = np.sign(np.sum(L[:, :same] * Lo, axis=0))
    np.testing.assert_allclose(L[:, :same] * sign, Lo, rtol=0, atol=(1e-5 if fp32 else 1e-8) * np.abs(Lo).max())
    for a in range(k):  # columns chosen before basis vector a are exactly zero
        assert np.all(L[row_perm[:a], a] == 0.0)
    T = handle.T().cpu().numpy()
    Tn = _notebook_T_from_L(L, row_perm, k)
    np.testing.assert_allclose(Tn, T, rtol=0, atol=(1e-4 if fp32 else 1e-8) * max(1.0, np.abs(T).max()))


def test_gexp1000_skeleton_bit_exact(handle):
    """The 1000 x 1000 FP64 workload, b = 40, squared tol 1e-12, Philox seed 0."""
    A = W.gaussian_exp()
    r, o = check_against_oracle(handle, A, 40, 1e-12)
    assert r.k == 310


@pytest.mark.parametrize("m,n,b,decay", [(300, 200, 16, 8.0), (129, 257, 7, 6.0), (90, 333, 64, 10.0),
                                         (513, 65, 33, 5.0), (64, 64, 64, 3.0)])
def test_ragged_shapes(handle, m, n, b, decay):
    A = W.gaussian_exp(m, n, decay=decay, seed=m + n)
    check_against_oracle(handle, A, b, 1e-10)


@pytest.mark.parametrize("sampler", ["es", "np"])
def test_samplers(handle, sampler):
    A = W.snn(160, 240, r=80, r1=10, density=0.1, seed=5)
    check_against_oracle(handle, A, 12, 1e-12, sampler=sampler, seed=3)


def test_greedy_mode(handle):
    A = W.gaussian_exp(200, 300, decay=7.0, seed=2)
    check_against_oracle(handle, A, 20, 1e-10, mode="gp")


def test_gmm_small(handle):
    """Imbalanced mixture (cluster sizes down to one point): every cluster is in S."""
    A, labels = W.gmm(256, 4000, nclusters=12, seed=2)
    r, o = check_against_oracle(handle, A, 32, 1e-4)
    S = r.perm[: r.k].cpu().numpy()
    assert len(set(labels[S].tolist())) == 12


def test_np_sampler_long_chunks_and_repeat_draws(handle):
    """n = 20000 (20 positions per sampler thread) with 30 dominant columns, so draws
    repeat and the rejection rounds recompute the chunks that lost an index."""
    A = W.gaussian_exp(100, 20000, decay=8.0, seed=21)
    heavy = np.random.default_rng(21).choice(20000, size=30, replace=False)
    A[:, heavy] *= 50.0
    r, o = check_against_oracle(handle, A, 32, 1e-10)
    assert o["draws"] > r.k   # some draws were rejected as repeats


def test_run_to_full_rank_and_kmax(handle):
    A = W.gaussian_exp(120, 150, decay=30.0, seed=4)
    check_against_oracle(handle, A, 16, None)
    check_against_oracle(handle, A, 16, None, kmax=37)


def test_zero_and_duplicate_columns(handle):
    rng = np.random.default_rng(0)
    B = rng.standard_normal((70, 12))
    A = np.asfortranarray(np.concatenate([np.zeros((70, 5)), B, B, np.zeros((70, 3)), B], axis=1))
    # exact duplicates leave residual weights that are 0 in one arithmetic and
    # 1e-30 in the other, so only the uniform count may differ
    r, o = check_against_oracle(handle, A, 16, 1e-13, check_draws=False)
    assert r.k == 12
    S = r.perm[: r.k].cpu().numpy()
    assert all(5 <= s for s in S)


def test_exact_rank(handle):
    rng = np.random.default_rng(1)
    A = np.asfortranarray(rng.standard_normal((100, 6)) @ rng.standard_normal((6, 140)))
    r, _ = check_against_oracle(handle, A, 16, 1e-13)
    assert r.k == 6


def test_zero_matrix_and_tiny_shapes(handle):
    r = handle.column_id(dev(np.zeros((30, 20))), b=8, tol=1e-12)
    assert r.k == 0 and r.nblocks == 0
    check_against_oracle(handle, np.ones((1, 5)), 4, 1e-12)
    check_against_oracle(handle, np.arange(1.0, 8.0).reshape(7, 1), 4, 1e-12)


# FP32 resolution of an ID computed from FP32 data (u = 2^-24): squared errors of the
# mixed form are compared as e <= 1.05^2 e_ref + (4u)^2; where the oracle's error at
# that rank is below (4u)^2 (exact or full rank) the rank must match and e <= tol
FP32_FLOOR_SQ = (4 * 2.0 ** -24) ** 2


def _mixed_vs_fp64(handle, A, b, tol, kslack):
    """FP32 residual-form run against the FP64 oracle on the same (FP32-rounded)
    matrix: the relative Frobenius error within 1.05x of the oracle's at the
    GPU's rank (``oracle.error_at_rank``), the first block's columns equal."""
    A32 = A.astype(np.float32).astype(np.float64)
    o = rbrp_column_id(A32, b, tol=tol, seed=0)
    r = handle.column_id(dev(A, torch.float32), b=b, tol=tol, seed=0)
    perm = r.perm.cpu().numpy()
    assert sorted(perm.tolist()) == list(range(A.shape[1]))
    e_gpu = id_error(A32, perm, r.T.cpu().numpy())
    e_same, how = error_at_rank(A32, r.k, b, tol=tol, seed=0, run=o)
    if e_same <= FP32_FLOOR_SQ:
        # exact (or full) rank in FP32 terms: the oracle's error is 0 to FP32 resolution and
        # the GPU's is set by the FP32 data of T; the same rank and the tolerance must hold
        assert r.k == o["k"] and e_gpu <= max(tol, FP32_FLOOR_SQ), (e_gpu, r.k, o["k"])
    else:
        assert e_gpu <= 1.05 ** 2 * e_same + FP32_FLOOR_SQ, (e_gpu, e_same, how, r.k, o["k"])
    assert r.err_est <= tol and abs(r.k - o["k"]) <= kslack, (r.k, o["k"])
    k1 = int(o["ranks"][0])
    assert np.array_equal(perm[:k1], o["perm"][:k1])
    np.testing.assert_allclose(handle.id_error(dev(A, torch.float32)), e_gpu, rtol=1e-4)
    return r, o


def test_fp32_mixed_error_bound(handle):
    _mixed_vs_fp64(handle, W.gaussian_exp(400, 400, decay=12.0, seed=9), 32, 1e-8, 32)


def test_fp32_mixed_snn(handle):
    A = W.snn(700, 900, r=400, r1=40, density=0.05, seed=11)
    r, o = _mixed_vs_fp64(handle, A, 64, 1e-12, 64)
    assert r.k <= 400


def test_fp32_mixed_gmm_clusters(handle):
    A, labels = W.gmm(256, 4000, nclusters=12, seed=2)
    r, o = _mixed_vs_fp64(handle, A, 32, 1e-4, 64)
    assert len(set(labels[r.perm[: r.k].cpu().numpy()].tolist())) == 12


def test_gmm65k_full_size_coverage_matches_oracle(handle):
    """The full imbalanced-mixture workload (1024 x 65536, 20 clusters of 2^-c weight,
    b = 32, squared tol 1e-4) on its FP32 values.  The oracle itself covers 17 of
    the 20 clusters at k = 1023: the five last clusters are single points, each
    drawn with ~2e-4 of the weight per draw, and at rank 1023 of 1024 the span
    already holds them.  The FP64 form reproduces the oracle's skeleton bit for
    bit (so its coverage too); the mixed form covers as many clusters and meets
    the same-rank error bound."""
    A, labels = W.gmm(1024, 65536, 20, 0)
    A32 = A.astype(np.float32).astype(np.float64)
    o = rbrp_column_id(A32, 32, tol=1e-4, seed=0)
    cover = lambda S: len(set(labels[S].tolist()))
    r = handle.column_id(dev(A32), b=32, tol=1e-4, seed=0)
    assert r.k == o["k"] and np.array_equal(r.ranks, o["ranks"])
    assert np.array_equal(r.perm.cpu().numpy()[: r.k], o["perm"][: o["k"]])
    assert cover(o["perm"][: o["k"]]) == 17
    rm = handle.column_id(dev(A, torch.float32), b=32, tol=1e-4, seed=0)
    pm = rm.perm.cpu().numpy()
    assert cover(pm[: rm.k]) == cover(o["perm"][: o["k"]])
    e_gpu = handle.id_error(dev(A, torch.float32))
    e_same, how = error_at_rank(A32, rm.k, 32, tol=1e-4, seed=0, run=o)
    assert e_gpu <= 1.05 ** 2 * e_same + FP32_FLOOR_SQ, (e_gpu, e_same, how, rm.k, o["k"])


def test_tensor_core_projection_matches_cuda_core(handle):
    """The tcgen05 projection (3xTF32) against the CUDA-core one on the same FP32 matrix.

    The tensor core rounds its FP32 accumulator once per MMA with a bias, so W
    carries ~1e-6 relative error where the double-float CUDA-core sums carry
    ~1e-8; both runs must meet the tolerance and stay within a block of ranks.
    """
    tol = 1e-12
    A = W.snn(1200, 1500, r=300, r1=30, density=0.05, seed=13)
    A32 = dev(A, torch.float32)
    A32h = A.astype(np.float32).astype(np.float64)
    o = rbrp_column_id(A32h, 64, tol=tol, seed=0)
    runs = {}
    for variant in (1, 0):
        handle.set_variant(variant)
        try:
            r = handle.column_id(A32, b=64, tol=tol, seed=0)
        finally:
            handle.set_variant(0)
        runs[variant] = (r, handle.id_error(A32))
    for variant, (r, e) in runs.items():
        e_same, how = error_at_rank(A32h, r.k, 64, tol=tol, seed=0, run=o)
        if e_same <= FP32_FLOOR_SQ:   # past the exact rank (300): the oracle's error is FP32 noise
            assert r.err_est <= tol and e <= max(tol, FP32_FLOOR_SQ), (variant, r.k, e, e_same, how)
        else:
            assert r.err_est <= tol and e <= 1.05 ** 2 * e_same + FP32_FLOOR_SQ, (variant, r.k, e, e_same, how)
        assert abs(r.k - o["k"]) <= 64, (variant, r.k, o["k"])
    assert abs(runs[0][0].k - runs[1][0].k) <= 64
    # the first block (before any accumulated difference) selects the same columns
    k1 = int(runs[0][0].ranks[0])
    assert np.array_equal(runs[0][0].perm.cpu().numpy()[:k1], runs[1][0].perm.cpu().numpy()[:k1])


@pytest.mark.parametrize("n", [900, 6400, 8400])
def test_double_float_T_solve_matches_fp64(handle, n):
    """T = R11^{-1} R12 with double-float block updates against the FP64-pipe solve, for
    about 600, 6100 and 8100 columns of T (several 64-row blocks each)."""
    A = dev(W.gaussian_exp(500, n, decay=15.0, seed=17))
    Ts = []
    for fp64 in (True, False):
        handle.set_tsolve_fp64(fp64)
        try:
            r = handle.column_id(A, b=48, tol=1e-12, seed=0)
        finally:
            handle.set_tsolve_fp64(False)
        Ts.append(r.T.cpu().numpy())
    assert Ts[0].shape == Ts[1].shape and Ts[0].shape[0] > 64
    np.testing.assert_allclose(Ts[1], Ts[0], rtol=0, atol=1e-9 * np.abs(Ts[0]).max())


def test_invalid_inputs_rejected(handle):
    from robust_blockwise_random_pivoting_gb300._lib import RBRPError
    A = dev(W.gaussian_exp(50, 60, seed=1))
    with pytest.raises(RBRPError):
        handle.column_id(A, b=65)
    with pytest.raises(RBRPError):
        handle.column_id(A, b=0)
    bad = A.clone()
    bad[3, 7] = float("nan")
    with pytest.raises(RBRPError) as ei:
        handle.column_id(bad, b=8)
    assert ei.value.status == 5
    # the handle stays usable after errors
    check_against_oracle(handle, W.gaussian_exp(50, 60, seed=1), 8, 1e-10)


def test_host_buffer_entry_point(handle):
    A = W.gaussian_exp(200, 180, decay=9.0, seed=6)
    o = rbrp_column_id(A, 24, tol=1e-11, seed=0)
    k, perm, T, res = handle.column_id_host(A, b=24, tol=1e-11, seed=0)
    assert k == o["k"] and np.array_equal(perm, o["perm"])
    To = interp_sid(A, o["perm"], k)
    assert id_error(A, perm, np.ascontiguousarray(T)) <= 1.05 * id_error(A, o["perm"], To) + ERR_FLOOR


def test_dropin_RBRP_and_rand_adap(rbrp_lib, handle):
    from robust_blockwise_random_pivoting_gb300.rbrp import RBRP, rand_adap_rbrp
    A = W.gaussian_exp(150, 170, decay=10.0, seed=7)
    ranks, err, t_ranks, t_total, flops = RBRP(dev(A), 20)
    o = rbrp_column_id(A, 20, tol=None, seed=0)
    assert np.array_equal(ranks, o["ranks"])
    np.testing.assert_allclose(err, o["residuals"], rtol=1e-6, atol=1e-14)
    assert t_total > 0 and flops > 0 and np.all(np.diff(t_ranks) >= 0)
    sk, rd, T, k, flops = rand_adap_rbrp(dev(A), tol=1e-10, blk=20)
    o = rbrp_column_id(A, 20, tol=1e-10, seed=0)
    assert k == o["k"]
    assert np.array_equal(sk.cpu().numpy(), o["perm"][:k]) and np.array_equal(rd.cpu().numpy(), o["perm"][k:])
    perm = np.concatenate([sk.cpu().numpy(), rd.cpu().numpy()])
    assert id_error(A, perm, T.cpu().numpy()) <= 1.05 * id_error(A, o["perm"], interp_sid(A, o["perm"], k)) + ERR_FLOOR


def test_golden_oracle_fixture_cfg0(handle, golden_dir):
    """The committed oracle output for the 1000 x 1000 workload matches the GPU."""
    import os
    g = np.load(os.path.join(golden_dir, "oracle_gexp1000_philox0.npz"))
    r = handle.column_id(dev(W.gaussian_exp()), b=40, tol=1e-12, seed=0)
    assert r.k == int(g["k"])
    assert np.array_equal(r.perm.cpu().numpy(), g["perm"])
    assert r.draws == int(g["draws"])
