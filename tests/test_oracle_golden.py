"""CPU: the oracle against the reference's own outputs (golden fixtures)."""
import os

import numpy as np
import pytest

from oracle import (PhiloxStream, corrected_swap, es_topb, id_error, interp_r11,
                    interp_sid, local_clip, np_compat_choice, philox4x64_10,
                    rbrp_column_id)
from oracle.philox import es_uniforms, u64_to_unit


def _load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def test_philox_matches_numpy_bit_generator():
    for seed in (0, 1, 2**40 + 3):
        raw = np.random.Philox(key=seed).random_raw(37)
        mine = [philox4x64_10([1 + t // 4, 0, 0, 0], [seed, 0])[t % 4] for t in range(37)]
        assert [int(x) for x in raw] == mine
        u = np.random.Generator(np.random.Philox(key=seed)).random(37)
        assert np.array_equal(u, u64_to_unit(raw))


def test_es_stream_counter_layout():
    u = es_uniforms(5, 3, 9)
    for c in range(9):
        raw = philox4x64_10([1 + c // 4, 4, 0x4553, 0], [5, 0])[c % 4]
        assert u[c] == (raw >> 11) * 2.0 ** -53


def test_sampler_restatement_matches_numpy_choice(golden_dir):
    g = _load(golden_dir, "sampler_numpy_choice.npz")
    off_w = np.concatenate([[0], np.cumsum(g["wlen"])])
    off_i = np.concatenate([[0], np.cumsum(g["size"])])
    for c in range(int(g["n"])):
        w = g["w"][off_w[c]:off_w[c + 1]]
        size = int(g["size"][c])
        stream = PhiloxStream(int(g["seed"][c]))
        got = np_compat_choice(w, size, stream.random)
        exp = g["idx"][off_i[c]:off_i[c + 1]]
        assert np.array_equal(got, exp), c
        # same number of uniforms consumed as numpy (counter and buffer position)
        bg = np.random.Philox(key=int(g["seed"][c]))
        bg.random_raw(stream.draws)
        st = bg.state
        assert np.array_equal(np.array(st["state"]["counter"], np.uint64), g["counter"][c])
        assert st["buffer_pos"] == g["buffer_pos"][c]


def test_sampler_live_numpy_choice():
    rng = np.random.default_rng(3)
    for _ in range(50):
        N = int(rng.integers(2, 300))
        w = rng.random(N) ** 4
        size = int(rng.integers(1, min(N, 64) + 1))
        seed = int(rng.integers(0, 2**31))
        exp = np.random.Generator(np.random.Philox(key=seed)).choice(N, size, p=w / sum(w), replace=False)
        got = np_compat_choice(w, size, PhiloxStream(seed).random)
        assert np.array_equal(got, exp)


def test_filter_matches_reference_local_clip(golden_dir):
    g = _load(golden_dir, "filter_local_clip.npz")
    off = 0
    for c, (shape, tol, bs) in enumerate(zip(g["shape"], g["tol"], g["bs"])):
        n = int(shape[0] * shape[1])
        R = g["R"][off:off + n].reshape(shape)
        off += n
        assert local_clip(R, tol) == bs, c


@pytest.mark.parametrize("name", ["gexp", "snn", "gmm", "gexp_b1tol"])
def test_oracle_matches_patched_reference(golden_dir, name):
    g = _load(golden_dir, "blocked_rpid_patched.npz")
    A = g[f"{name}__A"]
    b = int(g[f"{name}__b"])
    tol = float(g[f"{name}__tol"])
    tol = None if tol < 0 else tol
    r = rbrp_column_id(A, b, tol=tol, rng=np.random.default_rng(42))
    k = r["k"]
    assert np.array_equal(r["ranks"], g[f"{name}__ranks"])
    assert np.array_equal(r["perm"], g[f"{name}__row_perm"])
    np.testing.assert_allclose(r["residuals"], g[f"{name}__residuals"], rtol=1e-8, atol=1e-15)
    np.testing.assert_allclose(r["L"], g[f"{name}__L"][:, :k], rtol=1e-9, atol=1e-11)
    T = interp_sid(A, r["perm"], k)
    np.testing.assert_allclose(T.T, g[f"{name}__W"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(id_error(A, r["perm"], T), float(g[f"{name}__err"]), rtol=1e-6, atol=1e-18)


def test_oracle_with_numpy_choice_is_identical():
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    A = W.gaussian_exp(200, 260, decay=10.0, seed=3)
    a = rbrp_column_id(A, 16, tol=1e-10, seed=9)
    b = rbrp_column_id(A, 16, tol=1e-10, rng=np.random.Generator(np.random.Philox(key=9)),
                       sampler_impl="numpy")
    assert a["k"] == b["k"] and np.array_equal(a["perm"], b["perm"])


def test_unpatched_reference_swap_bug_recorded(golden_dir):
    g = _load(golden_dir, "blocked_rpid_unpatched_gexp1000.npz")
    assert int(g["unique_in_S"]) < int(g["k"])        # duplicates in the skeleton
    assert not bool(g["is_permutation"])


def test_corrected_swap_is_permutation_and_matches_matlab():
    rng = np.random.default_rng(0)
    for _ in range(300):
        n = int(rng.integers(4, 80))
        i = int(rng.integers(0, n - 1))
        bs = int(rng.integers(1, n - i + 1))
        kept = rng.choice(np.arange(i, n), size=bs, replace=False)
        perm = rng.permutation(n)
        old = perm.copy()
        corrected_swap(perm, i, kept)
        assert sorted(perm.tolist()) == list(range(n))
        assert np.array_equal(perm[i:i + bs], old[kept])
        # positions outside the block and outside kept are untouched
        untouched = np.setdiff1d(np.arange(n), np.concatenate([np.arange(i, i + bs), kept]))
        assert np.array_equal(perm[untouched], old[untouched])


def test_es_topb_exact_frequencies():
    """Inclusion frequencies of the exponential-key sampler: chi-square for size 1."""
    w = np.array([1.0, 2.0, 3.0, 4.0, 0.0, 10.0])
    counts = np.zeros(w.size)
    trials = 20000
    for t in range(trials):
        u = es_uniforms(1, t, w.size)
        counts[es_topb(w, 1, u)[0]] += 1
    p = w / w.sum()
    assert counts[4] == 0
    nz = p > 0
    chi2 = (((counts[nz] - trials * p[nz]) ** 2) / (trials * p[nz])).sum()
    assert chi2 < 20.5  # 4 dof, p ~ 4e-4


def test_exact_rank_stop_and_reconstruction():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((90, 7))
    Y = rng.standard_normal((120, 7))
    A = np.asfortranarray(X @ Y.T)
    # the squared-residual downdate has an FP64 floor near 1e-16, so the
    # tolerance sits above it
    r = rbrp_column_id(A, 16, tol=1e-13, seed=4)
    assert r["k"] == 7
    T = interp_sid(A, r["perm"], r["k"])
    assert id_error(A, r["perm"], T) < 1e-24
    T2 = interp_r11(r["R"], r["perm"], r["k"])
    assert id_error(A, r["perm"], T2) < 1e-24


def test_duplicate_columns_cut_by_filter():
    rng = np.random.default_rng(2)
    B = rng.standard_normal((50, 10))
    A = np.asfortranarray(np.concatenate([B, B, B], axis=1))
    r = rbrp_column_id(A, 16, tol=1e-13, seed=1)
    S = r["perm"][: r["k"]]
    assert r["k"] == 10
    assert len(set((S % 10).tolist())) == 10


def test_oracle_fixture_cfg0_reproduces(golden_dir):
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    g = _load(golden_dir, "oracle_gexp1000_philox0.npz")
    r = rbrp_column_id(W.gaussian_exp(), 40, tol=1e-12, seed=0)
    assert r["k"] == int(g["k"]) and r["draws"] == int(g["draws"])
    assert np.array_equal(r["perm"], g["perm"])
