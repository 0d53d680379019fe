"""GPU: the allocation-free ID-error entry point against the handle's one.

rbrp_id_error_f64_noalloc serves callers that cannot let the library call
cudaMalloc (a host runtime that owns a fixed device pool, a hard memory
budget, work enqueued where an allocation would synchronise).  Its scratch is
a fixed device array inside the library, so it must agree with the handle's
rbrp_id_error_f64 - whose scratch lives in the handle's workspace - on
consecutive calls (the array keeps the previous call's contents), and it must
refuse sizes beyond that array.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from robust_blockwise_random_pivoting_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
RTOL = 1e-10  # only the summation order of the partial sums differs


def _noalloc(lib, A, perm, k, T, normA2, out, stream):
    m, n = A.shape
    return lib.rbrp_id_error_f64_noalloc(m, n, ctypes.c_void_p(A.data_ptr()), A.stride(1),
                                         ctypes.c_void_p(perm.data_ptr()), k, ctypes.c_void_p(T.data_ptr()),
                                         max(1, T.stride(1)), normA2, ctypes.c_void_p(out.data_ptr()),
                                         ctypes.c_void_p(stream.cuda_stream))


def test_noalloc_id_error_matches_handle_entry_point(rbrp_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    stream = torch.cuda.current_stream()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    cases = [W.gaussian_exp(300, 420, decay=10.0, seed=21), W.snn(250, 600, r=120, r1=12, density=0.1, seed=22)]
    with Handle(0) as h:
        for A_np in cases:
            A = torch.from_numpy(A_np).cuda().t().contiguous().t()
            r = h.column_id(A, b=32, tol=1e-10, seed=0)
            e_ref = h.id_error(A)
            assert 0 < r.k < A.shape[1]
            for _ in range(2):   # two calls in a row on the shared scratch array
                out.fill_(-1.0)
                assert _noalloc(rbrp_lib, A, r.perm, r.k, r.T, r.res0, out, stream) == 0
                torch.cuda.synchronize()
                np.testing.assert_allclose(out.item(), e_ref, rtol=RTOL, atol=1e-300)


def test_noalloc_empty_and_full_skeletons(rbrp_lib):
    """k == 0 and k == n are valid IDs: 1.0 and 0.0, as the handle's entry point reports them."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    stream = torch.cuda.current_stream()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    A = torch.from_numpy(W.gaussian_exp(40, 30, decay=3.0, seed=5)).cuda().t().contiguous().t()
    with Handle(0) as h:
        r = h.column_id(A, b=8, tol=0.0, seed=0)          # full rank: k == n
        assert r.k == A.shape[1]
        e_full = h.id_error(A)
    perm = r.perm
    T = torch.zeros((0, 0), dtype=torch.float64, device="cuda")
    for k, want in ((0, 1.0), (A.shape[1], e_full)):
        for _ in range(2):
            out.fill_(-1.0)
            assert _noalloc(rbrp_lib, A, perm, k, T, r.res0, out, stream) == 0
            torch.cuda.synchronize()
            assert out.item() == want, (k, out.item(), want)
    assert e_full == 0.0


def test_noalloc_rejects_sizes_beyond_scratch(rbrp_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    A = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    perm = torch.arange(64, dtype=torch.int32, device="cuda")
    T = torch.zeros((8, 56), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # ceil((n-k)/32) * ceil(m/64) far above 262144: refused before any launch
    rc = rbrp_lib.rbrp_id_error_f64_noalloc(1 << 20, 1 << 20, ctypes.c_void_p(A.data_ptr()), 1 << 20,
                                            ctypes.c_void_p(perm.data_ptr()), 8, ctypes.c_void_p(T.data_ptr()), 8,
                                            1.0, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 6   # RBRP_ERR_CAPACITY
    assert rbrp_lib.rbrp_id_error_f64_noalloc(64, 64, None, 64, None, 8, None, 8, 1.0, None, None) == 1
