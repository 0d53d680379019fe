"""GPU: the bounded device-side waits run out cleanly.

The library's kernels that wait on other threads of the GPU - the grid barrier
of the LU pivots (a cooperative launch) and the mbarrier waits of the tcgen05
projection - give up after a clock64 limit, set an error status, let their own
asynchronous copies and MMAs finish, and exit.  The test-only limit of
``rbrp_set_wait_budget`` (a few cycles) makes the waits run out on purpose,
without any fault or hang: the call must return RBRP_ERR_DEVICE_TIMEOUT (7),
and the same handle, with the default limit back, must give exactly the
results of an untouched handle.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from robust_blockwise_random_pivoting_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
DEVICE_TIMEOUT = 7


@pytest.fixture()
def handle(rbrp_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    h = Handle(0)
    yield h
    h.close()


def test_lu_grid_barrier_timeout_is_clean(handle):
    from robust_blockwise_random_pivoting_gb300._lib import RBRPError
    from robust_blockwise_random_pivoting_gb300.sketch_ids import lupp_pivots
    W_ = torch.from_numpy(np.random.default_rng(3).standard_normal((130, 3000))).cuda()
    ref = lupp_pivots(W_, handle=handle).cpu().numpy()
    handle.set_wait_budget(1)
    try:
        with pytest.raises(RBRPError) as e:
            lupp_pivots(W_, handle=handle)
        assert e.value.status == DEVICE_TIMEOUT
    finally:
        handle.set_wait_budget(0)
    torch.cuda.synchronize()   # the context is intact
    assert np.array_equal(lupp_pivots(W_, handle=handle).cpu().numpy(), ref)


def test_tcgen05_projection_timeout_is_clean(handle):
    from robust_blockwise_random_pivoting_gb300._lib import RBRPError
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    A = torch.from_numpy(W.snn(1200, 1500, r=300, r1=30, density=0.05, seed=13)).float().cuda()
    A = A.t().contiguous().t()
    with Handle(0) as fresh:
        want = fresh.column_id(A, b=64, tol=1e-10, seed=0)
        want_perm, want_T = want.perm.cpu().numpy(), want.T.cpu().numpy()
    handle.set_wait_budget(1)
    try:
        with pytest.raises(RBRPError) as e:
            handle.column_id(A, b=64, tol=1e-10, seed=0)
        assert e.value.status == DEVICE_TIMEOUT
    finally:
        handle.set_wait_budget(0)
    torch.cuda.synchronize()
    r = handle.column_id(A, b=64, tol=1e-10, seed=0)
    assert r.k == want.k
    assert np.array_equal(r.perm.cpu().numpy(), want_perm)
    assert np.array_equal(r.T.cpu().numpy(), want_T)
