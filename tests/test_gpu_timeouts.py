"""GPU: the bounded device-side waits run out cleanly.

The library's kernels that wait on other threads of the GPU - the grid barrier
of the LU pivots (a cooperative launch) and the mbarrier waits of the tcgen05
projection, of the adjoint's tcgen05 GEMMs and of the sketch GEMM - give up after a clock64 limit, set an error status, let their own
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


def test_tcgen05_adjoint_gemm_timeout_is_clean(handle):
    """The adjoint's tensor-core GEMMs (the same bounded pipeline) run out cleanly too."""
    import ctypes
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id, fixed_skeleton_loss_and_grad
    A = torch.from_numpy(W.gaussian_exp(400, 500, decay=20.0, seed=3)).float().cuda().t().contiguous().t()
    S = torch.arange(0, 500, 5, dtype=torch.int32, device="cuda")
    w = torch.randn(500, generator=torch.Generator(device="cpu").manual_seed(1)).cuda()
    loss_ref, G_ref = fixed_skeleton_loss_and_grad(handle, A, S, w, b=32)
    fixed_skeleton_id(handle, A, S, 32)                  # forward with the default budget
    G = torch.empty((500, 400), dtype=torch.float32, device="cuda").t()
    loss = ctypes.c_double()
    handle.set_wait_budget(1)
    try:
        rc = handle.lib.rbrp_fixed_id_adjoint_f32(handle.h, 400, 500, ctypes.c_void_p(A.data_ptr()), 400,
                                                  ctypes.c_void_p(w.data_ptr()), ctypes.c_float(1.0),
                                                  ctypes.c_void_p(G.data_ptr()), 400, ctypes.byref(loss))
        assert rc == DEVICE_TIMEOUT, rc
    finally:
        handle.set_wait_budget(0)
    torch.cuda.synchronize()
    loss2, G2 = fixed_skeleton_loss_and_grad(handle, A, S, w, b=32)
    assert loss2 == loss_ref and torch.equal(G2, G_ref)


def test_tcgen05_sketch_gemm_timeout_is_clean(handle):
    """The sketch's tensor-core GEMM (the same bounded pipeline) runs out cleanly."""
    from robust_blockwise_random_pivoting_gb300._lib import RBRPError
    from robust_blockwise_random_pivoting_gb300.sketch_ids import gaussian_sketch
    A = torch.from_numpy(np.random.default_rng(4).standard_normal((800, 900))).float().cuda().t().contiguous().t()
    want = gaussian_sketch(A, 96, seed=2, handle=handle)
    handle.set_wait_budget(1)
    try:
        with pytest.raises(RBRPError) as e:
            gaussian_sketch(A, 96, seed=2, handle=handle)
        assert e.value.status == DEVICE_TIMEOUT
    finally:
        handle.set_wait_budget(0)
    torch.cuda.synchronize()
    assert torch.equal(gaussian_sketch(A, 96, seed=2, handle=handle), want)
