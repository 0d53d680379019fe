"""GPU: the fixed-skeleton ID and its FP32 adjoint against FP64 references.

The FP64 reference computes the same loss with torch in FP64 (T by a QR
least-squares solve) and differentiates it with torch's autograd.  Tolerances:
T against the FP64 least-squares T to 1e-4 relative (FP32 data, double-float
panels and projections; cond(A(:, S)) ~ 1e3); the loss to 1e-4 relative; the gradient with respect to A to 2e-3
relative in the Frobenius norm (FP32 GEMMs over thousands of terms); the
gradient with respect to the kernel lengthscale to 2e-3 relative against the
FP64 gradient on the same FP32-rounded matrix and to 1e-2 against the FP64
gradient on the unrounded matrix, which itself agrees to 1e-3 with central
finite differences (h = 1e-4) of the FP64 loss.
"""
import numpy as np
import pytest

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


def colmajor(A):
    return A.t().contiguous().t()


def ref_loss(A64, S, w64):
    n = A64.shape[1]
    mask = torch.ones(n, dtype=torch.bool, device=A64.device)
    mask[S.long()] = False
    rd = torch.nonzero(mask).flatten()
    C, B = A64[:, S.long()], A64[:, rd]
    Q, R = torch.linalg.qr(C)
    T = torch.linalg.solve_triangular(R, Q.t() @ B, upper=True)
    E = B - C @ T
    return (E * E).sum() + ((T @ w64[rd]) ** 2).sum(), T, rd


def kernel_problem(n=640, dim=4, ls=1.5, seed=0):
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    P = torch.from_numpy(W.gaussian_kernel_points(n, dim, seed)).cuda()
    return P, ls


def skeleton(handle, A32, tol=1e-6, b=64):
    r = handle.column_id(colmajor(A32), b=b, tol=tol, seed=0)
    return r.perm[: r.k].clone()


def test_fixed_skeleton_T_matches_least_squares(handle):
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id
    g = torch.Generator(device="cpu").manual_seed(3)
    A64 = torch.randn(300, 260, generator=g, dtype=torch.float64)
    A64 = (A64 @ torch.diag(torch.exp(-torch.arange(260, dtype=torch.float64) / 60))).cuda()
    A32 = colmajor(A64.float())
    S = torch.randperm(260, generator=g)[:90].to(torch.int32).cuda()
    perm, r = fixed_skeleton_id(handle, A32, S, b=32)
    assert r.k == 90
    p = perm.cpu().numpy()
    assert sorted(p[:90].tolist()) == sorted(S.cpu().numpy().tolist())
    T = handle.T().cpu().numpy()                       # rows perm[:k], columns perm[k:]
    A = A32.double()
    _, Tref, rd = ref_loss(A, torch.from_numpy(p[:90]).cuda(), torch.zeros(260, dtype=torch.float64, device="cuda"))
    # reference T rows follow perm[:k] (same S order), columns follow rd (ascending): reorder ours
    order = np.argsort(p[90:])
    Tn = T[:, order]
    err = np.linalg.norm(Tn - Tref.cpu().numpy()) / np.linalg.norm(Tref.cpu().numpy())
    assert err < 1e-4, err


def test_fixed_skeleton_reproduces_adaptive_T(handle):
    """With the skeleton of an adaptive FP32 run, the fixed run gives the same skeleton and T."""
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id
    from robust_blockwise_random_pivoting_gb300.adjoint import gaussian_kernel_matrix
    P, ls = kernel_problem(512)
    A32 = colmajor(gaussian_kernel_matrix(P, ls).float())
    handle.set_variant(1)  # CUDA-core (double-float) projection, as the fixed-skeleton run uses
    try:
        r = handle.column_id(A32, b=64, tol=1e-6, seed=0)
    finally:
        handle.set_variant(0)
    Sa, Ta = r.perm[: r.k].cpu().numpy(), r.T.cpu().numpy()
    perm, rf = fixed_skeleton_id(handle, A32, r.perm[: r.k], b=64)
    pf = perm.cpu().numpy()
    assert rf.k == r.k and sorted(pf[: r.k].tolist()) == sorted(Sa.tolist())
    Tf = handle.T().cpu().numpy()
    # same rows/columns up to order
    ia = {c: i for i, c in enumerate(Sa)}
    ja = {c: j for j, c in enumerate(r.perm[r.k:].cpu().numpy())}
    Tf_in_a = np.zeros_like(Ta)
    rows = np.array([ia[c] for c in pf[: r.k]])
    cols = np.array([ja[d] for d in pf[r.k:]])
    Tf_in_a[np.ix_(rows, cols)] = Tf
    err = np.linalg.norm(Tf_in_a - Ta) / np.linalg.norm(Ta)
    assert err < 1e-3, err


def test_adjoint_matches_fp64_autograd(handle):
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id_loss, gaussian_kernel_matrix
    P, ls = kernel_problem(640)
    A32 = colmajor(gaussian_kernel_matrix(P, ls).float())
    S = skeleton(handle, A32)
    k = S.numel()
    assert 60 < k < 400, k
    w = torch.randn(640, generator=torch.Generator(device="cpu").manual_seed(1)).cuda()
    A = A32.clone().requires_grad_(True)
    loss = fixed_skeleton_id_loss(A, S, w, b=64, handle=handle)
    loss.backward()
    A64 = A32.double().requires_grad_(True)
    lref, _, _ = ref_loss(A64, S, w.double())
    lref.backward()
    assert abs(loss.item() - lref.item()) <= 1e-4 * abs(lref.item()), (loss.item(), lref.item())
    G, Gref = A.grad.double(), A64.grad
    rel = (torch.linalg.norm(G - Gref) / torch.linalg.norm(Gref)).item()
    assert rel < 2e-3, rel


def test_lengthscale_gradient_fd_and_fp64(handle):
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id_loss, gaussian_kernel_matrix
    P, ls0 = kernel_problem(512, seed=4)
    A0 = colmajor(gaussian_kernel_matrix(P, ls0).float())
    S = skeleton(handle, A0)
    w = torch.randn(512, generator=torch.Generator(device="cpu").manual_seed(2)).cuda()
    ls = torch.tensor(ls0, dtype=torch.float64, device="cuda", requires_grad=True)
    A = gaussian_kernel_matrix(P, ls).float()
    loss = fixed_skeleton_id_loss(A, S, w, b=64, handle=handle)
    loss.backward()
    g_ours = ls.grad.item()

    def ref(l, rounded):
        A = gaussian_kernel_matrix(P, l)
        return ref_loss(A.float().double() if rounded else A, S, w.double())[0]
    # FP64 gradient on the same FP32-rounded matrix our kernels see
    ls64 = torch.tensor(ls0, dtype=torch.float64, device="cuda", requires_grad=True)
    ref(ls64, True).backward()
    g_ref = ls64.grad.item()
    assert abs(g_ours - g_ref) <= 2e-3 * abs(g_ref), (g_ours, g_ref)
    # the FP64 gradient formula against central differences of the unrounded FP64 loss (rounding A
    # to FP32 at l +- h would add noise above the 2 h g signal)
    lsx = torch.tensor(ls0, dtype=torch.float64, device="cuda", requires_grad=True)
    ref(lsx, False).backward()
    g64 = lsx.grad.item()
    h = 1e-4
    with torch.no_grad():
        g_fd = (ref(torch.tensor(ls0 + h, dtype=torch.float64, device="cuda"), False) -
                ref(torch.tensor(ls0 - h, dtype=torch.float64, device="cuda"), False)).item() / (2 * h)
    assert abs(g64 - g_fd) <= 1e-3 * abs(g64), (g64, g_fd)
    assert abs(g_ours - g64) <= 1e-2 * abs(g64), (g_ours, g64)


def test_backward_reuses_the_forward_factorisation(handle):
    """The backward takes the handle's factorisation from the forward when nothing ran in
    between (no second fixed-skeleton ID), and recomputes it when something did; the gradient
    equals the one computed from scratch bit for bit either way."""
    from robust_blockwise_random_pivoting_gb300.adjoint import (fixed_skeleton_id_loss, fixed_skeleton_loss_and_grad,
                                                                gaussian_kernel_matrix)
    P, ls = kernel_problem(384, seed=7)
    A32 = colmajor(gaussian_kernel_matrix(P, ls).float())
    S = skeleton(handle, A32)
    w = torch.randn(384, generator=torch.Generator(device="cpu").manual_seed(3)).cuda()
    loss_ref, G_ref = fixed_skeleton_loss_and_grad(handle, A32, S, w, b=64, grad=True)
    # reuse: forward, then backward with nothing in between
    A = A32.clone().requires_grad_(True)
    loss = fixed_skeleton_id_loss(A, S, w, b=64, handle=handle)
    e0 = handle.epoch
    loss.backward()
    assert handle.epoch == e0          # no fixed-skeleton ID ran in the backward
    assert loss.item() == loss_ref and torch.equal(A.grad, G_ref)
    # an intervening run on the handle: the backward recomputes
    A2 = A32.clone().requires_grad_(True)
    loss2 = fixed_skeleton_id_loss(A2, S, w, b=64, handle=handle)
    handle.column_id(A32, b=32, tol=1e-6, seed=1)
    e1 = handle.epoch
    loss2.backward()
    assert handle.epoch == e1 + 1      # the backward ran the fixed-skeleton ID again
    assert torch.equal(A2.grad, G_ref)


def test_adjoint_requires_matching_run(handle):
    from robust_blockwise_random_pivoting_gb300._lib import RBRPError
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id
    A = colmajor(torch.randn(50, 40, device="cuda"))
    with pytest.raises(RBRPError):
        fixed_skeleton_id(handle, A, torch.tensor([3, 3], dtype=torch.int32, device="cuda"))
    with pytest.raises(RBRPError):
        fixed_skeleton_id(handle, A, torch.tensor([45], dtype=torch.int32, device="cuda"))


def test_tensor_core_adjoint_matches_ffma(handle):
    """The adjoint GEMMs on the tensor cores (tcgen05 3xTF32, variant 0, default) against
    the FP32 FFMA kernels (variant 1) on the same problem, each against the FP64 autograd
    gradient: the tensor-core loss and gradient no further from FP64 than the FFMA ones
    (1.5x; the variants also differ in the forward's projection, 3xTF32 against CUDA-core
    double-float)."""
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_loss_and_grad, gaussian_kernel_matrix
    P, ls = kernel_problem(n=1500, dim=6, ls=1.2, seed=5)
    A32 = colmajor(gaussian_kernel_matrix(P, ls).float())
    S = skeleton(handle, A32, tol=1e-8)
    w = torch.randn(1500, generator=torch.Generator(device="cpu").manual_seed(2)).cuda()
    A64 = A32.double().requires_grad_(True)
    lref, _, _ = ref_loss(A64, S, w.double())
    lref.backward()
    out = {}
    for variant in (0, 1):
        handle.set_variant(variant)
        try:
            loss, G = fixed_skeleton_loss_and_grad(handle, A32, S, w, b=64)
        finally:
            handle.set_variant(0)
        out[variant] = (abs(loss - lref.item()) / abs(lref.item()),
                        (torch.linalg.norm(G.double() - A64.grad) / torch.linalg.norm(A64.grad)).item())
    # (measured: loss 1.3e-4 / 1.6e-4 and gradient 4.9e-3 / 4.3e-3 relative to FP64, tensor
    # core / FFMA; at squared tol 1e-8 this skeleton is less well conditioned than the others)
    assert out[0][0] <= 1.5 * out[1][0] + 1e-5 and out[0][0] <= 5e-4, out
    assert out[0][1] <= 1.5 * out[1][1] + 1e-4 and out[0][1] <= 1e-2, out
