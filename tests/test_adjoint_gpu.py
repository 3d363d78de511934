"""Hand-written adjoints of the factorisation and the solve (gbllt_dpotrf_adjoint_dev,
gbllt_dpotrs_adjoint_dev) against an FP64 CPU reference gradient and central finite differences.

Tolerances: the GPU adjoint matches the symbolic FP64 reference (numpy, oracle.chol_adjoint_ref)
within 1e-10 relative (Frobenius, lower triangle); directional derivatives match central finite
differences with h = 1e-6 within 1e-6 relative.  The GP objective logdet A + y^T A^{-1} y is wrapped
in a torch.autograd.Function here, in the test harness only, and checked against the closed form
dA = A^{-1} - a a^T, dy = 2 a and against torch.autograd.gradcheck.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _cm(a):  # numpy column-major matrix -> torch tensor whose storage is that column-major layout
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


def _np(t):  # inverse of _cm
    return np.asfortranarray(t.cpu().numpy().T)


def _stream():
    return torch.cuda.current_stream().cuda_stream


def gpu_factor(gbllt, a):
    n = a.shape[0]
    d = _cm(a)
    info = torch.zeros(1, dtype=torch.int64, device="cuda")
    gbllt.potrf_dev(d, n, n, info, "L", _stream())
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    return d


@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 63, 64, 65, 100, 129, 257, 700])
@pytest.mark.parametrize("mixed", [False, True])
def test_chol_adjoint_matches_reference(oracle, gbllt, n, mixed):
    # FP64 adjoint within 1e-10 of the symbolic reference; the mixed-precision adjoint (28-bit panel
    # products) within 1e-6
    a = oracle.gen_gram(n, seed=80 + n)
    dL = gpu_factor(gbllt, a)
    L = np.tril(_np(dL))
    rng = np.random.default_rng(n)
    Lbar = np.tril(rng.standard_normal((n, n)))
    M = _cm(Lbar)
    gbllt.potrf_adjoint_dev(dL, n, n, M, n, _stream(), mixed=mixed)
    torch.cuda.synchronize()
    got = np.tril(_np(M))
    ref = np.tril(oracle.chol_adjoint_ref(L, Lbar))
    assert np.linalg.norm(got - ref) <= (1e-6 if mixed else 1e-10) * np.linalg.norm(ref)


def _f_weights(gbllt, a, W):
    """f(A) = sum W .* chol(A) (W lower) evaluated with the GPU factorisation."""
    return float(np.sum(W * np.tril(_np(gpu_factor(gbllt, a)))))


@pytest.mark.parametrize("n", [40, 130])
def test_chol_adjoint_finite_differences(oracle, gbllt, n):
    a = oracle.gen_gram(n, seed=90 + n)
    rng = np.random.default_rng(7)
    W = np.tril(rng.standard_normal((n, n)))
    dL = gpu_factor(gbllt, a)
    M = _cm(W)
    gbllt.potrf_adjoint_dev(dL, n, n, M, n, _stream())
    torch.cuda.synchronize()
    G = np.tril(_np(M))
    G = G + np.tril(G, -1).T  # full symmetric gradient
    for trial in range(3):
        E = rng.standard_normal((n, n))
        E = np.asfortranarray(E + E.T)
        h = 1e-6
        fd = (_f_weights(gbllt, a + h * E, W) - _f_weights(gbllt, a - h * E, W)) / (2 * h)
        an = float(np.sum(G * E))
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1.0), (fd, an)


def _gp_gradient(gbllt, a, y, mixed):
    """The GP objective's gradient through the hand-written adjoints: (dA lower, symmetric
    convention, as a full symmetric matrix; dy)."""
    n = a.shape[0]
    s = _stream()
    L = gpu_factor(gbllt, a)
    alpha = torch.from_numpy(y.copy()).cuda().reshape(1, n)
    gbllt.potrs_dev(L, n, n, alpha, 1, n, "L", s)
    M = torch.zeros_like(L)
    M.diagonal().copy_(2.0 / torch.diagonal(L))
    gbllt.potrf_adjoint_dev(L, n, n, M, n, s, mixed=mixed)
    bbar = torch.empty_like(alpha)
    yt = torch.from_numpy(y.copy()).cuda().reshape(1, n)
    gbllt.potrs_adjoint_dev(L, n, n, alpha, n, yt, n, bbar, n, 1, M, n, s)
    torch.cuda.synchronize()
    G = np.tril(_np(M))
    return G + np.tril(G, -1).T, (alpha + bbar).cpu().numpy().reshape(n)


@pytest.mark.parametrize("mixed", [False, True])
def test_gp_gradient_full_size_rbf(oracle, gbllt, mixed):
    # the C5 problem size: an RBF kernel matrix of n = 2048 points (lengthscale 0.2, noise 1e-2).  The
    # gradient of logdet A + y^T A^-1 y is A^-1 - a a^T (a = A^-1 y) in the symmetric convention, and
    # 2 a for y: checked against that closed form (an FP64 cuSOLVER inverse), and the FP64 gradient
    # against central finite differences (h = 1e-6) along three random symmetric directions.  Stated
    # errors (relative, Frobenius): FP64 1e-8; mixed precision (28-bit panel products, amplified by the
    # condition number, about 1e5 here) 1e-4.
    n = 2048
    a = oracle.gen_rbf(n, seed=31, ell=0.2, sigma2=1.0, noise=1e-2)
    y = oracle.normal(32, n)
    G, gy = _gp_gradient(gbllt, a, y, mixed)
    A = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Ainv = torch.cholesky_inverse(torch.linalg.cholesky(A)).cpu().numpy()
    al = np.linalg.solve(a, y)
    want = Ainv - np.outer(al, al)
    tol = 1e-4 if mixed else 1e-8
    assert np.linalg.norm(G - want) <= tol * np.linalg.norm(want)
    assert np.linalg.norm(gy - 2.0 * al) <= 1e-10 * np.linalg.norm(al)
    if mixed:
        return

    def f(ap):
        Lp = np.linalg.cholesky(ap)
        return 2.0 * np.sum(np.log(np.diag(Lp))) + float(y @ np.linalg.solve(ap, y))

    rng = np.random.default_rng(5)
    for _ in range(3):
        E = rng.standard_normal((n, n)) * 1e-3
        E = E + E.T
        h = 1e-6
        fd = (f(a + h * E) - f(a - h * E)) / (2 * h)
        an = float(np.sum(G * E))
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1.0), (fd, an)


class GPObjective(torch.autograd.Function):
    """f(A, y) = logdet A + y^T A^{-1} y through the GPU factorisation, solve and their adjoints.
    A is read through its lower triangle (so its gradient lives there: off-diagonal entries carry
    both symmetric halves)."""

    @staticmethod
    def forward(ctx, A, y):
        import gbllt
        n = A.shape[0]
        s = torch.cuda.current_stream().cuda_stream
        L = A.detach().T.contiguous()  # column-major storage of A
        info = torch.zeros(1, dtype=torch.int64, device=A.device)
        gbllt.potrf_dev(L, n, n, info, "L", s)
        alpha = y.detach().clone().reshape(1, n)
        gbllt.potrs_dev(L, n, n, alpha, 1, n, "L", s)
        diag = torch.diagonal(L)
        f = 2.0 * torch.log(diag).sum() + torch.dot(y.detach(), alpha.reshape(n))
        ctx.save_for_backward(L, alpha, y.detach())
        return f

    @staticmethod
    def backward(ctx, g):
        import gbllt
        L, alpha, y = ctx.saved_tensors
        n = L.shape[0]
        s = torch.cuda.current_stream().cuda_stream
        # logdet: Lbar = diag(2 / L_ii); the adjoint of the factorisation turns it into Abar
        M = torch.zeros_like(L)
        M.diagonal().copy_(2.0 / torch.diagonal(L))
        gbllt.potrf_adjoint_dev(L, n, n, M, n, s)
        # quadratic term: x = A^{-1} y with xbar = y  ->  bbar = A^{-1} y, Abar -= sym(bbar x^T)
        bbar = torch.empty_like(alpha)
        gbllt.potrs_adjoint_dev(L, n, n, alpha, n, y.reshape(1, n), n, bbar, n, 1, M, n, s)
        Abar = M.T.tril()  # row-major view of the column-major lower triangle
        gA = (2.0 * Abar - torch.diag(torch.diagonal(Abar))) * g
        gy = (alpha.reshape(n) + bbar.reshape(n)) * g
        return gA, gy


def test_gp_objective_gradient_matches_closed_form(oracle, gbllt):
    n = 300
    a = oracle.gen_rbf(n, seed=31, ell=0.2, sigma2=1.0, noise=1e-2)
    y = oracle.normal(32, n)
    A = torch.from_numpy(np.ascontiguousarray(a)).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda().requires_grad_(True)
    f = GPObjective.apply(A, yt)
    f.backward()
    fr, dA, dy = oracle.gp_objective_ref(a, y)
    assert abs(float(f) - fr) <= 1e-10 * abs(fr)
    got = A.grad.cpu().numpy()
    want = np.tril(2.0 * dA - np.diag(np.diag(dA)))
    assert np.linalg.norm(got - want) <= 1e-8 * np.linalg.norm(want)
    assert np.linalg.norm(yt.grad.cpu().numpy() - dy) <= 1e-8 * np.linalg.norm(dy)


def test_gp_objective_gradcheck(oracle, gbllt):
    n = 24
    a = oracle.gen_gram(n, seed=11)
    y = oracle.normal(12, n)
    A = torch.from_numpy(np.ascontiguousarray(a)).cuda().requires_grad_(True)
    yt = torch.from_numpy(y).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(GPObjective.apply, (A, yt), eps=1e-6, atol=1e-7, rtol=1e-6)
