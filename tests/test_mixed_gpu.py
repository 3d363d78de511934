"""Mixed-precision solve with FP64 iterative refinement (gbllt_dposv_mixed[_dev]) against the
FP64 oracle.

Bar: the returned X has normwise backward error ||AX-B||_F/(||A||_F ||X||_F) <= 1e-14, measured
independently by the oracle (double-double residual), and agrees with the oracle's FP64 solution
to within kappa * 1e-13 (relative Frobenius; the forward error of any solution with backward error
1e-14 is bounded by a small multiple of kappa * 1e-14), where kappa is the condition number of
the seeded Householder-spectrum matrix.  Which low precisions must converge without the FP64 fallback follows
the usual IR condition kappa * u_factor < 1: every precision at kappa = 1e2; FP32, TF32x3, BF16x3
and TF32 at 1e4; FP32, TF32x3, BF16x3 and BF16x6 at 1e6.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRECS = ["fp32", "tf32", "tf32x3", "bf16", "bf16x3", "bf16x6"]
MUST_CONVERGE = {1e2: set(PRECS), 1e4: {"fp32", "tf32", "tf32x3", "bf16x3", "bf16x6"},
                 1e6: {"fp32", "tf32x3", "bf16x3", "bf16x6"}}


def _dev_solve(gbllt, a, b, opts, uplo="L"):
    import torch
    n, k = a.shape[0], b.shape[1]
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    X = torch.zeros_like(B)
    rc, rep = gbllt.posv_mixed_dev(A, n, n, B, n, X, n, k, opts, uplo, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, rep, np.asfortranarray(X.cpu().numpy().T)


@pytest.fixture(scope="module")
def spectra(oracle):
    n = 1536
    return {kappa: oracle.gen_householder(n, kappa) for kappa in (1e2, 1e4, 1e6)}


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6])
@pytest.mark.parametrize("prec", PRECS)
def test_mixed_refines_to_fp64(oracle, gbllt, spectra, kappa, prec):
    pytest.importorskip("torch")
    a = spectra[kappa]
    n = a.shape[0]
    b = np.asfortranarray(oracle.normal(12, n * 2).reshape(n, 2, order="F"))
    _, xr, info = oracle.solve(a, b)
    assert info == 0
    # without fallback: the low precision alone must get there where the theory says it can
    rc, rep, x = _dev_solve(gbllt, a, b, gbllt.mixed_opts(prec, 10, 1e-14, fallback=False))
    if prec in MUST_CONVERGE[kappa]:
        assert rc == gbllt.SUCCESS and rep["converged"] and not rep["used_fallback"], rep
        assert rep["steps"] <= 10
        assert oracle.backward_error(a, x, b) <= 1e-14
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= kappa * 1e-13
        # the first step already reflects the factor's precision (a broken tensor-core update would not)
        first = {"fp32": 1e-7, "tf32": 1e-5, "tf32x3": 1e-7, "bf16": 1e-4, "bf16x3": 1e-7, "bf16x6": 1e-8}[prec]
        assert rep["history"][0] <= first * max(1.0, kappa / 1e2)
    # with fallback: always FP64-accurate
    rc, rep, x = _dev_solve(gbllt, a, b, gbllt.mixed_opts(prec, 10, 1e-14, fallback=True))
    assert rc == gbllt.SUCCESS and rep["info"] == 0, rep
    assert oracle.backward_error(a, x, b) <= 1e-14
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= kappa * 1e-13


@pytest.mark.parametrize("n", [1, 7, 64, 200, 257, 300, 700])
@pytest.mark.parametrize("nrhs", [1, 3, 17, 70])
@pytest.mark.parametrize("residual", ["auto", "tensor", "fp64"])
def test_mixed_sizes(oracle, gbllt, n, nrhs, residual):
    pytest.importorskip("torch")
    a = oracle.gen_gram(n, seed=60 + n)
    b = np.asfortranarray(oracle.normal(61, n * nrhs).reshape(n, nrhs, order="F"))
    rc, rep, x = _dev_solve(gbllt, a, b, gbllt.mixed_opts("tf32x3", 10, 1e-14, fallback=False, residual=residual))
    assert rc == gbllt.SUCCESS and rep["converged"], rep
    assert oracle.backward_error(a, x, b) <= 1e-14


@pytest.mark.parametrize("n", [257, 700, 1000])
@pytest.mark.parametrize("prec", ["bf16x3", "bf16x6"])
def test_mixed_ragged_bf16(oracle, gbllt, n, prec):
    # orders that leave the tensor-core panel solve a last CTA of fewer than 64 rows, with the BF16
    # parts of the in-panel operand written from it
    pytest.importorskip("torch")
    a = oracle.gen_gram(n, seed=90 + n)
    b = np.asfortranarray(oracle.normal(91, n * 3).reshape(n, 3, order="F"))
    rc, rep, x = _dev_solve(gbllt, a, b, gbllt.mixed_opts(prec, 10, 1e-14, fallback=False))
    assert rc == gbllt.SUCCESS and rep["converged"] and not rep["used_fallback"], rep
    assert oracle.backward_error(a, x, b) <= 1e-14


@pytest.mark.parametrize("panel", [64, 128, 192, 320, 384, 512])
@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3", "bf16x6"])
def test_mixed_panel_widths(oracle, gbllt, spectra, panel, prec):
    # outer panels of any multiple of 64 (the default is 256 below n = 16384; from there on 384, and
    # 512 / 640 for BF16x3):
    # a ragged last panel (1536 = 4 * 384 = 3 * 512), the look-ahead split and the in-panel updates
    pytest.importorskip("torch")
    a = spectra[1e4]
    n = a.shape[0]
    b = np.asfortranarray(oracle.normal(13, n * 5).reshape(n, 5, order="F"))
    rc, rep, x = _dev_solve(gbllt, a, b, gbllt.mixed_opts(prec, 10, 1e-14, fallback=False, panel=panel))
    assert rc == gbllt.SUCCESS and rep["converged"] and not rep["used_fallback"], rep
    assert oracle.backward_error(a, x, b) <= 1e-14
    assert rep["history"][0] <= 1e-5


def test_mixed_panel_width_checked(gbllt):
    import torch
    n = 100
    A = torch.eye(n, dtype=torch.float64, device="cuda")
    B = torch.ones(1, n, dtype=torch.float64, device="cuda")
    X = torch.zeros_like(B)
    rc, _ = gbllt.posv_mixed_dev(A, n, n, B, n, X, n, 1, gbllt.mixed_opts("bf16x6", panel=100), "L", 0,
                                 raise_on_error=False)
    assert rc == -10  # LAPACK-style: argument 10 (opts) is invalid


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
def test_mixed_upper_and_host_api(oracle, gbllt, prec):
    n, k = 900, 2
    a = oracle.gen_householder(n, 1e4)
    b = np.asfortranarray(oracle.normal(70, n * k).reshape(n, k, order="F"))
    up = np.array(a, order="F")
    up[np.tril_indices(n, -1)] = np.nan  # only the upper triangle may be read
    rc, rep, x = _dev_solve(gbllt, up, b, gbllt.mixed_opts(prec, 10, 1e-14, fallback=False), uplo="U")
    assert rc == gbllt.SUCCESS and rep["converged"], rep
    assert oracle.backward_error(a, x, b) <= 1e-14
    lo = np.array(a, order="F")
    lo[np.triu_indices(n, 1)] = np.nan  # only the lower triangle may be read
    xh, rc, rep = gbllt.posv_mixed(lo, b, gbllt.mixed_opts(prec, 10, 1e-14, fallback=False), "L")
    assert rc == gbllt.SUCCESS and rep["converged"], rep
    assert oracle.backward_error(a, xh, b) <= 1e-14
    # row-major storage through the host entry point
    arow = np.ascontiguousarray(a)
    brow = np.ascontiguousarray(b)
    xrow = np.zeros_like(brow)
    r = gbllt.MixedReport()
    opts = gbllt.mixed_opts(prec, 10, 1e-14, fallback=False)
    rc = gbllt.lib().gbllt_dposv_mixed(gbllt.ROW_MAJOR, b"L", n, k, arow.ctypes.data, n, brow.ctypes.data, k,
                                       xrow.ctypes.data, k, ctypes.byref(opts), ctypes.byref(r))
    assert rc == gbllt.SUCCESS and r.converged
    assert oracle.backward_error(a, np.asfortranarray(xrow), b) <= 1e-14


def test_mixed_not_positive_definite(oracle, gbllt):
    n = 500
    a = oracle.gen_gram(n, seed=4)
    a[123, 123] = -5.0
    b = np.asfortranarray(oracle.normal(5, n).reshape(n, 1))
    rc, rep, x = _dev_solve(gbllt, a, b, gbllt.mixed_opts("tf32x3", 10, 1e-14, fallback=True))
    assert rc == gbllt.SUCCESS and rep["info"] == 124 and rep["used_fallback"]


def test_mixed_concurrent_host_threads(oracle, gbllt):
    """Mixed solves issued from 4 host threads on 4 streams at once (the look-ahead updates of the
    different solves then compete for SMs) give the same solutions as the same solves run one after
    another: the entry points are thread-safe and every kernel is deterministic."""
    torch = pytest.importorskip("torch")
    from concurrent.futures import ThreadPoolExecutor

    n, k, nsol = 1100, 3, 8
    mats = [np.asfortranarray(oracle.gen_householder(n, 1e4, v_seed0=60 + i)) for i in range(nsol)]
    rhs = [np.asfortranarray(oracle.normal(80 + i, n * k).reshape(n, k, order="F")) for i in range(nsol)]
    A = [torch.from_numpy(np.ascontiguousarray(m.T)).cuda() for m in mats]
    B = [torch.from_numpy(np.ascontiguousarray(r.T)).cuda() for r in rhs]
    opts = gbllt.mixed_opts("bf16x6", 10, 1e-14, False)

    def solve(i, stream):
        X = torch.zeros_like(B[i])
        rc, rep = gbllt.posv_mixed_dev(A[i], n, n, B[i], n, X, n, k, opts, "L", stream.cuda_stream,
                                       raise_on_error=False)
        stream.synchronize()
        return rc, rep, X

    serial = [solve(i, torch.cuda.current_stream()) for i in range(nsol)]
    streams = [torch.cuda.Stream() for _ in range(4)]

    def chain(t):
        torch.cuda.set_device(0)
        return [(i, solve(i, streams[t])) for i in range(t, nsol, 4)]

    with ThreadPoolExecutor(4) as pool:
        par = dict(kv for c in pool.map(chain, range(4)) for kv in c)
    for i in range(nsol):
        rc_s, rep_s, x_s = serial[i]
        rc_p, rep_p, x_p = par[i]
        assert rc_s == 0 and rc_p == 0, (rc_s, rc_p)
        assert rep_p["steps"] == rep_s["steps"]
        assert torch.equal(x_p, x_s)
        x = np.asfortranarray(x_p.cpu().numpy().T)
        assert oracle.backward_error(mats[i], x, rhs[i]) <= 1e-14


@pytest.mark.slow
@pytest.mark.parametrize("prec", ["bf16x6", "bf16x3"])
def test_mixed_full_size_default_panel(oracle, gbllt, prec):
    """n = 16384, 64 right-hand sides, Householder spectrum with kappa = 1e6: the default schedule at
    this order (outer panel 384, 512 for BF16x3, look-ahead with the growing SM reservation,
    tensor-core residual) reaches backward error 1e-14 without the FP64 fallback, checked by an
    independent FP64 residual (cuBLAS through torch)."""
    torch = pytest.importorskip("torch")
    n, k = 16384, 64
    A = torch.from_numpy(np.ascontiguousarray(oracle.gen_householder(n, 1e6))).cuda()  # symmetric
    g = torch.Generator(device="cuda").manual_seed(5)
    B = torch.randn(k, n, generator=g, dtype=torch.float64, device="cuda")  # column-major n x k
    X = torch.zeros_like(B)
    rc, rep = gbllt.posv_mixed_dev(A, n, n, B, n, X, n, k, gbllt.mixed_opts(prec, 10, 1e-14, fallback=False), "L",
                                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == gbllt.SUCCESS and rep["converged"] and not rep["used_fallback"], rep
    assert rep["steps"] <= 6
    be = float(torch.linalg.norm(A @ X.T - B.T) / (torch.linalg.norm(A) * torch.linalg.norm(X)))
    assert be <= 1e-14
