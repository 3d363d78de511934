"""Batched uneven small-system factor + solve (gbllt_?posv_batched[_dev]) against the oracle.

Every system is an independent LLT(A_s).solve(b_s); the oracle runs the restated Eigen blocked
LLT and two-sweep solve on each (oracle_?batched_posv).  Tolerances: factors and solutions within
1e-12 relative (double) and 2e-4 (float) of the oracle, per system; failing columns exact.  The
sizes include the edges of the shared-memory staging (double stages n <= ~167, float n <= ~238;
larger systems run in place in global memory) and the 1024 maximum.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EDGE = [0, 1, 2, 3, 31, 32, 33, 63, 64, 65, 100, 160, 166, 167, 168, 200, 237, 238, 239, 256, 300, 513, 1024]


def _batch(oracle, sizes, dtype, seed=100, shift=0.1):
    mats, rhs = [], []
    for i, n in enumerate(sizes):
        n = int(n)
        mats.append(oracle.gen_gram(n, seed=seed + i, shift=shift) if n else np.zeros((0, 0), order="F"))
        rhs.append(oracle.normal(seed + 50000 + i, n))
    a = np.concatenate([m.ravel(order="F") for m in mats] + [np.zeros(0)]).astype(dtype)
    b = np.concatenate(rhs + [np.zeros(0)]).astype(dtype)
    return mats, a, b


def _check(oracle, sizes, a_in, b_in, a_out, b_out, info, dtype):
    ref_a = a_in.copy()
    ref_b = b_in.copy()
    ref_info = oracle.batched_posv(np.asarray(sizes, dtype=np.int64), ref_a, ref_b)
    assert np.array_equal(info, ref_info)
    tol = 1e-12 if dtype == np.float64 else 2e-4
    off = boff = 0
    for n, inf in zip(sizes, ref_info):
        n = int(n)
        if n and inf == 0:
            lo = np.tril_indices(n)
            lg = a_out[off:off + n * n].reshape(n, n, order="F")[lo].astype(np.float64)
            lr = ref_a[off:off + n * n].reshape(n, n, order="F")[lo].astype(np.float64)
            assert np.linalg.norm(lg - lr) <= tol * np.linalg.norm(lr), n
            xg, xr = b_out[boff:boff + n].astype(np.float64), ref_b[boff:boff + n].astype(np.float64)
            assert np.linalg.norm(xg - xr) <= tol * 10 * np.linalg.norm(xr), n
        off += n * n
        boff += n


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batched_host_matches_oracle(oracle, gbllt, dtype):
    sizes = list(oracle.batch_sizes(200, seed=21, lo=4, hi=256)) + EDGE
    _, a, b = _batch(oracle, sizes, dtype)
    plan = gbllt.BatchPlan(sizes, dtype)
    a2, b2 = a.copy(), b.copy()
    info = plan.solve(a2, b2)
    _check(oracle, sizes, a, b, a2, b2, info, dtype)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("variant", list(range(16)))
def test_batched_every_variant_graph_replay(oracle, gbllt, variant, dtype):
    torch = pytest.importorskip("torch")
    assert gbllt.BATCH_VARIANTS == 16
    sizes = list(oracle.batch_sizes(120, seed=22, lo=4, hi=256)) + [1, 2, 4, 5, 16, 17, 33, 170, 255, 256]
    _, a, b = _batch(oracle, sizes, dtype, seed=300)
    plan = gbllt.BatchPlan(sizes, dtype)
    plan.set_variant(variant)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    di = torch.full((len(sizes),), -7, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    plan.solve_dev(da, db, di, s)           # captures the graph
    torch.cuda.synchronize()
    _check(oracle, sizes, a, b, da.cpu().numpy(), db.cpu().numpy(), di.cpu().numpy(), dtype)
    # replay the same graph on fresh inputs in the same buffers
    da.copy_(torch.from_numpy(a))
    db.copy_(torch.from_numpy(b))
    plan.solve_dev(da, db, di, s)
    torch.cuda.synchronize()
    _check(oracle, sizes, a, b, da.cpu().numpy(), db.cpu().numpy(), di.cpu().numpy(), dtype)


@pytest.mark.parametrize("variant", [3, 7, 8, 11, 12, 14])
def test_batched_failing_systems(oracle, gbllt, variant):
    sizes = [10, 70, 200, 40]
    mats, _, _ = _batch(oracle, sizes, np.float64, seed=500)
    mats[1][0, 0] = -1.0       # fails at column 0
    mats[2][150, 150] = -3.0   # fails at column 150 (in the second panel block)
    a = np.concatenate([m.ravel(order="F") for m in mats])
    b = np.concatenate([oracle.normal(9 + i, n) for i, n in enumerate(sizes)])
    plan = gbllt.BatchPlan(sizes, np.float64)
    plan.set_variant(variant)
    a2, b2 = a.copy(), b.copy()
    info = plan.solve(a2, b2)
    assert list(info) == [0, 1, 151, 0]
    _check(oracle, sizes, a, b, a2, b2, info, np.float64)


def test_batched_autotuner_cache(oracle, gbllt, tmp_path):
    sizes = list(oracle.batch_sizes(300, seed=23, lo=4, hi=256))
    cache = tmp_path / "tune.json"
    plan = gbllt.BatchPlan(sizes, np.float32)
    v = plan.tune(str(cache))
    assert 0 <= v < gbllt.BATCH_VARIANTS
    entries = json.loads(cache.read_text())
    assert len(entries) == 1
    (entry,) = entries.values()
    assert entry["variant"] == v and len(entry["ms"]) == gbllt.BATCH_VARIANTS and min(entry["ms"]) > 0
    plan2 = gbllt.BatchPlan(sizes, np.float32)
    assert plan2.tune(str(cache)) == v  # read back, no new sweep
    _, a, b = _batch(oracle, sizes, np.float32, seed=700)
    a2, b2 = a.copy(), b.copy()
    info = plan2.solve(a2, b2)
    _check(oracle, sizes, a, b, a2, b2, info, np.float32)


def _systems(a, b, sizes):
    off = boff = 0
    for n in sizes:
        n = int(n)
        yield a[off:off + n * n].reshape(n, n, order="F"), b[boff:boff + n], boff
        off += n * n
        boff += n


def _mixed(gbllt, plan, a, b, opts):
    torch = pytest.importorskip("torch")
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    dx = torch.zeros_like(db)
    di = torch.full((len(plan.sizes),), -7, dtype=torch.int64, device="cuda")
    rep = plan.solve_mixed_dev(da, db, dx, di, opts, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    # A and b are read only
    assert np.array_equal(da.cpu().numpy(), a) and np.array_equal(db.cpu().numpy(), b)
    return rep, dx.cpu().numpy(), di.cpu().numpy()


def test_batched_mixed_refines_every_system(oracle, gbllt):
    # FP32 factors + FP64 refinement: every system to backward error 1e-14 (the oracle's
    # double-double residual), within 1e-12 of the oracle's FP64 solution (kappa < 100 here)
    sizes = list(oracle.batch_sizes(300, seed=23, lo=4, hi=256)) + EDGE
    mats, a, b = _batch(oracle, sizes, np.float64, seed=500)
    plan = gbllt.BatchPlan(sizes, np.float64)
    rep, x, info = _mixed(gbllt, plan, a, b, gbllt.mixed_opts("fp32", 10, 1e-14, fallback=False))
    assert np.all(info == 0)
    assert rep["converged"] == len(sizes) and rep["fallback"] == 0
    assert 1 <= rep["steps"] <= 4 and rep["max_backward_error"] <= 1e-14
    ref_a, ref_b = a.copy(), b.copy()
    assert np.all(oracle.batched_posv(np.asarray(sizes, dtype=np.int64), ref_a, ref_b) == 0)
    for (m, bs, off), n in zip(_systems(a, b, sizes), sizes):
        if not n:
            continue
        xs = x[off:off + n]
        assert oracle.backward_error(np.asfortranarray(m), xs.reshape(n, 1), bs.reshape(n, 1)) <= 1e-14, n
        xr = ref_b[off:off + n]
        assert np.linalg.norm(xs - xr) <= 1e-12 * np.linalg.norm(xr), n


def test_batched_mixed_fallback_and_failures(oracle, gbllt):
    # ill-conditioned systems (kappa 1e10: the FP32 factorisation fails or the refinement stalls) and
    # a system that is not positive definite, among well-conditioned ones
    good = [40, 130, 7, 256]
    ill = [(64, 1e10), (200, 1e10)]
    sizes = good[:2] + [n for n, _ in ill] + good[2:] + [150]
    mats = [oracle.gen_gram(40, seed=1), oracle.gen_gram(130, seed=2), oracle.gen_householder(64, 1e10),
            oracle.gen_householder(200, 1e10), oracle.gen_gram(7, seed=3), oracle.gen_gram(256, seed=4)]
    bad = np.array(oracle.gen_gram(150, seed=5), order="F")
    bad[77, 77] = -1.0
    mats.append(bad)
    a = np.concatenate([m.ravel(order="F") for m in mats])
    b = np.concatenate([oracle.normal(600 + i, n) for i, n in enumerate(sizes)])
    plan = gbllt.BatchPlan(sizes, np.float64)
    # without fallback: the ill systems report a failed FP32 column or no convergence, the
    # indefinite one its FP32 failing column
    rep, x, info = _mixed(gbllt, plan, a, b, gbllt.mixed_opts("fp32", 10, 1e-14, fallback=False))
    assert list(info[[0, 1, 4, 5]]) == [0, 0, 0, 0]
    assert all(v == gbllt.BATCH_NOT_CONVERGED or v > 0 for v in info[[2, 3]])
    assert info[6] > 0 and rep["converged"] == 4
    # with fallback: the ill systems are solved in FP64 (backward error 1e-15), the indefinite one
    # reports the FP64 failing column of the oracle
    rep, x, info = _mixed(gbllt, plan, a, b, gbllt.mixed_opts("fp32", 10, 1e-14, fallback=True))
    want = oracle.blocked(np.array(bad, order="F"))
    assert list(info) == [0, 0, 0, 0, 0, 0, want + 1]
    assert rep["fallback"] == 3 and rep["converged"] == 4
    for k, ((m, bs, off), n) in enumerate(zip(_systems(a, b, sizes), sizes)):
        if k == 6:
            continue
        assert oracle.backward_error(np.asfortranarray(m), x[off:off + n].reshape(n, 1),
                                     bs.reshape(n, 1)) <= 1e-14, k


def test_batched_mixed_arguments(gbllt):
    torch = pytest.importorskip("torch")
    empty = gbllt.BatchPlan([], np.float64)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    i = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert empty.solve_mixed_dev(t, t, t, i)["converged"] == 0
    f32 = gbllt.BatchPlan([3], np.float32)
    rep = gbllt.BatchMixedReport()
    rc = gbllt.lib().gbllt_batch_dposv_mixed_dev(f32.handle, t.data_ptr(), t.data_ptr(), t.data_ptr(), i.data_ptr(),
                                                 None, None, 0)
    assert rc == -1  # an FP32 plan
    plan = gbllt.BatchPlan([3], np.float64)
    rc = gbllt.lib().gbllt_batch_dposv_mixed_dev(plan.handle, None, t.data_ptr(), t.data_ptr(), i.data_ptr(), None,
                                                 None, 0)
    assert rc == -2
    del rep
