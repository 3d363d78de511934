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
