"""Per-launch profiling: gbllt_profile_read (per-class totals) and gbllt_profile_trace (one record per
launch, with its stream and device start / end) agree with each other, and the trace shows the
mixed-precision factorisation's launches on more than one stream."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trace_matches_class_totals(oracle, gbllt):
    torch = pytest.importorskip("torch")
    n, k = 1100, 3
    a = oracle.gen_householder(n, 1e4)
    b = np.asfortranarray(oracle.normal(3, n * k).reshape(n, k, order="F"))
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    X = torch.zeros_like(B)
    s = torch.cuda.current_stream().cuda_stream
    gbllt.profile_enable(True)
    try:
        rc, rep = gbllt.posv_mixed_dev(A, n, n, B, n, X, n, k, gbllt.mixed_opts("bf16x6", 10, 1e-14, False), "L", s)
        torch.cuda.synchronize()
        assert rc == gbllt.SUCCESS and rep["converged"]
        totals = gbllt.profile_read()
        trace = gbllt.profile_trace()
    finally:
        gbllt.profile_enable(False)
    assert len(trace) == sum(v["launches"] for v in totals.values())
    assert trace[0]["start_ms"] == 0.0
    for r in trace:
        assert 0.0 <= r["start_ms"] <= r["end_ms"]
        assert r["name"] in totals
    for name, v in totals.items():
        recs = [r for r in trace if r["name"] == name]
        assert len(recs) == v["launches"]
        # event times resolve to about half a microsecond: a few microseconds per launch at most
        assert sum(r["end_ms"] - r["start_ms"] for r in recs) == pytest.approx(v["ms"], rel=1e-3,
                                                                                abs=0.005 * v["launches"])
        assert sum(r["flops"] for r in recs) == pytest.approx(v["flops"], rel=1e-12)
    # the look-ahead schedule: the factorisation's launches run on several internal streams
    assert len({r["stream"] for r in trace}) >= 2
    # the whole solve spans the last launch's end
    assert max(r["end_ms"] for r in trace) > 0.0
    # after disabling, nothing is recorded
    assert gbllt.profile_trace() == []
