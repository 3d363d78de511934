"""Failure detection: a device-side bounded wait that runs out is reported, and the GPU stays usable.

The library's kernels wait on one another's signals (the solve's look-back flags, the tensor-core
pipelines' mbarriers, the rank update's block flags).  Every such wait gives up after a time limit
(2 s in normal calls), sets an error word and returns.  gbllt_selftest_wait_timeout runs two
triangular sweeps (FP64 and FP32) in which block 0 is never solved, so every other block waits for
a signal that nothing sets, with the limit shortened to a few milliseconds.  No GPU is faulted or
hung: the waits end by themselves and the kernels return.
"""
import numpy as np
import pytest


@pytest.mark.gpu
def test_bounded_wait_runs_out_and_is_reported(oracle, gbllt):
    rc, observed = gbllt.selftest_wait_timeout(20000)
    assert rc == gbllt.SUCCESS, gbllt.lib().gbllt_last_error()
    assert observed == gbllt.ERR_TIMEOUT
    # the context is still usable: a normal factor + solve right after, twice
    for seed in (1, 2):
        n, k = 300, 3
        a = oracle.gen_gram(n, seed=seed)
        b = np.asfortranarray(oracle.normal(seed + 10, n * k).reshape(n, k, order="F"))
        f = np.array(a, order="F", copy=True)
        x = np.array(b, order="F", copy=True)
        assert gbllt.posv(f, x) == 0
        assert oracle.backward_error(a, x, b) <= 1e-15


@pytest.mark.gpu
def test_selftest_runs_again(gbllt):
    # a second run starts from cleared error words and finds the same outcome
    for _ in range(2):
        rc, observed = gbllt.selftest_wait_timeout(5000)
        assert rc == gbllt.SUCCESS and observed == gbllt.ERR_TIMEOUT


def test_selftest_argument_checks(gbllt):
    # checked on the host before any device is touched
    assert gbllt.selftest_wait_timeout(10)[0] == -1
    assert gbllt.selftest_wait_timeout(10 ** 9)[0] == -1
