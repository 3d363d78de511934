"""The FP64-to-FP32 rounding of the mixed solve's working copy (integer arithmetic on the bits, round
to nearest even), against the GPU's own conversion, bit for bit: random values over the whole FP32
range and beyond, exact ties on both sides, carries into the exponent, the largest float and the
values that round to infinity, the normal / subnormal boundary, zeros, infinities and NaN."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(sign, exp, frac):
    return np.array([(int(s) << 63) | (int(e) << 52) | int(f) for s, e, f in zip(sign, exp, frac)], dtype=np.uint64)


def _cases():
    rng = np.random.default_rng(7)
    out = []
    m = 1_000_000
    # random normal doubles with exponents from below the FP32 range to above it
    sign = rng.integers(0, 2, m)
    exp = rng.integers(1023 - 160, 1023 + 140, m)
    frac = rng.integers(0, 1 << 52, m, dtype=np.uint64)
    out.append(_bits(sign, exp, frac))
    # exact ties (the 29 dropped bits are 1000...0), kept part odd and even, and one ulp either side
    k = 4096
    keep = rng.integers(0, 1 << 23, k, dtype=np.uint64)
    e = rng.integers(1023 - 126, 1023 + 128, k)
    for delta in (0, 1, -1):
        f = (keep << np.uint64(29)) | np.uint64(1 << 28)
        f = f + np.uint64(delta) if delta >= 0 else f - np.uint64(1)
        out.append(_bits(rng.integers(0, 2, k), e, f))
    # all-ones kept part: rounding up carries into the exponent (and at the top, to infinity)
    f = (np.uint64((1 << 23) - 1) << np.uint64(29)) | np.uint64(1 << 28)
    out.append(_bits([0, 1, 0, 1], [1023 + 127, 1023 + 127, 1023 - 3, 1023 + 5], [f - np.uint64(1), f, f, f]))
    # around the largest float, the smallest normal float and below
    specials = np.array([3.4028234663852886e38, 3.4028235677973366e38, 3.402823567797337e38, 1e39, -1e300,
                         1.1754943508222875e-38, 1.1754942807573643e-38, 1e-40, 1e-46, 5e-324, 0.0, -0.0,
                         np.inf, -np.inf, np.nan, 1.0, -1.0, 0.1, 2.0 ** -126, 2.0 ** -127, 2.0 ** 127,
                         2.0 ** 128], dtype=np.float64)
    out.append(specials.view(np.uint64))
    return np.concatenate(out).view(np.float64)


def test_f64_to_f32_matches_the_hardware_conversion(gbllt):
    torch = pytest.importorskip("torch")
    x = torch.from_numpy(_cases()).cuda()
    n = x.numel()
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    ref = torch.empty(n, dtype=torch.float32, device="cuda")
    rc = gbllt.lib().gbllt_selftest_f64_to_f32(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                              ctypes.c_void_p(ref.data_ptr()), n,
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert rc == gbllt.SUCCESS
    o = out.cpu().numpy().view(np.uint32)
    r = ref.cpu().numpy().view(np.uint32)
    nan = np.isnan(ref.cpu().numpy())
    assert np.array_equal(np.isnan(out.cpu().numpy()), nan)
    bad = np.nonzero((o != r) & ~nan)[0]
    assert bad.size == 0, (x.cpu().numpy()[bad[:5]], o[bad[:5]], r[bad[:5]])
    # and the same as torch's own conversion
    assert np.array_equal(o[~nan], x.float().cpu().numpy().view(np.uint32)[~nan])


def test_f64_to_f32_argument_checks(gbllt):
    assert gbllt.lib().gbllt_selftest_f64_to_f32(None, None, None, -1, None) == -4
    assert gbllt.lib().gbllt_selftest_f64_to_f32(None, None, None, 5, None) == -1
    assert gbllt.lib().gbllt_selftest_f64_to_f32(None, None, None, 0, None) == gbllt.SUCCESS
