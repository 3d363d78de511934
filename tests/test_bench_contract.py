"""The bench's own arithmetic, on the CPU: the FP64-equivalent work of a solve, the laws that scale
an ncu DRAM capture to a launch of another size, and the roofline object's bound, peak and fraction
for each kind of kernel the bench can name."""
import importlib.util
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


PEAKS = {"hbm_gbs": 6000.0, "bf16_tflops": 2000.0, "tf32_tflops": 1000.0, "fp64_tflops": 1.0,
         "source": {"hbm_gbs": "h", "bf16_tflops": "b", "tf32_tflops": "t", "fp64_tflops": "d"}}


def test_llt_flops(bench):
    assert bench.llt_flops(3, 2) == pytest.approx(9.0 + 36.0)
    assert bench.llt_flops(16384, 64) == pytest.approx(16384 ** 3 / 3 + 2 * 16384 ** 2 * 64)


def test_ncu_traffic_scaling_laws(bench):
    n0, k0, ratio, law = bench.NCU_TRAFFIC["tc_update_bf16"]
    assert law == "ratio" and bench.ncu_traffic("tc_update_bf16", 32768, 64, 1e9) == pytest.approx(ratio * 1e9)
    assert bench.ncu_traffic("tc_update_bf16", 32768, 64, None) is None
    n0, k0, by, _ = bench.NCU_TRAFFIC["sweep_f32"]
    assert bench.ncu_traffic("sweep_f32", n0, k0) == pytest.approx(by)
    assert bench.ncu_traffic("sweep_f32", 2 * n0, k0) == pytest.approx(4 * by)
    assert bench.ncu_traffic("sweep_f32", n0, 4 * k0) == pytest.approx(by)  # L once, whatever k is
    n0, k0, by, _ = bench.NCU_TRAFFIC["symm_residual_f64"]
    assert bench.ncu_traffic("symm_residual_f64", n0, 2 * k0) == pytest.approx(2 * by)  # per 16-column chunk
    assert bench.ncu_traffic("symm_residual_f64", n0, k0 + 1) == pytest.approx(by * 5 / 4)
    assert bench.ncu_traffic("no_such_kernel", n0, k0) is None
    assert bench.ncu_traffic("sweep_f32", n0, 8) is None  # below one 16-column chunk: not captured


# profiled flops: tc_update_* counts every split product (nseg per algorithmic product); the ozaki
# kernels count the FP64 product once.  `achieved` is always the algorithmic rate; the executed
# split-product rate is reported beside it.
@pytest.mark.parametrize("name,nseg,bound,peak,algo_scale,products", [
    ("tc_update_bf16", 6, "tensor", 2000.0, 1 / 6, 6),
    ("tc_update_bf16", 1, "tensor", 2000.0, 1.0, 1),
    ("tc_update_tf32", 3, "tensor", 1000.0, 1 / 3, 3),
    ("syrk_tc_f64", 1, "tensor", 2000.0, 1.0, 36),
    ("residual_tc", 1, "tensor", 2000.0, 1.0, 36),
    ("syrk_lower_f64", 1, "tensor", 1.0, 1.0, 1),
])
def test_roofline_flop_bound_kernels(bench, name, nseg, bound, peak, algo_scale, products):
    st = {"ms": 2.0, "flops": 4e12, "bytes": 1e9, "launches": 4}
    r = bench.roofline_for(name, st, PEAKS, 16384, 64, nseg)
    assert r["bound"] == bound and r["unit"] == "TFLOP/s" and r["peak"] == peak
    assert r["achieved"] == pytest.approx(algo_scale * 4e12 / 2e-3 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    assert r["per_launch_flops"] == pytest.approx(algo_scale * 1e12)
    if products > 1:
        sp = r["split_products"]
        assert sp["products_per_algorithmic_product"] == products
        assert sp["tensor_achieved"] == pytest.approx(r["achieved"] * products)
        assert sp["tensor_frac"] == pytest.approx(sp["tensor_achieved"] / peak)
    else:
        assert "split_products" not in r


def test_default_config_is_the_metric_config(bench):
    # the metric (FP64 vs mixed + refinement at backward error <= 1e-14) is quoted on n = 32768
    c = bench.CONFIGS[bench.DEFAULT_CONFIG]
    assert (c["n"], c["nrhs"], c["kappa"]) == (32768, 64, 1e6)
    assert bench.SPLIT_PRODUCTS["bf16x6"] == 6 and bench.SPLIT_PRODUCTS["tf32x3"] == 3


def test_roofline_bandwidth_bound_kernel(bench):
    st = {"ms": 4.0, "flops": 1e10, "bytes": 2e9, "launches": 8}
    r = bench.roofline_for("sweep_f32", st, PEAKS, 16384, 64)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] == 6000.0
    assert r["achieved"] == pytest.approx(2e9 / 4e-3 / 1e9)
    assert r["traffic"] == pytest.approx(bench.ncu_traffic("sweep_f32", 16384, 64))
    assert "n^2" in r["traffic_source"]
