"""The whole-step roofline of bench.py: T_roof = sum over the step's kernels
of max(bytes / BW_HBM, flops / peak), with the exact GEMMs against the bf16
tensor rate and FP64 work against the FP64 rate.  Host arithmetic only."""
import math

import bench
from channel_flow_gb300 import config

MIXED_STEP = ("k_tc_split_z1", "k_tc_gemm_z1", "k_yinv", "k_xprod", "k_yfwd", "k_tc_split_z2",
              "k_tc_gemm_z2", "k_curl", "k_tc_gemm_gl", "k_inc_solve", "k_inc_recover")
FP64_STEP = ("k_zc2v", "k_yinv", "k_xprod", "k_yfwd", "k_zcurl", "k_solve")


def test_sum_of_per_kernel_bounds():
    work = {"k_xprod": (6.0e8, 1.0e12), "k_tc_gemm_z1": (1.0e8, 4.0e12), "k_curl": (1.0e8, 3.0e9)}
    r = bench.step_roofline(work, "mixed", 1.0, 6000.0, 2000.0, 1.5)
    per = r["kernels"]
    # FP32 kernels of the mixed path: HBM only, whatever their flops
    assert per["k_xprod"]["bound"] == "hbm" and math.isclose(per["k_xprod"]["roof_us"], 100.0)
    # GEMM: 4e12 / 2e15 = 2 ms beats 1e8 / 6e12 = 16.7 us
    assert per["k_tc_gemm_z1"]["bound"] == "tensor" and math.isclose(per["k_tc_gemm_z1"]["roof_us"], 2000.0)
    # curl: 3e9 / 1.5e12 = 2 ms of FP64 work
    assert per["k_curl"]["bound"] == "fp64" and math.isclose(per["k_curl"]["roof_us"], 2000.0)
    assert math.isclose(r["t_roof_ms"], 4.1)
    assert math.isclose(r["achieved"], 4.1)


def test_fp64_path_counts_every_kernel_against_the_fp64_rate():
    cfg = config.CONFIGS["c3_retau180_128"]
    w = bench.kernel_work(cfg, 0, "fp64")
    r = bench.step_roofline({k: w[k] for k in FP64_STEP}, "fp64", 7.5, 6697.2, 1711.1, 1.2)
    assert all(v["bound"] == "fp64" for v in r["kernels"].values())
    assert 0.3 < r["achieved"] < 1.0


def test_mixed_channel_roofline_is_mostly_hbm():
    cfg = config.CONFIGS["c3_retau180_128"]
    w = bench.kernel_work(cfg, 0, "mixed")
    r = bench.step_roofline({k: w[k] for k in MIXED_STEP}, "mixed", 0.72, 6697.2, 1711.1, 1.2)
    per = r["kernels"]
    # the increment solve streams its operators once: about 772 MB per step
    assert math.isclose(per["k_inc_solve"]["roof_us"], w["k_inc_solve"][0] / 6697.2e9 * 1e6)
    assert 700e6 < w["k_inc_solve"][0] < 850e6
    assert per["k_inc_solve"]["bound"] == "hbm"
    # the step's bound is well under the measured step and above a third of it
    assert 0.3 < r["achieved"] < 1.0
    # at the 384x193x384 channel the Z1 and Z2 GEMMs turn tensor-bound
    cfg4 = config.CONFIGS["c4_retau550_384"]
    w4 = bench.kernel_work(cfg4, 0, "mixed")
    r4 = bench.step_roofline({k: w4[k] for k in MIXED_STEP}, "mixed", 13.2, 6697.2, 1711.1, 1.2)
    assert r4["kernels"]["k_tc_gemm_z1"]["bound"] == "tensor"
    assert r4["kernels"]["k_tc_gemm_z2"]["bound"] == "tensor"
