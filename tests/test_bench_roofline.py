"""The roofline arithmetic of bench.py on CPU: the algorithmic work per launch of the dominant
kernel group, the achieved rate against the measured peak, and the DRAM traffic scaled from
the ncu capture, for made-up per-kernel CUDA-event times."""
import math

import pytest


@pytest.fixture(scope="module")
def bench():
    import bench as b
    return b


def test_lu_gemm_flops_counts_every_panel_step(bench):
    # n = 64, panel width 32: one trailing update of 32 x 32 entries with K = 32
    assert bench.lu_gemm_flops(64, per_mac=1) == 32 * 32 * 32
    # n = 100: steps k = 0, 32, 64 (widths 32, 32, 32) and k = 96 (width 4, nothing left)
    want = 68 * 68 * 32 + 36 * 36 * 32 + 4 * 4 * 32
    assert bench.lu_gemm_flops(100, per_mac=1) == want
    assert bench.lu_gemm_flops(100, per_mac=8) == 8 * want


def test_ozaki_roofline(bench):
    n, n_omega, steps = 2000, 30, 5
    launches_per_step = 71
    per_launch_ms = 0.36
    prof = {"lu_gemm_ozaki": (per_launch_ms * launches_per_step * steps, launches_per_step * steps),
            "assemble_wave_wu": (22.0 * steps, steps)}
    peaks = {"bf16_tflops": 1938.2, "hbm_gbs": 6690.8, "source": "measured"}
    r = bench.roofline(prof, steps, n, n_omega, 1.058, peaks)
    macs = bench.lu_gemm_flops(n, per_mac=1) * n_omega / launches_per_step
    achieved = macs * bench.OZAKI_TENSOR_FLOPS_PER_MAC / (per_launch_ms * 1e-3) / 1e12
    assert r["kernel"] == "lu_gemm_ozaki" and r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert math.isclose(r["achieved"], achieved, rel_tol=1e-12)
    assert math.isclose(r["frac"], achieved / 1938.2, rel_tol=1e-12)
    assert math.isclose(r["fp64_equivalent_tflops"], macs * 8 / (per_launch_ms * 1e-3) / 1e12, rel_tol=1e-12)
    # traffic: bytes per trailing entry (32 complex multiply-adds each) times the entries
    assert math.isclose(r["traffic"], bench.NCU["lu_gemm_ozaki"]["dram_bytes_per_trailing_entry"] * macs / 32,
                        rel_tol=1e-12)
    total = prof["lu_gemm_ozaki"][0] + prof["assemble_wave_wu"][0]
    assert math.isclose(r["share"], prof["lu_gemm_ozaki"][0] / total, rel_tol=1e-12)


def test_wu_roofline_as_the_next_group(bench):
    n, n_omega, steps = 2000, 30, 5
    prof = {"assemble_wave_wu": (22.0 * steps, steps), "lu_panel_f64": (14.8 * steps, 144 * steps)}
    r = bench.roofline(prof, steps, n, n_omega, 1.058, {"bf16_tflops": 1938.2, "hbm_gbs": 6690.8,
                                                       "source": "measured"}, total_ms=300.0)
    pairs = n * (n + 1) / 2 * n_omega
    achieved = pairs * bench.WU_FLOPS_PER_UNORDERED_PAIR / 22.0e-3 / 1e12
    assert r["kernel"] == "assemble_wave_wu" and r["bound"] == "fp64"
    assert math.isclose(r["achieved"], achieved, rel_tol=1e-12)
    assert math.isclose(r["frac"], achieved / 1.058, rel_tol=1e-12)
    assert math.isclose(r["share"], 22.0 * steps / 300.0, rel_tol=1e-12)
