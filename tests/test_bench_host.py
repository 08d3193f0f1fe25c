"""bench.py's host-side logic: the integrated autocorrelation time, phase shares, JSON line helpers."""
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_tau_int_of_independent_samples_is_one_half():
    x = np.random.default_rng(0).normal(size=(400, 64))
    assert abs(bench.tau_int(x)[0] - 0.5) < 0.1


def test_tau_int_of_short_chains_with_different_means():
    """Many short chains whose means differ (as chains still drifting after a short thermalisation):
    subtracting each chain's own mean keeps the offsets out of the autocorrelation."""
    rng = np.random.default_rng(2)
    x = rng.normal(size=(25, 456)) + 3.0 * rng.normal(size=(1, 456))
    tau, info = bench.tau_int(x)
    assert tau < 0.7 and info["n_per_chain"] == 25 and info["chains"] == 456


def test_default_workload_is_the_headline_configuration():
    """The default step is config 2 as stated: 8x8 U(1) bonds {-1:2, 0:2, +1:2}, Dcut 36, 4096 samples,
    at fixed error (double-float, checked against float64 in the line)."""
    w = bench.WORKLOADS[bench.DEFAULT_WORKLOAD]
    assert (w["L1"], w["L2"], w["D"], tuple(w["sectors"]), w["cut"]) == (8, 8, 6, (2, 2, 2), 36)
    assert w["chains"] == 4096 and w["precision"] == "dd" and w["config"] == "C2"


def test_tau_int_of_an_ar1_process():
    """x_t = a x_{t-1} + noise has tau_int = (1 + a) / (2 (1 - a)) (= 4.5 for a = 0.8)."""
    rng = np.random.default_rng(1)
    a, n, chains = 0.8, 4000, 32
    x = np.zeros((n, chains))
    for t in range(1, n):
        x[t] = a * x[t - 1] + rng.normal(size=chains)
    assert abs(bench.tau_int(x[200:])[0] - (1 + a) / (2 * (1 - a))) < 0.6


def test_tau_int_short_series_floor():
    assert bench.tau_int(np.ones((2, 4)))[0] == 0.5
    assert bench.tau_int(np.ones((10, 4)))[0] == 0.5  # no variance


def test_phase_share_ignores_event_count_slots():
    cycles = np.arange(1.0, 13.0)
    share = bench.phase_share(cycles)
    assert abs(sum(share.values()) - 1.0) < 1e-12
    assert set(share) == {n for n in bench.PHASE_NAMES if n is not None}


def test_json_line_accepts_numpy_values():
    line = json.dumps({"a": np.int32(2), "b": np.float64(0.5), "c": np.arange(3)}, default=bench._jsonable)
    assert json.loads(line) == {"a": 2, "b": 0.5, "c": [0, 1, 2]}


def test_reduce_over_ranks_without_a_group_is_identity():
    assert bench.reduce_over_ranks(None, 3.5) == 3.5


def test_workloads_are_consistent():
    for name, w in bench.WORKLOADS.items():
        assert w["precision"] in ("fp64", "dd", "fp32", "mixed"), name
        assert w["chains"] >= 0 and w["steps"] >= 1  # chains 0: one resident wave
    assert bench.DEFAULT_WORKLOAD in bench.WORKLOADS
    assert abs(bench.DD_NOMINAL_GFLOPS * bench.DD_FMA_INSTRUCTIONS - bench.FP32_NOMINAL_GFLOPS) < 1e-6


def test_roofline_fields_follow_from_the_counts():
    """achieved = algorithmic GEMM flops per sample x samples per launch / launch time; frac = achieved /
    the measured sustained bf16 rate; the per-sample split comes from the kernel's counters."""
    from tnsp_gb300._lib import TNSP_DD
    counters = np.zeros(16)
    counters[:4] = [4e12, 1e12, 2e12, 0.5e12]   # two steps: contraction, QR, SVD, strip flops
    counters[4:] = np.arange(1.0, 13.0)
    r = bench._roofline("heis8x8u1", TNSP_DD, counters, 2, 9000.0, 456)
    expect = bench.GEMM_FLOPS_PER_SAMPLE["heis8x8u1"] * 456 / 9.0 / 1e12
    assert abs(r["achieved"] - expect) < 1e-12 * expect
    peak = bench._measured_peaks().get("bf16_tflops_sustained")
    if peak:
        assert abs(r["frac"] - expect / peak) < 1e-12
    assert abs(r["per_sample"]["qr_svd_algorithmic"] - 1.5e12 / 456) < 1.0
    assert abs(r["per_sample"]["contraction_executed"] - 2.25e12 / 456) < 1.0
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"


def test_gemm_counts_name_known_workloads():
    assert set(bench.GEMM_FLOPS_PER_SAMPLE) <= set(bench.WORKLOADS)
    for members in bench.BATCH_WORKLOADS.values():
        assert all(n in bench.WORKLOADS for n, _ in members)
    assert all(v in bench.WORKLOADS for v in bench.PROPOSAL_WORKLOADS.values())
