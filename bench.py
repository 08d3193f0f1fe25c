"""Throughput of the sampling-lattice hot path: effective samples/s of (sweep + E_loc + gradient).

One step = one sweep of every chain followed by the observation of its configuration (local
energy, gradient holes, reweighted accumulators).  B chains run at once; a step yields B samples.
Effective samples/s = samples/s / (2 tau_int(E_loc)), tau_int estimated from the E_loc series of every
chain (each chain's own mean subtracted, autocovariance pooled over chains, Sokal window c=5).

Workloads (seeded synthetic PEPS, no dataset involved; the configurations of the reference's
benchmark statement, C1..C5):
  heis4x4      C1: 4x4 Heisenberg (J=1), no symmetry, D=4, Dcut=16, tensors N(0,1)/sqrt(2 D^z),
               Neel start, 64 thermalisation sweeps, 1024 chains
  heis8x8u1    C2 (default): 8x8 Heisenberg, U(1) bonds {-1:2, 0:2, +1:2} (D=6), Dcut=36, blocks
               N(0,1), Neel start (total Sz = 0), 4096 chains = 4096 samples per step (the resident
               blocks, 3 x 152 SMs, take the chains in nine waves), 2 thermalisation sweeps, 1 timed step
  tv8x8        C3: 8x8 spinless t-V (t = V = 1), Fermi U(1), 32 particles, bonds {Q-1:2, Q:4, Q+1:2}
               along the charge flow and {-1:2, 0:4, +1:2} on interior D bonds (D=8), Dcut=64; one
               resident wave of chains from random fillings with nonzero amplitude
  heis6x6u1d4  C4 member: 6x6, U(1) {-1:1, 0:2, +1:1} (D=4), Dcut=16, 2048 chains
  heis12x12u1  C4 member: 12x12, U(1) {-1:2, 0:4, +1:2} (D=8), Dcut=64, one resident wave
  heis10x10u1  C5 lattice: 10x10, U(1) {-1:2, 0:2, +1:2} (D=6), Dcut=36, 456 chains
  heis6x6u1    a small U(1) case (D=6, Dcut=16, 16 chains) for ncu captures
  c4batch      C4: heis6x6u1d4, heis8x8u1 and heis12x12u1 swept in one CUDA-graph launch
               (tnsp_sweep_batch), blocks per SM chosen per lattice by tnsp_gb300.autotune
  heis10x10u1_proposal  C5: the learned proposal (autoregressive network trained on plain-sweep
               configurations, Metropolis-Hastings independence moves with exact amplitudes between
               sweeps) against the plain sweep on the 10x10 lattice

Precision: the metric is quoted at fixed error against float64 (|dE/site| <= 1e-6).  The U(1) and t-V
workloads run the double-float sampler (dd: float pairs, ~46-bit, on the FP32 pipe, which GB300 runs at
64x its FP64 rate); heis4x4 and heis6x6u1 run float64.  Outside float64 the chains' final
configurations are observed once more in the same precision and in float64 (observe-only launches)
and the E_loc, energy-per-site and gradient differences are reported under "fp64_check".  float32
and the mixed sampler (float32 contractions) do not meet the bar on the 8x8 lattice.

Roofline: the block GEMMs of the path are its tensor-pipe work (the reference's per-sector 2mnk count,
measured on the reference by oracle/count_gemm_flops.py, per sample); achieved = that count x samples
per launch / CUDA-event launch time, against the measured sustained bf16 tensor rate.  The kernel runs
them as double-float on the FP32 pipe; the per-sector QR / SVD work (counted in the kernel with the
Golub-Van Loan operation counts) and the executed (dense, padded) flops are reported beside it.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--precision fp64|dd|fp32|mixed]
python bench.py --impl reference ...   (the oracle restatement of the reference on host cores)
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "heis4x4": dict(kind="heis", L1=4, L2=4, D=4, sectors=None, cut=16, scale=True, chains=1024, therm=64, steps=5,
                    precision="fp64", config="C1"),
    "heis8x8u1": dict(kind="heis", L1=8, L2=8, D=6, sectors=(2, 2, 2), cut=36, scale=False, chains=4096, therm=2,
                      steps=1, precision="dd", config="C2"),
    "tv8x8": dict(kind="tv", L1=8, L2=8, D=(2, 4, 2), interior=((-1, 2), (0, 4), (1, 2)), particles=32, cut=64,
                  chains=0, therm=1, steps=1, precision="dd", config="C3"),
    "heis6x6u1d4": dict(kind="heis", L1=6, L2=6, D=4, sectors=(1, 2, 1), cut=16, scale=False, chains=2048, therm=2,
                        steps=2, precision="dd", config="C4"),
    "heis12x12u1": dict(kind="heis", L1=12, L2=12, D=8, sectors=(2, 4, 2), cut=64, scale=False, chains=0, therm=1,
                        steps=1, precision="dd", config="C4"),
    "heis10x10u1": dict(kind="heis", L1=10, L2=10, D=6, sectors=(2, 2, 2), cut=36, scale=False, chains=456, therm=2,
                        steps=2, precision="dd", config="C5"),
    # a small U(1) case for kernel profiling (ncu --set full ends by itself on it)
    "heis6x6u1": dict(kind="heis", L1=6, L2=6, D=6, sectors=(2, 2, 2), cut=16, scale=False, chains=16, therm=1,
                      steps=1, precision="fp64", config="small"),
}
DEFAULT_WORKLOAD = "heis8x8u1"
BATCH_WORKLOADS = {"c4batch": (("heis6x6u1d4", 2048), ("heis8x8u1", 2048), ("heis12x12u1", 0))}
PROPOSAL_WORKLOADS = {"heis10x10u1_proposal": "heis10x10u1"}
# Algorithmic block-GEMM flops per sample (sweep + observation with energy and gradient) of the
# reference's path on each lattice: 2 x the multiply-adds between allowed blocks of every Tensor.contract,
# measured by running the reference itself with its contract wrapped (oracle/count_gemm_flops.py; two to
# four samples after one thermalisation sweep, the reference's own seeding of the same lattice shape).
GEMM_FLOPS_PER_SAMPLE = {"heis4x4": 3.5745e6, "heis8x8u1": 1.2953e9, "tv8x8": 3.4186e10, "heis6x6u1d4": 3.1951e6,
                         "heis10x10u1": 3.3284e9, "heis12x12u1": 1.7904e11}
FP64_NOMINAL_GFLOPS = 1250.0
# FP32 pipe: 152 SMs x 128 FMA/clk x 2 flops x 2.07 GHz; one double-float multiply-add (the sampler's
# inner operation in TNSP_DD mode: 1 FMUL + 3 FFMA + 11 FADD) issues 15 FP32 instructions, so its flop
# peak is 1/15 of the FP32 flop rate
FP32_NOMINAL_GFLOPS = 152 * 128 * 2 * 2.07
DD_FMA_INSTRUCTIONS = 15
DD_NOMINAL_GFLOPS = FP32_NOMINAL_GFLOPS / DD_FMA_INSTRUCTIONS
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per chain-sample of the sweep kernel, from
# one ncu capture of a small launch of the same kernel and lattice (one sweep + observation of a few
# dozen chains), divided by its chains: the traffic of a launch is the chains it processes times this
MEASURED_DRAM_BYTES_PER_SAMPLE = {("heis8x8u1", "dd"): 1.187e9}  # 15.11 GB read + 22.88 GB written, 32 chains
# seconds per sample of the oracle port over the reference's own compiled CPU path, one thread each, on
# the 8x8 U(1) lattice (oracle/time_reference.py on an x86 core: reference 1.160 s, port 2.426 s)
PORT_OVER_REFERENCE_TIME = 2.09


def _jsonable(o):
    """numpy scalars and arrays in the result line"""
    return o.tolist() if hasattr(o, "tolist") else str(o)


def _measured_peaks():
    """The machine's measured peaks (MEASURED_PEAKS.json beside this file: STREAM-style HBM copy GB/s,
    cuBLAS bf16 TFLOP/s burst and sustained), or {}."""
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def make_lattice(w, seed=20240601):
    """The workload's lattice (a tnsp_gb300 SamplingLattice; t-V lattices carry their fermion tables)."""
    if w["kind"] == "tv":
        from tnsp_gb300.fermion import random_tv
        return random_tv(w["L1"], w["L2"], w["D"], w["particles"], seed=seed,
                         interior=[tuple(x) for x in w["interior"]]).sampling_lattice()
    from tnsp_gb300.lattice import random_heisenberg
    return random_heisenberg(w["L1"], w["L2"], w["D"], seed=seed, scale=w["scale"], sectors=w["sectors"])


def _first_filling(w, lat):
    """A configuration of the workload's sector: the Neel state, or the first sites filled (t-V)."""
    from tnsp_gb300.lattice import neel
    if w["kind"] != "tv":
        return neel(lat.L1, lat.L2)
    c = np.zeros(lat.L1 * lat.L2, dtype=np.int32)
    c[:w["particles"]] = 1
    return c.reshape(lat.L1, lat.L2)


def chain_starts(w, sampler, lat, B, seed=11):
    """Start configurations of B chains: the Neel state (total Sz = 0) for spin lattices; for t-V lattices
    random fillings with the lattice's particle number and a nonzero amplitude (checked on the device
    with the sampler's amplitude kernel, as the reference's start is checked with hole(()))."""
    if w["kind"] != "tv":
        return np.broadcast_to(_first_filling(w, lat), (B, lat.L1, lat.L2)).copy()
    rng = np.random.default_rng(seed)
    n = lat.L1 * lat.L2
    found = []
    batch = max(B, sampler.resident_chains())
    while len(found) < B:
        cand = np.zeros((batch, n), dtype=np.int32)
        for c in cand:
            c[rng.choice(n, size=w["particles"], replace=False)] = 1
        m, _ = sampler.amplitude(cand.reshape(-1, lat.L1, lat.L2))
        found += [c for c, x in zip(cand, m) if x != 0.0]
    return np.array(found[:B]).reshape(B, lat.L1, lat.L2)


# svd_other = the SVD's gather, pivoted QR, Q*J, global selection and output (everything but the Jacobi)
PHASE_NAMES = ("two_line", "sectors", "qr", "r_absorb", "jacobi", "svd_other", "us_absorb", "strip", None, "observe",
               None, None)


def phase_share(cycles):
    """Share of the timed phases in the summed SM cycles of all blocks (counter slots 4..15; the
    unnamed slots hold event counts)."""
    timed = {n: float(c) for n, c in zip(PHASE_NAMES, cycles) if n is not None}
    tot = max(1.0, sum(timed.values()))
    return {n: c / tot for n, c in timed.items() if c > 0}


def tau_int(series, window=5.0):
    """Integrated autocorrelation time of E_loc from independent chains; ``series`` has shape
    (n_samples, n_chains).  Each chain's own mean is subtracted, the autocovariance at lag t is pooled
    over chains (sum over chains and over the n - t pairs of each) and normalised by the pooled
    lag-0 variance, and the sum 1/2 + sum_t rho(t) is cut by Sokal's automatic window (the first
    t >= window * tau(t)).  Returns (tau, details); tau is floored at 1/2 (independent samples)."""
    x = np.asarray(series, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    n, c = x.shape
    if n < 3:
        return 0.5, {"n_per_chain": int(n), "chains": int(c), "window": 0, "raw": None}
    x = x - x.mean(axis=0, keepdims=True)
    var = (x * x).sum() / (n * c)
    if var <= 0:
        return 0.5, {"n_per_chain": int(n), "chains": int(c), "window": 0, "raw": None}
    tau, t = 0.5, 0
    for t in range(1, n - 1):
        rho = (x[:-t] * x[t:]).sum() / ((n - t) * c) / var
        tau += rho
        if t >= window * tau:
            break
    return max(tau, 0.5), {"n_per_chain": int(n), "chains": int(c), "window": int(t), "raw": float(tau)}


# ---------------------------------------------------------------------------------------------
# CPU arm: the oracle (numpy restatement of the reference path), one chain per process
# ---------------------------------------------------------------------------------------------
def _cpu_worker(args):
    workload, seed, seconds, max_samples = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle.peps_oracle import DensePEPS, ObserverAccumulator, SweepChain
    from tnsp_gb300.lattice import neel
    w = WORKLOADS[workload]
    lat = make_lattice(w)
    peps = DensePEPS([[lat[l1, l2] for l2 in range(lat.L2)] for l1 in range(lat.L1)], list(lat._hamiltonians.items()),
                     w["cut"], lat.charges)
    chain = SweepChain(peps, neel(lat.L1, lat.L2), seed)
    acc = ObserverAccumulator(peps)
    t0 = time.perf_counter()
    elocs = []
    while time.perf_counter() - t0 < seconds and len(elocs) < max_samples:
        poss, conf = chain.sweep()
        _, e, _ = acc.add(poss, conf, chain.env)
        elocs.append(e)
    return len(elocs), time.perf_counter() - t0, elocs


def cpu_baseline(workload, seconds, cores=None):
    """The oracle port on every host core: one single-threaded process per core (os.cpu_count()), one
    chain each, as the reference runs one chain per MPI rank."""
    import multiprocessing as mp
    cores = cores or (os.cpu_count() or 1)
    # one BLAS thread per process: the spawned workers inherit these before importing numpy
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(workload, 1000 + i, seconds, 10**9) for i in range(cores)])
    wall = time.perf_counter() - t0
    n = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    m = min(len(r[2]) for r in res)
    series = np.array([r[2][:m] for r in res]).T if m > 0 else np.zeros((0, cores))
    return dict(samples=n, seconds=busy, wall=wall, cores=cores, tau=tau_int(series)[0] if m >= 3 else None)


# ---------------------------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def reduce_over_ranks(dist, value, op="max", device="cpu"):
    """Max (timing) or sum (sample counts) of a float over all ranks; identity without dist."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def dist_setup(gpus):
    if gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, dist


def _sampler(w, lat, local, precision, B, seeds, tune=False, blocks_per_sm=0):
    """A Sampler with B chains of the workload (B <= 0: one resident wave), started by chain_starts;
    blocks_per_sm > 0 fixes the thread blocks (chains) resident per SM instead of the library's choice."""
    from tnsp_gb300.engine import Sampler
    from tnsp_gb300._lib import TNSP_OPT_BLOCKS_PER_SM
    s = Sampler(lat, w["cut"], device=local)
    first = _first_filling(w, lat)
    s.init_chains(first[None], seeds[:1], precision=precision)
    if blocks_per_sm > 0:
        s.set_option(TNSP_OPT_BLOCKS_PER_SM, blocks_per_sm)
    elif tune:
        from tnsp_gb300.autotune import tune_blocks_per_sm
        tune_blocks_per_sm(s, first[None], device=local)
    # plan for as many chains as the device holds at once (the library caps the slots it allocates)
    s.init_chains(np.broadcast_to(first, (4096,) + first.shape).copy(), np.arange(4096, dtype=np.uint64),
                  precision=precision)
    if B <= 0:
        B = s.resident_chains()
    starts = chain_starts(w, s, lat, B)
    seeds = np.arange(B, dtype=np.uint64) + seeds[0]
    s.init_chains(starts, seeds, precision=precision)
    return s, B, seeds


def _fp64_check(lat, w, local, conf, seeds, prec):
    """The chains' final configurations observed once in the run's precision and once in float64
    (observe-only launches): E_loc, reweighted energy per site and gradient differences."""
    from tnsp_gb300.engine import Sampler, estimators, gradient_from
    from tnsp_gb300._lib import TNSP_FP64
    obs = {}
    for p in (prec, TNSP_FP64):
        sx = Sampler(lat, w["cut"], device=local)
        sx.init_chains(conf, seeds, precision=p)
        sx.reset_observer()
        sx.sweep(0, observe=True)
        sc, de, ed = sx.read_observer(with_gradient=True)
        obs[p] = (np.asarray(sx.read_samples(1)[0][0]), estimators(sc, lat.site_number)[0], gradient_from(sc, de, ed))
        sx.close()
    (el, en, gr), (e64, en64, g64) = obs[prec], obs[TNSP_FP64]
    return {"chains": int(len(seeds)), "eloc_max_abs_err": float(np.abs(el - e64).max()),
            "eloc_max_rel_err": float((np.abs(el - e64) / np.maximum(np.abs(e64), 1e-300)).max()),
            "energy_per_site_err": float(abs(en - en64)),
            "gradient_max_rel_err": float(np.abs(gr - g64).max() / max(np.abs(g64).max(), 1e-300)),
            "bar": "|dE/site| <= 1e-6"}


def _roofline(workload, prec, counters, steps, launch_ms, samples_per_launch):
    """The roofline object of the sweep kernel (see the module docstring)."""
    from tnsp_gb300._lib import TNSP_DD, TNSP_FP64, TNSP_MIXED
    peaks = _measured_peaks()
    flops = np.asarray(counters[:4], dtype=np.float64) / steps
    cycles = counters[4:]
    gemm = GEMM_FLOPS_PER_SAMPLE.get(workload)
    peak = peaks.get("bf16_tflops_sustained")
    launch_s = launch_ms * 1e-3
    achieved = gemm * samples_per_launch / launch_s / 1e12 if gemm else None
    per_sample = MEASURED_DRAM_BYTES_PER_SAMPLE.get((workload, {TNSP_FP64: "fp64", TNSP_DD: "dd"}.get(prec)))
    traffic = per_sample * samples_per_launch if per_sample else None
    hbm = peaks.get("hbm_gbs")
    kname = {TNSP_FP64: "sweep_kernel<double, double>", TNSP_DD: "sweep_kernel<dd, dd>",
             TNSP_MIXED: "sweep_kernel<dd, float>"}.get(prec, "sweep_kernel<float, float>")
    executed = float(flops[0] + flops[3])
    factor = float(flops[1] + flops[2])
    dd_like = prec in (TNSP_DD, TNSP_MIXED)
    return {
        "bound": "tensor", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
        "frac": achieved / peak if (achieved is not None and peak) else None,
        "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured; cuBLAS bf16 GEMM, seconds-long loop)",
        "achieved_source": ("algorithmic block-GEMM flops per sample of the reference's path "
                            "(oracle/count_gemm_flops.py) x samples per launch / CUDA-event launch time"),
        "gemm_flops_per_sample": gemm,
        "traffic": traffic,
        "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a small launch of the same kernel "
                           "and lattice, per chain-sample, times the chains of this launch") if traffic else None,
        "dram_gbs": traffic / launch_s / 1e9 if traffic else None,
        "dram_frac_of_measured_hbm": traffic / launch_s / 1e9 / hbm if (traffic and hbm) else None,
        "limiter": ("latency: the kernel issues on a small fraction of its cycles (stalls on dependent FP32 "
                    "operations, memory and block barriers), far from both the FP32-pipe and the HBM roofs"),
        "per_sample": {"gemm_algorithmic": gemm,
                       "qr_svd_algorithmic": factor / samples_per_launch,
                       "contraction_executed": executed / samples_per_launch},
        "fp32_pipe": {"executed_gflops": (executed + factor) / launch_s / 1e9,
                      "peak_gflops": DD_NOMINAL_GFLOPS if dd_like else
                      FP64_NOMINAL_GFLOPS if prec == TNSP_FP64 else FP32_NOMINAL_GFLOPS,
                      "peak_source": ("nominal: FP32 152 SMs x 128 FMA/clk x 2.07 GHz / 15 instructions per "
                                      "double-float multiply-add" if dd_like else
                                      "nominal FP64 1.25 TFLOP/s" if prec == TNSP_FP64 else "nominal FP32")},
        "phase_cycle_share": phase_share(cycles),
        # counter slots 14 and 15: truncated SVDs and their Jacobi sweeps (max over a call's sectors)
        "jacobi_sweeps_per_svd": float(counters[15] / counters[14]) if counters[14] > 0 else None,
    }


def run_ours(args):
    import torch
    from tnsp_gb300.engine import PRECISIONS, TNSP_DD, TNSP_FP32, TNSP_FP64, TNSP_MIXED, estimators
    rank, world, dist = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", 0))
    w = WORKLOADS[args.workload]
    lat = make_lattice(w)
    prec = PRECISIONS[args.precision]
    s, B, seeds = _sampler(w, lat, local, prec, args.chains or w["chains"],
                           np.array([7919 * (rank + 1)], dtype=np.uint64), blocks_per_sm=args.blocks_per_sm)
    t_setup = time.perf_counter()
    s.sweep(w["therm"])
    therm_s = time.perf_counter() - t_setup
    # warm-up steps (observed, untimed)
    s.reset_observer()
    warm_eloc = []
    for _ in range(args.warmup):
        s.sweep(1, observe=True)
        warm_eloc.append(s.read_samples(1)[0][0])
    s.counters(reset=True)
    # timed region: K steps, inputs resident on the device; the working set (per-chain scratch slots)
    # is far larger than L2
    elocs = []
    kernel_ms = 0.0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(os.path.join(tempfile.gettempdir(), f"tnsp_clocks_{rank}.csv"))
    with clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.sweep(1, observe=True)
            ms, _ = s.last_timing()
            kernel_ms += ms
            elocs.append(s.read_samples(1)[0][0])
        torch.cuda.synchronize()
        t_dev = time.perf_counter() - t0
    if dist:
        t_dev = reduce_over_ranks(dist, t_dev, "max", "cuda")
        dist.barrier()
    counters = s.counters(reset=True)
    scal, _, _ = s.read_observer(with_gradient=False)
    fp64_check = None
    if prec != TNSP_FP64:
        conf, _ = s.read_chains()
        fp64_check = _fp64_check(lat, w, local, conf, seeds, prec)
    # end-to-end through the public C ABI with host buffers: upload the tensors, sweep + observe,
    # read the accumulators (energy scalars, Delta, E*Delta) and the per-sample record
    n_params = int(sum(lat[l1, l2].size for l1, l2 in lat.sites()))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.upload()
        s.sweep(1, observe=True)
        s.read_observer(with_gradient=True)
        s.read_samples(1)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    if dist:
        t_e2e = reduce_over_ranks(dist, t_e2e, "max", "cuda")
    tau, tau_info = tau_int(np.array(warm_eloc + elocs))
    samples = B * args.steps * world
    raw = samples / t_dev
    value = raw / (2 * tau)
    e2e_raw = samples / t_e2e
    # per step: the float64 tensors (a fermionic lattice: its eight sign-folded slices per site too),
    # the bond extents and the index charges
    fermion = getattr(lat, "fermion", None)
    h2d = n_params * 8 * (5 if fermion is not None else 1) + lat.L1 * lat.L2 * 4 * 4
    if lat.charges is not None:
        h2d += lat.L1 * lat.L2 * 4 * int(np.max(lat.dims())) * 4 + lat.P * 4 + lat.L1 * lat.L2 * 4
    d2h = 8 * 8 + 2 * n_params * 8 + 3 * B * 8 + 4
    resident = s.resident_chains()
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu and world == 1 and w["kind"] == "heis":
        c = cpu_baseline(args.workload, args.cpu_seconds)
        cpu_raw = c["samples"] / c["seconds"]
        cpu = {"value": cpu_raw / (2 * tau), "unit": "effective samples/s", "cores": c["cores"], "kind": "port",
               "host_cpu_count": os.cpu_count(),
               "sample": (f"{c['samples']} samples: {c['cores']} single-threaded processes (every host core), one "
                          f"chain each from the Neel state, {args.cpu_seconds:.0f} s each; raw {cpu_raw:.3f} "
                          f"samples/s divided by 2*tau_int of the GPU chains (identical chain dynamics); the port "
                          f"takes {PORT_OVER_REFERENCE_TIME:.2f}x the reference's own compiled time per sample on one "
                          f"x86 core (oracle/time_reference.py), so the reference would reach about "
                          f"{cpu_raw * PORT_OVER_REFERENCE_TIME:.1f} raw samples/s here")}
    e_site = estimators(scal, lat.site_number)
    out = {
        "metric": "effective samples/s (E_loc + gradient) at fixed error vs FP64 oracle, 1 GB300",
        "value": value,
        "unit": "effective samples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_dev / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {TNSP_FP64: "f64", TNSP_FP32: "f32", TNSP_DD: "f32x2 (double-float)",
                  TNSP_MIXED: "f32 contractions, f32x2 (double-float) factorisations"}[prec],
        "data": "synthetic (seeded random PEPS; " + ("random fillings" if w["kind"] == "tv" else "Neel start") + ")",
        "config": {"workload": args.workload, "statement": w["config"], "lattice": f"{w['L1']}x{w['L2']}", "D": w["D"],
                   "sectors": w.get("sectors"), "Dcut": w["cut"], "precision": args.precision, "chains_per_gpu": B,
                   "blocks_per_sm": args.blocks_per_sm or "library default",
                   "resident_chains": resident, "thermalisation_sweeps": w["therm"],
                   "parallelism": f"replicas{world}", "l2": "working set larger than L2 (per-chain scratch slots)"},
        "raw_samples_per_s": raw,
        "tau_int": tau,
        "tau_int_estimate": dict(tau_info, method="per-chain means, pooled autocovariance, Sokal window c=5"),
        "energy_per_site": e_site[0],
        "energy_error": e_site[1],
        "acceptance": float(scal[7]) / max(1.0, float(scal[0])),
        "thermalisation_s": therm_s,
        "e2e": {"value": e2e_raw / (2 * tau), "unit": "effective samples/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps,
        "roofline": _roofline(args.workload, prec, counters, args.steps, kernel_ms / args.steps, B),
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "fp64_check": fp64_check,
    }
    print(json.dumps(out, default=_jsonable))


def run_batch(args):
    """C4: several lattices in one CUDA-graph launch (tnsp_sweep_batch), each with the blocks per SM the
    autotuner picked for it; per-lattice throughput in the batch and alone (double-float and float64,
    one wave), and double-float's error against float64 on the same configurations."""
    import torch
    from tnsp_gb300.engine import Sampler, TNSP_DD, TNSP_FP64
    from tnsp_gb300.autotune import tune_blocks_per_sm
    from tnsp_gb300._lib import TNSP_OPT_BLOCKS_PER_SM
    local = int(os.environ.get("LOCAL_RANK", 0))
    members = BATCH_WORKLOADS[args.workload]
    lats, samplers, tuned, Bs = [], [], {}, []
    for name, chains in members:
        w = WORKLOADS[name]
        lat = make_lattice(w)
        first = _first_filling(w, lat)[None]
        s = Sampler(lat, w["cut"], device=local)
        s.init_chains(first, np.array([1], dtype=np.uint64), precision=TNSP_DD)
        best, rates = tune_blocks_per_sm(s, first, device=local)
        s.init_chains(np.broadcast_to(first[0], (4096,) + first.shape[1:]).copy(), np.arange(4096, dtype=np.uint64),
                      precision=TNSP_DD)
        resident = s.resident_chains()
        B = chains if chains > 0 else resident
        s.init_chains(np.broadcast_to(first[0], (B,) + first.shape[1:]).copy(),
                      np.arange(B, dtype=np.uint64) + np.uint64(31), precision=TNSP_DD)
        tuned[name] = {"blocks_per_sm": best, "amplitudes_per_s": rates, "resident_chains": resident}
        lats.append(lat)
        samplers.append(s)
        Bs.append(B)
    Sampler.sweep_batch(samplers, 1)
    for s in samplers:
        s.reset_observer()
    for _ in range(args.warmup):
        Sampler.sweep_batch(samplers, 1, observe=True)
    torch.cuda.synchronize()
    clocks = Clocks(os.path.join(tempfile.gettempdir(), "tnsp_clocks_batch.csv"))
    elocs = [[] for _ in samplers]
    with clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            Sampler.sweep_batch(samplers, 1, observe=True)
            for k, s in enumerate(samplers):
                elocs[k].append(s.read_samples(1)[0][0])
        torch.cuda.synchronize()
        t_batch = time.perf_counter() - t0
    per = {}
    total_eff = 0.0
    for (name, _), s, lat, B, el in zip(members, samplers, lats, Bs, elocs):
        w = WORKLOADS[name]
        tau, _ = tau_int(np.array(el))
        conf, _ = s.read_chains()
        seeds = np.arange(B, dtype=np.uint64) + np.uint64(31)
        check = _fp64_check(lat, w, local, conf, seeds, TNSP_DD)
        # the same lattice alone, one resident wave, one observed sweep in each precision
        alone = {}
        nres = tuned[name]["resident_chains"]
        for pname, p in (("dd", TNSP_DD), ("fp64", TNSP_FP64)):
            sx = Sampler(lat, w["cut"], device=local)
            sx.set_option(TNSP_OPT_BLOCKS_PER_SM, tuned[name]["blocks_per_sm"])
            sx.init_chains(conf[:nres], seeds[:nres], precision=p)
            sx.sweep(1, observe=True)
            ms, _ = sx.last_timing()
            alone[pname] = min(nres, B) / (ms * 1e-3)
            sx.close()
        rate = B * args.steps / t_batch
        total_eff += rate / (2 * tau)
        per[name] = {"chains": B, "samples_per_s_in_batch": rate, "tau_int": tau,
                     "samples_per_s_alone_one_wave": alone, "fp64_check": check, "tuning": tuned[name]}
    out = {
        "metric": "effective samples/s (E_loc + gradient) at fixed error vs FP64 oracle, 1 GB300",
        "value": total_eff, "unit": "effective samples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_batch / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32x2 (double-float)", "data": "synthetic (seeded random PEPS, Neel start)",
        "config": {"workload": args.workload, "statement": "C4", "members": [n for n, _ in members],
                   "launch": "one CUDA graph per step (tnsp_sweep_batch)"},
        "per_lattice": per, "clocks": clocks.summary(), "gpu_launches": args.steps,
    }
    print(json.dumps(out, default=_jsonable))


def run_proposal(args):
    """C5: the plain sweep against sweeps mixed with learned independence proposals on the same
    lattice and chains; acceptance, tau_int(E_loc) and effective samples/s of both."""
    import torch
    from tnsp_gb300.engine import PRECISIONS, estimators
    from tnsp_gb300.proposal import AutoregressiveProposal, independence_step
    local = int(os.environ.get("LOCAL_RANK", 0))
    w = WORKLOADS[PROPOSAL_WORKLOADS[args.workload]]
    lat = make_lattice(w)
    prec = PRECISIONS[args.precision]
    n = lat.L1 * lat.L2
    s, B, seeds = _sampler(w, lat, local, prec, args.chains or w["chains"], np.array([4242], dtype=np.uint64))
    s.sweep(w["therm"])
    # training data: plain-sweep configurations, one per chain and sweep
    t0 = time.perf_counter()
    data = []
    for _ in range(args.train_sweeps):
        s.sweep(1)
        data.append(s.read_chains()[0].reshape(B, n))
    data = np.concatenate(data)
    t_data = time.perf_counter() - t0
    net = AutoregressiveProposal(n, hidden=256, seed=5, batch_capacity=max(1024, B))
    t0 = time.perf_counter()
    history = net.fit(data, epochs=args.train_epochs, batch=1024, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    state = s.read_chains()[0]
    rng = np.random.default_rng(9)
    result = {}
    for mode in ("plain", "proposal"):
        s.write_chains(state)
        s.reset_observer()
        el, acc = [], []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            if mode == "proposal":
                acc.append(independence_step(s, net, rng))
            s.sweep(1, observe=True)
            el.append(s.read_samples(1)[0][0])
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tau, info = tau_int(np.array(el))
        scal, _, _ = s.read_observer(with_gradient=False)
        e_site = estimators(scal, lat.site_number)
        result[mode] = {"samples_per_s": B * args.steps / dt, "tau_int": tau, "tau_int_estimate": info,
                        "effective_samples_per_s": B * args.steps / dt / (2 * tau),
                        "energy_per_site": e_site[0], "energy_error": e_site[1],
                        "acceptance": float(np.mean(acc)) if acc else None}
    gain = result["proposal"]["effective_samples_per_s"] / result["plain"]["effective_samples_per_s"]
    out = {
        "metric": "effective samples/s (E_loc + gradient) at fixed error vs FP64 oracle, 1 GB300",
        "value": result["proposal"]["effective_samples_per_s"], "unit": "effective samples/s", "n_gpus": 1,
        "steps": args.steps, "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32x2 (double-float); network bf16 weights, f32 accumulation",
        "data": "synthetic (seeded random PEPS, Neel start)",
        "config": {"workload": args.workload, "statement": "C5", "lattice": f"{w['L1']}x{w['L2']}", "D": w["D"],
                   "Dcut": w["cut"], "chains": B, "network": "masked MLP, 2 hidden layers of 256",
                   "training_configurations": int(data.shape[0]), "training_epochs": args.train_epochs},
        "training": {"data_s": t_data, "train_s": t_train, "nll_first_epoch": history[0], "nll_last_epoch": history[-1]},
        "plain": result["plain"], "proposal": result["proposal"], "effective_gain": gain,
    }
    print(json.dumps(out, default=_jsonable))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = WORKLOADS[args.workload]
    total = 0
    secs = 0.0
    taus = []
    per_step = max(5.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_baseline(args.workload, 2.0)
    for _ in range(args.steps):
        c = cpu_baseline(args.workload, per_step)
        total += c["samples"]
        secs += c["seconds"]
        if c["tau"]:
            taus.append(c["tau"])
    tau = float(np.mean(taus)) if taus else 0.5
    raw = total / secs
    value = raw / (2 * tau)
    cores = os.cpu_count() or 1
    out = {
        "metric": "effective samples/s (E_loc + gradient) at fixed error vs FP64 oracle, 1 GB300",
        "impl": "reference",
        "value": value,
        "unit": "effective samples/s",
        "n_gpus": 0,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded random PEPS, Neel start)",
        "config": {"workload": args.workload, "lattice": f"{w['L1']}x{w['L2']}", "D": w["D"], "sectors": w["sectors"],
                   "Dcut": w["cut"], "precision": "fp64", "parallelism": f"{cores} processes"},
        "raw_samples_per_s": raw,
        "tau_int": tau,
        "cpu_baseline": {"value": value, "unit": "effective samples/s", "cores": cores, "kind": "port",
                         "sample": (f"{total} samples over {args.steps} steps of {per_step:.0f} s, one chain per "
                                    f"single-threaded process on each of the {cores} host cores (the reference's "
                                    f"compiled module cannot be built on this host: its sources are not here); the "
                                    f"port takes {PORT_OVER_REFERENCE_TIME:.2f}x the reference's own time per sample on "
                                    "one x86 core (oracle/time_reference.py)")},
        "e2e": {"value": value, "unit": "effective samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out, default=_jsonable))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="timed steps (default: per workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) + sorted(PROPOSAL_WORKLOADS))
    ap.add_argument("--precision", default="", choices=["", "fp64", "dd", "fp32", "mixed"], help="default: per workload")
    ap.add_argument("--chains", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="chains resident per SM (default: the library's)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--train-sweeps", type=int, default=10, help="learned proposal: plain sweeps of training data")
    ap.add_argument("--train-epochs", type=int, default=20)
    args = ap.parse_args()
    if args.impl == "reference" and args.workload not in WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU port times single-lattice spin workloads"}))
        return
    if args.workload in BATCH_WORKLOADS:
        args.steps = args.steps or 1
        run_batch(args)
        return
    if args.workload in PROPOSAL_WORKLOADS:
        w = WORKLOADS[PROPOSAL_WORKLOADS[args.workload]]
        args.steps = args.steps or 12
        args.precision = args.precision or w["precision"]
        run_proposal(args)
        return
    w = WORKLOADS[args.workload]
    args.steps = args.steps or w["steps"]
    args.precision = args.precision or w["precision"]
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        if w["kind"] != "heis":
            print(json.dumps({"impl": "reference", "unavailable": "the CPU port times the spin lattices only"}))
            return
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
