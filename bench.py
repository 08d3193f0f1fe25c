"""Throughput of the sampling-lattice hot path: effective samples/s of (sweep + E_loc + gradient).

One step = one sweep of every chain followed by the observation of its configuration (local
energy, gradient holes, reweighted accumulators).  B chains run at once; a step yields B samples.
Effective samples/s = samples/s / (2 tau_int(E_loc)), tau_int estimated from the per-chain E_loc
series (pooled autocorrelation, Sokal window c=5).

Workloads (seeded synthetic PEPS, no dataset involved):
  heis4x4    4x4 Heisenberg (J=1), no symmetry, D=4, Dcut=16, tensors N(0,1)/sqrt(2 D^z),
             Neel start, 64 thermalisation sweeps, 1024 chains (1024 samples per step)
  heis6x6u1  6x6 Heisenberg, U(1) D=6, Dcut=16, 16 chains: the small case used for ncu captures
  heis8x8u1  8x8 Heisenberg, U(1) bonds {-1:2, 0:2, +1:2} (D=6), Dcut=36, blocks N(0,1),
             Neel start (total Sz = 0), 456 chains = one resident wave of 3 blocks x 152 SMs
             (the 4096-sample launch runs the same kernel for nine waves), 2 thermalisation sweeps
             (throughput does not depend on thermalisation)

Precision: the metric is quoted at fixed error against float64 (|dE/site| <= 1e-6).  The 8x8 U(1)
headline runs the double-float sampler (dd: float pairs, ~46-bit, on the FP32 pipe, which GB300 runs
at 64x its FP64 rate); heis4x4 and heis6x6u1 run float64.  Outside float64 the chains' final
configurations are observed once more in the same precision and in float64 (observe-only launches)
and the E_loc, energy-per-site and gradient differences are reported under "fp64_check".  float32
does not meet the bar on the 8x8 lattice (amplitude cancellations amplify its rounding).

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--precision fp64|dd|fp32]
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
    "heis4x4": dict(L1=4, L2=4, D=4, sectors=None, cut=16, scale=True, chains=1024, therm=64, steps=5,
                    precision="fp64"),
    "heis8x8u1": dict(L1=8, L2=8, D=6, sectors=(2, 2, 2), cut=36, scale=False, chains=456, therm=2, steps=2,
                      precision="dd"),
    # a small U(1) case for kernel profiling (ncu --set full ends by itself on it)
    "heis6x6u1": dict(L1=6, L2=6, D=6, sectors=(2, 2, 2), cut=16, scale=False, chains=16, therm=1, steps=1,
                      precision="fp64"),
}
DEFAULT_WORKLOAD = "heis8x8u1"
FP64_NOMINAL_GFLOPS = 1250.0
# FP32 pipe: 152 SMs x 128 FMA/clk x 2 flops x 2.07 GHz; one double-float multiply-add (the sampler's
# inner operation in TNSP_DD mode: 1 FMUL + 3 FFMA + 11 FADD) issues 15 FP32 instructions, so its flop
# peak is 1/15 of the FP32 flop rate
FP32_NOMINAL_GFLOPS = 152 * 128 * 2 * 2.07
DD_FMA_INSTRUCTIONS = 15
DD_NOMINAL_GFLOPS = FP32_NOMINAL_GFLOPS / DD_FMA_INSTRUCTIONS
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per chain-sample of the sweep kernel, from
# one ncu capture of the timed launch (profiles/sweep_kernel_dd_launches_heis8x8u1.md: 0.779 + 0.873 TB
# for 456 chains); scaled by the chains of a launch
MEASURED_DRAM_BYTES_PER_SAMPLE = {("heis8x8u1", "dd"): (0.779428e12 + 0.873435e12) / 456}


def _jsonable(o):
    """numpy scalars and arrays in the result line"""
    return o.tolist() if hasattr(o, "tolist") else str(o)


def _measured_hbm_gbs():
    """HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json beside this file), or None."""
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except Exception:
        return None


def make_lattice(w, seed=20240601):
    from tnsp_gb300.lattice import random_heisenberg
    return random_heisenberg(w["L1"], w["L2"], w["D"], seed=seed, scale=w["scale"], sectors=w["sectors"])


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
    import multiprocessing as mp
    cores = cores or min(os.cpu_count() or 1, 16)
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


def run_ours(args):
    import torch
    from tnsp_gb300.engine import PRECISIONS, Sampler, TNSP_DD, TNSP_FP32, TNSP_FP64, TNSP_MIXED
    from tnsp_gb300.lattice import neel
    rank, world, dist = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", 0))
    w = WORKLOADS[args.workload]
    B = args.chains or w["chains"]
    lat = make_lattice(w)
    prec = PRECISIONS[args.precision]
    s = Sampler(lat, w["cut"], device=local)
    seeds = np.arange(B, dtype=np.uint64) + np.uint64(7919 * (rank + 1))
    s.init_chains(neel(lat.L1, lat.L2), seeds, precision=prec)
    t_setup = time.perf_counter()
    s.sweep(w["therm"] if not args.quick_therm else 2)
    therm_s = time.perf_counter() - t_setup
    # warm-up steps (observed, untimed)
    s.reset_observer()
    warm_eloc = []
    for _ in range(args.warmup):
        s.sweep(1, observe=True)
        warm_eloc.append(s.read_samples(1)[0][0])
    s.counters(reset=True)
    # timed region: K steps, inputs resident on the device
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
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
    flops = s.counters(reset=True)
    fp64_check = None
    if prec != TNSP_FP64:
        # the chains' final configurations observed once in this precision and once in float64
        # (observe-only launches): E_loc, reweighted energy per site and gradient differences
        from tnsp_gb300.engine import estimators, gradient_from
        conf, _ = s.read_chains()
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
        fp64_check = {"chains": int(B), "eloc_max_abs_err": float(np.abs(el - e64).max()),
                      "eloc_max_rel_err": float((np.abs(el - e64) / np.maximum(np.abs(e64), 1e-300)).max()),
                      "energy_per_site_err": float(abs(en - en64)),
                      "gradient_max_rel_err": float(np.abs(gr - g64).max() / max(np.abs(g64).max(), 1e-300)),
                      "bar": "|dE/site| <= 1e-6"}
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
    series = np.array(warm_eloc + elocs)
    tau, tau_info = tau_int(series)
    samples = B * args.steps * world
    raw = samples / t_dev
    value = raw / (2 * tau)
    e2e_raw = samples / t_e2e
    # per step: the float64 tensors, the bond extents and (U(1) lattices) the index charges
    h2d = n_params * 8 + lat.L1 * lat.L2 * 4 * 4
    if lat.charges is not None:
        h2d += lat.L1 * lat.L2 * 4 * int(np.max(lat.dims())) * 4 + lat.P * 4 + lat.L1 * lat.L2 * 4
    d2h = 8 * 8 + 2 * n_params * 8 + 3 * B * 8 + 4
    avg_launch_ms = kernel_ms / args.steps
    cycles = flops[4:]
    flops = flops[:4]
    achieved = float(flops.sum()) / args.steps / (avg_launch_ms * 1e-3) / 1e9
    if rank != 0:
        return
    per_sample = MEASURED_DRAM_BYTES_PER_SAMPLE.get((args.workload, args.precision))
    traffic = per_sample * B if per_sample else None
    dram_gbs = traffic / (avg_launch_ms * 1e-3) / 1e9 if traffic else None
    hbm = _measured_hbm_gbs()
    dram_frac = dram_gbs / hbm if (dram_gbs and hbm) else None
    if prec == TNSP_FP64:
        bound, kname, peak = "fp64", "sweep_kernel<double>", FP64_NOMINAL_GFLOPS
        peak_src = "nominal GB300 FP64 1.25 TFLOP/s (MEASURED_PEAKS.json has no FP64 figure)"
    elif prec in (TNSP_DD, TNSP_MIXED):
        bound, kname, peak = "fp32 (double-float)", "sweep_kernel<dd>", DD_NOMINAL_GFLOPS
        peak_src = (f"nominal GB300 FP32 {FP32_NOMINAL_GFLOPS:.0f} GFLOP/s / {DD_FMA_INSTRUCTIONS} FP32 instructions "
                    "per double-float multiply-add (MEASURED_PEAKS.json has no FP32 figure)")
    else:
        bound, kname, peak = "fp32", "sweep_kernel<float>", FP32_NOMINAL_GFLOPS
        peak_src = "nominal GB300 FP32 (MEASURED_PEAKS.json has no FP32 figure)"
    cpu = None
    if not args.no_cpu and world == 1:
        c = cpu_baseline(args.workload, args.cpu_seconds)
        cpu_raw = c["samples"] / c["seconds"]
        cpu = {"value": cpu_raw / (2 * tau), "unit": "effective samples/s", "cores": c["cores"], "kind": "port",
               "sample": (f"{c['samples']} samples: {c['cores']} single-threaded processes, one chain each from the "
                          f"Neel state, {args.cpu_seconds:.0f} s each; raw {cpu_raw:.3f} samples/s divided by "
                          f"2*tau_int of the GPU chains (identical chain dynamics)")}
    scal, _, _ = s.read_observer(with_gradient=False)
    from tnsp_gb300.engine import estimators
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
        "data": "synthetic (seeded random PEPS, Neel start)",
        "config": {"workload": args.workload, "lattice": f"{w['L1']}x{w['L2']}", "D": w["D"],
                   "sectors": w["sectors"], "Dcut": w["cut"], "precision": args.precision, "chains_per_gpu": B,
                   "thermalisation_sweeps": w["therm"], "parallelism": f"replicas{world}",
                   "l2": "working set larger than L2 (per-chain scratch slots)"},
        "raw_samples_per_s": raw,
        "tau_int": tau,
        "energy_per_site": e_site[0],
        "energy_error": e_site[1],
        "acceptance": float(scal[7]) / max(1.0, float(scal[0])),
        "thermalisation_s": therm_s,
        "e2e": {"value": e2e_raw / (2 * tau), "unit": "effective samples/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps,
        "roofline": {"bound": bound, "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
                     "frac": achieved / peak if peak else None, "peak_source": peak_src,
                     "dram_gbs": dram_gbs, "dram_frac_of_measured_hbm": dram_frac,
                     "flops_per_launch": float(flops.sum()) / args.steps,
                     "flops_split": {"contract": flops[0] / args.steps, "qr": flops[1] / args.steps,
                                     "svd": flops[2] / args.steps, "strip": flops[3] / args.steps},
                     "traffic": traffic,
                     "traffic_source": "ncu capture of the same workload (per launch, scaled by chains)" if traffic else None,
                     "phase_cycle_share": phase_share(cycles)},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "fp64_check": fp64_check,
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
    vals = []
    for _ in range(args.steps):
        c = cpu_baseline(args.workload, per_step)
        total += c["samples"]
        secs += c["seconds"]
        vals.append(c["samples"] / c["seconds"])
        if c["tau"]:
            taus.append(c["tau"])
    tau = float(np.mean(taus)) if taus else 0.5
    raw = total / secs
    value = raw / (2 * tau)
    cores = min(os.cpu_count() or 1, 16)
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
                         "sample": f"{total} samples over {args.steps} steps of {per_step:.0f} s, one chain per "
                                   "single-threaded process (the reference itself is not installable on the GPU box)"},
        "e2e": {"value": value, "unit": "effective samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out, default=_jsonable))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="timed steps (default: per workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="", choices=["", "fp64", "dd", "fp32", "mixed"], help="default: per workload")
    ap.add_argument("--chains", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick-therm", action="store_true")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    args.steps = args.steps or w["steps"]
    args.precision = args.precision or w["precision"]
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
