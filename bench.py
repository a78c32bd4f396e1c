#!/usr/bin/env python
"""GFN2-xTB single points/s on GB300: served (continuous batching) vs plain GPU SCC.

Workloads (``--workload``):

  served   (default) the seeded request stream of the served benchmark: atom counts
           log-uniform in 3..1500 (alkanes and water clusters, 1/2 each), gradient
           requested with probability 1/2.  One step = one pass of the stream through the
           request loop (xtbgb_serverSubmit / xtbgb_serverWait).  Besides the served
           throughput the line carries p50/p99 latency and the plain per-molecule GPU path
           timed on the same requests in the same run, with the largest energy, charge and
           gradient difference between the two.
  h2o300   plain FP64 single point of the seeded (H2O)300 cluster (900 atoms, 1800 AOs).
  batch4096 one launch set of the batched engine over 4096 seeded molecules (alkanes
           C1..C20, water clusters 2..30).
  split_c200h402 / split_h2o1000  split-precision products vs the FP64 mode.

``value`` counts device-side time (for served: from the first request's start on the
device to the last completion); ``e2e`` is wall clock through the C ABI with host buffers
(geometry in, energy/gradient/charges out, every copy inside the timing).

``--impl reference`` times the reference's CPU algorithm on the host cores: the C++/OpenMP +
LAPACK restatement of the oracle (oracle/twin.cpp, pinned to the reference's known-answer
tests and to the oracle fixtures), over the same requests as the GPU arm.  The K timed steps
split the workload between them, so the run covers every request once.

The default line also carries, under ``configs``, the three single-GPU configurations beside
the served stream: the (H2O)300 plain FP64 single point, the 4096-molecule batched set and the
C200H402 split-precision single point, each with its own timing, parity and clocks.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# the headline metric, word for word in both arms
SERVED_METRIC = "single points/s + p99 latency, served vs plain GPU SCC, at |ΔE|≤1e-6 Eh"
METRIC = "GFN2-xTB single points/s (energy + Mulliken charges + gradient on request)"
PHASES = ("setup", "integrals", "cholesky", "hbuild", "stdform", "sytrd", "trieig", "backtransform", "density",
          "popmix", "gradient", "total")
# DRAM bytes per matrix element of one tridiagonalisation launch; traffic grows as n^2.
# Row form k_sytrd: ncu capture of the (H2O)300 single point (26.43 MB read + 4.47 MB written,
# n = 1800).  Upper-triangle form k_sytrd_sym: ncu capture at n = 3072 with the 16 x 64 tiles
# and 512 threads per block it runs from 1800 AOs (39.33 MB read + 242.39 MB written).
SYTRD_BYTES_PER_ELEM = (26.430976e6 + 4.467968e6) / 1800.0 ** 2
SYTRD_SYM_BYTES_PER_ELEM = (39.325952e6 + 242.387968e6) / 3072.0 ** 2


def sytrd_form(n):
    """(kernel, DRAM bytes per launch, note) of the tridiagonalisation the engine runs at n AOs on
    this device (the autotuner's crossover)."""
    from xtb_gb300 import interface as X
    if n >= X.get_tuning()["sytrd_sym_min"]:
        return "k_sytrd_sym", SYTRD_SYM_BYTES_PER_ELEM * float(n) ** 2, "traffic scaled as n^2 from the ncu capture at n = 3072"
    return "k_sytrd", SYTRD_BYTES_PER_ELEM * float(n) ** 2, "traffic scaled as n^2 from the ncu capture at n = 1800"


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        cmd = ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    return ws, rank, local


def dist_init(ws):
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")


def dist_max(x, ws):
    """Max of x over the replicas (the slowest rank sets the whole job's time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, seconds, ws):
    """Whole-job throughput of `ws` independent replicas: all units over the slowest rank's time."""
    return ws * units_per_rank / dist_max(seconds, ws)


def dist_barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def host_info():
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if not model:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.startswith("Model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    return f"{model or 'unknown CPU'} ({platform.machine()}, {os.cpu_count()} cores)"


def stream_requests(args):
    from xtb_gb300 import workloads as W
    return W.served_stream(args.requests, seed=args.seed, rate=args.rate)


def sp_flops(nao, nocc, iters):
    """Algorithmic FP64 flops of one single point's SCC: per iteration n^3 (standard form)
    + 4/3 n^3 (tridiagonalisation) + 2 n^3 (back-transformation) + n^3 (triangular solve)
    + 2 n^2 k (density)."""
    n = float(nao)
    return iters * ((16.0 / 3.0) * n ** 3 + 2.0 * n * n * nocc)


_PEAK = None


def fp64_peak(lib):
    """Roofline denominator for the FP64 kernels: the largest of two FMA-throughput probes and
    the engine's own FP64 GEMM at 4096^3, measured once per process on this GPU
    (MEASURED_PEAKS.json holds no FP64 figure)."""
    global _PEAK
    if _PEAK is None:
        import ctypes as C
        d = np.zeros(3)
        lib.xtbgb_fp64PeakDetail(d.ctypes.data_as(C.POINTER(C.c_double)))
        _PEAK = (float(np.max(d)), {"fma_probe": float(d[0]), "accumulator_probe": float(d[1]),
                                    "fp64_gemm_4096": float(d[2]),
                                    "source": "measured on this GPU in this run: the largest of the three"})
    return _PEAK


# ------------------------------------------------------------------ workloads, named once for both arms
PLAIN_WORKLOADS = {
    "h2o300": ("(H2O)300 seeded water cluster, 900 atoms, 1800 AOs, plain FP64 GPU single point",
               lambda W: W.water_cluster(300, seed=1)),
    "h2o1000": ("(H2O)1000 seeded water cluster, 3000 atoms, 6000 AOs, plain FP64 GPU single point",
                lambda W: W.water_cluster(1000, seed=1)),
    "c200h402": ("all-trans C200H402, sigma 0.02 A jitter, 602 atoms, 1202 AOs, plain FP64 GPU single point",
                 lambda W: W.alkane(200, 0.02, seed=1)),
}
SPLIT_WORKLOADS = {
    "split_c200h402": ("all-trans C200H402 (602 atoms, 1202 AOs), split-precision products vs FP64",
                       lambda W: W.alkane(200, 0.02, seed=1)),
    "split_h2o1000": ("(H2O)1000 seeded water cluster (3000 atoms, 6000 AOs), split-precision products vs FP64",
                      lambda W: W.water_cluster(1000, seed=1)),
}
BATCH_DESC = "4096 molecules: 2048 alkanes C_nH_2n+2 n~U{1..20}, 2048 water clusters m~U{2..30}, seed 7"


def served_desc(args):
    return (f"served stream: {args.requests} requests, atoms log-uniform 3..1500 (alkanes C_nH_2n+2 and "
            f"(H2O)_m, 1/2 each), gradient on 1/2, neutral, T_el 300 K, seed {args.seed}")


def workload_spec(args):
    """(metric, config.workload) of the selected workload: the same strings in both arms."""
    if args.workload == "served":
        return SERVED_METRIC, served_desc(args)
    if args.workload == "batch4096":
        return METRIC + ", batched engine (one thread block per molecule) vs plain GPU SCC", BATCH_DESC
    if args.workload in SPLIT_WORKLOADS:
        return METRIC + ", split-precision products (BF16 tensor cores) vs FP64", SPLIT_WORKLOADS[args.workload][0]
    return METRIC + ", plain FP64 GPU SCC", PLAIN_WORKLOADS[args.workload][0]


def workload_requests(args):
    """The workload as a list of requests (numbers, positions, gradient)."""
    from xtb_gb300 import workloads as W
    if args.workload == "served":
        return stream_requests(args)
    if args.workload == "batch4096":
        return [{"numbers": z, "positions": x, "gradient": True} for z, x in W.mixed_batch(4096, seed=7)]
    gen = (SPLIT_WORKLOADS.get(args.workload) or PLAIN_WORKLOADS[args.workload])[1]
    Z, xyz = gen(W)
    return [{"numbers": Z, "positions": xyz, "gradient": True}]


# ------------------------------------------------------------------ served stream
def served_pass(srv, reqs, rate):
    t0 = time.perf_counter()
    ids = []
    for r in reqs:
        if rate:
            delay = t0 + r["arrival"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
        ids.append(srv.submit(r["numbers"], r["positions"], gradient=r["gradient"]))
    res = [srv.wait(i, check=False) for i in ids]
    wall = time.perf_counter() - t0
    span = max(x.t_done for x in res) - min(x.t_start for x in res)
    return res, wall, span


def autotune_served(args, reqs):
    """The engine's autotuner, before any timing: the kernel-form crossovers of this device, then
    the request loop's schedule on this stream (unless given on the command line)."""
    from xtb_gb300 import tuning
    forms = device_forms(args)
    out = {"kernel_forms": forms}
    if args.workers is None or args.iters_per_step is None or args.pool_max_nao is None or args.coop_blocks is None:
        sched = tuning.schedule(reqs, pool_gib=args.pool_gib, precision=args.served_precision, slices=args.slices)
        out["schedule"] = sched
        if args.workers is None:
            args.workers = sched["plain_workers"]
        if args.iters_per_step is None:
            args.iters_per_step = sched["iters_per_step"]
        if args.pool_max_nao is None:
            args.pool_max_nao = sched["pool_max_nao"]
        if args.coop_blocks is None:
            args.coop_blocks = sched["coop_blocks"]
    return out


def device_forms(args):
    """The device's kernel-form choices: measured by the autotuner, or pinned with --forms
    (sytrd_sym_min,blocked_min_fp64,blocked_min_split), e.g. to repeat a measured run's choices
    under a profiler, whose per-launch overhead would skew the tuner's timings."""
    from xtb_gb300 import interface as X
    if args.forms:
        sym, fp64, split = (int(v) for v in args.forms.split(","))
        X.set_tuning(sym, fp64, split)
        return X.get_tuning()
    return X.autotune()


def run_served(args, ws, rank):
    from xtb_gb300 import interface as X
    lib = X.load_library()
    reqs = stream_requests(args)
    R = len(reqs)
    metric, wdesc = workload_spec(args)
    tuned = autotune_served(args, reqs)
    srv = X.Server(pool_gib=args.pool_gib, max_slots=1024, plain_workers=args.workers,
                   iters_per_step=args.iters_per_step, precision=args.served_precision, slices=args.slices,
                   pool_max_nao=args.pool_max_nao, coop_blocks=args.coop_blocks)
    for _ in range(args.warmup):
        served_pass(srv, reqs, args.rate)
    st0 = srv.stats()
    dist_barrier(ws)
    clocks = ClockSampler(0)
    clocks.start()
    passes = [served_pass(srv, reqs, args.rate) for _ in range(args.steps)]
    dist_barrier(ws)
    clk = clocks.stop()
    st1 = srv.stats()
    # the same requests once more with Poisson arrivals at 80% of the measured saturation
    # throughput (arrival times from their own seeded generator, so the molecules are the same):
    # throughput and latency under load below capacity, next to the capacity itself
    poisson = None
    if not args.rate:
        sat = sum(len(p[0]) for p in passes) / max(1e-9, sum(p[2] for p in passes))
        prate = 0.8 * sat
        arr = np.cumsum(np.random.default_rng(args.seed + 1).exponential(1.0 / prate, R)) - 1.0 / prate
        preqs = [dict(r, arrival=float(a)) for r, a in zip(reqs, arr)]
        pres, pwall, _ = served_pass(srv, preqs, prate)
        plat = np.array([x.latency for x in pres]) * 1e3
        poisson = {"rate": prate, "value": R / pwall, "unit": "single points/s",
                   "latency_ms": {"p50": float(np.percentile(plat, 50)), "p99": float(np.percentile(plat, 99)),
                                  "max": float(plat.max())},
                   "failed_requests": int(sum(1 for x in pres if x.status != 0)),
                   "note": "one pass, arrivals exponential at 0.8x the saturation throughput"}
    srv.close()
    span = dist_max(sum(p[2] for p in passes), ws)
    wall = dist_max(sum(p[1] for p in passes), ws)
    if rank != 0:
        return None
    d = {k: st1[k] - st0[k] for k in st1}
    lat = np.array([x.latency for p in passes for x in p[0]]) * 1e3
    served = passes[-1][0]
    bad = [x for p in passes for x in p[0] if x.status != 0]
    # plain per-molecule GPU path on the same requests (sequential, one process, one stream)
    plain_wall, plain_dev = 0.0, 0.0
    dE = dq = dg = 0.0
    iters_diff = 0
    plain = []
    for r, s in zip(reqs, served):
        t1 = time.perf_counter()
        p = X.Calculator(r["numbers"], r["positions"], keep_orbitals=False).singlepoint()
        plain_wall += time.perf_counter() - t1
        plain_dev += p.phase_ms[-1] / 1e3
        plain.append(p)
        dE = max(dE, abs(s.energy - p.energy))
        dq = max(dq, float(np.max(np.abs(s.charges - p.charges))))
        if r["gradient"]:
            dg = max(dg, float(np.max(np.abs(s.gradient - p.gradient))))
        iters_diff = max(iters_diff, abs(s.iterations - p.iterations))
    peak, peak_detail = fp64_peak(lib)
    # Roofline of the dominant kernel, the FP64 tridiagonalisation, from the sequential plain
    # pass: one request at a time, so its CUDA-event time is the kernel's own, not time spent
    # queued behind concurrent requests.  Taken on the largest request (the one that sets the
    # served makespan); 4/3 n^3 algorithmic flops per launch, one launch per SCC iteration.
    big = max(plain, key=lambda p: p.nao)
    sy_ms = big.phase_ms[PHASES.index("sytrd")] / big.iterations
    ach = (4.0 / 3.0) * float(big.nao) ** 3 / (sy_ms * 1e-3) / 1e12
    # the same kernel inside the served timed region (concurrent requests share the SMs, so
    # these event times include queueing) and the pool's SCC kernel
    plain_res = [x for p in passes for x in p[0] if x.engine == 1]
    ssy_ms = sum(x.sytrd_ms for x in plain_res)
    ssy_flops = sum((4.0 / 3.0) * float(x.nao) ** 3 * x.iterations for x in plain_res)
    pool_ms, pool_flops = d["pool_scc_ms"], d["pool_scc_flops"]
    served_kernels = {
        "k_batch_scc": {"device_ms": round(pool_ms, 2), "tflops": (pool_flops / (pool_ms * 1e-3) / 1e12)
                        if pool_ms > 0 else None, "launches": int(d["steps"])},
        "tridiagonalisation": {"kernels": sorted({sytrd_form(x.nao)[0] for x in plain_res}),
                               "device_ms": round(ssy_ms, 2), "tflops": (ssy_flops / (ssy_ms * 1e-3) / 1e12)
                               if ssy_ms > 0 else None, "launches": int(sum(x.iterations for x in plain_res))},
        "note": "CUDA-event times inside the served timed region, summed over concurrent requests "
                "(they overlap, and include time queued behind other requests' kernels)",
    }
    fp64_flops = sum((7.0 / 3.0) * float(x.nao) ** 3 * x.iterations for x in plain_res) + pool_flops
    fp64_job = fp64_flops / span / 1e12 if span > 0 else None   # rank 0 against one GPU
    out = {
        "metric": metric,
        "value": ws * args.steps * R / span,
        "unit": "single points/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * span / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded request stream; no public suite exists for this path)",
        "config": {"workload": wdesc,
                   "arrival": f"Poisson {args.rate}/s" if args.rate else "all requests at t=0 (saturation)",
                   "served_precision": (f"split products ({args.slices} bf16 digits) on the plain-engine workers"
                                        if args.served_precision == "split" else "fp64"),
                   "pool_gib": args.pool_gib, "plain_workers": args.workers, "iters_per_step": args.iters_per_step,
                   "pool_max_nao": args.pool_max_nao, "coop_blocks": args.coop_blocks,
                   "parallelism": f"replicas x{ws}",
                   "l2": "large requests hold n^2 matrices far above L2 (129 MB); no flush"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max())},
        "plain": {"value": R / plain_dev, "e2e": R / plain_wall, "unit": "single points/s",
                  "path": "xtb_singlepoint per request, one after another"},
        "speedup_vs_plain": (ws * args.steps * R / wall) / (R / plain_wall),
        "parity_vs_plain": {"max_abs_dE": dE, "max_abs_dq": dq, "max_abs_dg": dg, "max_iter_diff": iters_diff,
                            "failed_requests": len(bad),
                            "errors": sorted({f"nao {x.nao}: {x.error}" for x in bad})[:5]},
        "e2e": {"value": ws * args.steps * R / wall, "unit": "single points/s",
                "h2d_bytes_per_step": int(d["h2d_bytes"] / args.steps),
                "d2h_bytes_per_step": int(d["d2h_bytes"] / args.steps)},
        "gpu_launches": int(d["launches"]),
        "poisson": poisson,
        "served_mix": {"pool": int(sum(1 for x in served if x.engine == 0)),
                       "plain_engine": int(sum(1 for x in served if x.engine == 1)),
                       "peak_resident": int(st1["peak_resident"])},
        "served_kernels": served_kernels,
        "autotune": tuned,
        "roofline": {"bound": "fp64", "kernel": sytrd_form(big.nao)[0], "achieved": ach, "peak": peak,
                     "unit": "TFLOP/s", "frac": ach / peak if peak else None,
                     "traffic": sytrd_form(big.nao)[1], "traffic_unit": "bytes per launch",
                     "launch_ms": sy_ms, "nao": int(big.nao), "launches": int(big.iterations),
                     "note": "4/3 n^3 FP64 flops per launch / CUDA-event time per launch, largest request of the "
                             "stream in the sequential plain pass (no concurrent work); " + sytrd_form(big.nao)[2],
                     "peak_detail": peak_detail},
        # the whole run against the FP64 pipe: FP64-only algorithmic work of all requests (plain
        # engine: standard form n^3 + tridiagonal reduction 4/3 n^3 per SCC iteration, the counts
        # of LAPACK's dsygst and dsytrd; pool: its counted SCC flops) over the span
        "fp64_job": {"achieved": fp64_job, "peak": peak, "unit": "TFLOP/s",
                     "frac": (fp64_job / peak) if peak else None,
                     "note": "FP64-only algorithmic flops of every request / served span (split-precision "
                             "products on the tensor cores not counted)"},
        "clocks": clk,
    }
    if not args.no_configs and ws == 1:
        out["configs"] = run_configs(args)
    if not args.no_cpu_baseline and ws == 1:
        out["cpu_baseline"] = cpu_baseline(args, reqs)
    return out


def run_configs(args):
    """The three other single-GPU configurations, timed after the served passes, each with
    its own steps, timing, parity and clocks (3 timed steps after 3 warm-up steps)."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.no_cpu_baseline = 3, 3, True
    keep = ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config", "e2e", "gpu_launches",
            "parity", "error_vs_fp64", "fp64_mode", "plain", "roofline", "phase_ms_per_step", "clocks")
    out = {}
    for name, fn in (("h2o300", run_plain), ("batch4096", run_batch), ("split_c200h402", run_split)):
        sub.workload = name
        r = fn(sub, 1, 0)
        out[name] = {k: r[k] for k in keep if k in r}
    return out


# ------------------------------------------------------------------ plain single point
def fixture_parity(name, res):
    """Largest differences of a GPU result against the committed oracle fixture of the geometry."""
    path = os.path.join(ROOT, "tests", "golden", f"{name}.npz")
    if not name or not os.path.exists(path):
        return None
    f = np.load(path)
    return {"vs": f"oracle fixture tests/golden/{name}.npz", "abs_dE": abs(res.energy - float(f["energy"])),
            "max_abs_dq": float(np.max(np.abs(res.charges - f["charges"]))),
            "max_abs_dg": float(np.max(np.abs(res.gradient - f["gradient"]))),
            "iterations": [int(res.iterations), int(f["iterations"])]}


def run_plain(args, ws, rank):
    from xtb_gb300 import interface as X
    from xtb_gb300 import workloads as W
    metric, desc = workload_spec(args)
    Z, xyz = PLAIN_WORKLOADS[args.workload][1](W)
    lib = X.load_library()
    device_forms(args)    # the device's kernel forms, as the served run and the engine use them
    calc = X.Calculator(Z, xyz, keep_orbitals=False)
    for _ in range(args.warmup):
        r = calc.singlepoint()
    nao, nocc, iters = r.nao, int(round(np.sum(r.focc) / 2)), r.iterations
    dist_barrier(ws)
    clocks = ClockSampler(0)
    clocks.start()
    dev_ms, wall, phase = [], [], np.zeros(len(PHASES))
    h2d = d2h = launches = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = calc.singlepoint()            # host geometry in; energy, gradient, charges copied out
        wall.append(time.perf_counter() - t0)
        dev_ms.append(r.phase_ms[-1])
        phase += r.phase_ms
        h2d, d2h = r.h2d_bytes, r.d2h_bytes
        launches += r.launches
    dist_barrier(ws)
    clk = clocks.stop()
    dev_s = dist_max(sum(dev_ms) / 1e3, ws)
    wall_s = dist_max(sum(wall), ws)
    if rank != 0:
        return None
    per_step = phase / args.steps
    sy_ms = per_step[PHASES.index("sytrd")] / iters
    ach = (4.0 / 3.0) * float(nao) ** 3 / (sy_ms * 1e-3) / 1e12
    peak, peak_detail = fp64_peak(lib)
    out = {
        "metric": metric,
        "value": ws * args.steps / dev_s, "unit": "single points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, no public suite exists for this path)",
        "config": {"workload": desc,
                   "atoms": int(len(Z)), "nao": int(nao), "scc_iterations": int(iters),
                   "parallelism": f"replicas x{ws}",
                   "l2": f"working set > L2 (n^2 matrices of {8 * nao * nao / 1e6:.0f} MB each), no flush needed"},
        "e2e": {"value": ws * args.steps / wall_s, "unit": "single points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "parity": fixture_parity({"h2o300": "h2o_300_seed1"}.get(args.workload, ""), r),
        "phase_ms_per_step": {k: round(float(v), 3) for k, v in zip(PHASES, per_step)},
        "algorithmic_tflops_per_sp": sp_flops(nao, nocc, iters) / 1e12,
        "roofline": {"bound": "fp64", "kernel": sytrd_form(nao)[0], "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                     "frac": ach / peak if peak else None, "launch_ms": sy_ms,
                     "traffic": sytrd_form(nao)[1], "traffic_unit": "bytes per launch",
                     "note": "4/3 n^3 FP64 flops per launch / CUDA-event time per launch; " + sytrd_form(nao)[2],
                     "peak_detail": peak_detail},
        "clocks": clk,
    }
    if not args.no_cpu_baseline and ws == 1:
        out["cpu_baseline"] = cpu_baseline(args, workload_requests(args))
    return out


# ------------------------------------------------------------------ split precision vs FP64
def run_split(args, ws, rank):
    """Split-precision mode (back-transformation, P and W as BF16 tensor-core digit products) timed
    over `steps` single points; the FP64 mode on the same molecule gives the reference for the
    per-result errors |dE|, max |dq|, max |dg| and ||dP||_F / ||P||_F."""
    from xtb_gb300 import interface as X
    from xtb_gb300 import workloads as W
    metric, desc = workload_spec(args)
    Z, xyz = SPLIT_WORKLOADS[args.workload][1](W)
    lib = X.load_library()
    device_forms(args)    # the device's kernel forms, as the served run and the engine use them
    cs = X.Calculator(Z, xyz, keep_orbitals=False, precision="split", slices=args.slices)
    for _ in range(args.warmup):
        r = cs.singlepoint()
    dist_barrier(ws)
    clocks = ClockSampler(0)
    clocks.start()
    dev, wall = 0.0, 0.0
    phase = np.zeros(len(PHASES))
    launches = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = cs.singlepoint()
        wall += time.perf_counter() - t0
        dev += r.phase_ms[-1] / 1e3
        phase += r.phase_ms
        launches += r.launches
    dist_barrier(ws)
    clk = clocks.stop()
    dev = dist_max(dev, ws)
    wall = dist_max(wall, ws)
    if rank != 0:
        return None
    # FP64 mode and both densities (orbitals kept) for the error report

    def density(calc, res):
        """P = sum_j f_j c_j c_j^T from xtb_getOrbitalCoefficients (rows = orbitals)."""
        import ctypes as C
        nn = res.nao
        c = np.zeros((nn, nn))
        calc.lib.xtb_getOrbitalCoefficients(calc.env.h, calc.res, c.ctypes.data_as(C.POINTER(C.c_double)))
        calc.env.check()
        return (c.T * res.focc) @ c

    cf = X.Calculator(Z, xyz, keep_orbitals=True)
    f = cf.singlepoint()
    csp = X.Calculator(Z, xyz, keep_orbitals=True, precision="split", slices=args.slices)
    s = csp.singlepoint()
    Pf, Ps = density(cf, f), density(csp, s)
    err = {"max_abs_dE": abs(s.energy - f.energy), "max_abs_dq": float(np.max(np.abs(s.charges - f.charges))),
           "max_abs_dg": float(np.max(np.abs(s.gradient - f.gradient))), "iterations": [f.iterations, s.iterations],
           "rel_frobenius_dP": float(np.linalg.norm(Ps - Pf) / np.linalg.norm(Pf))}
    per = phase / args.steps
    peak, peak_detail = fp64_peak(lib)
    n = r.nao
    sy = per[PHASES.index("sytrd")] / r.iterations
    ach = (4.0 / 3.0) * float(n) ** 3 / (sy * 1e-3) / 1e12
    return {
        "metric": metric,
        "value": ws * args.steps / dev, "unit": "single points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": f"f64 (products: bf16 digits x{args.slices}, fp32 accumulate)",
        "data": "synthetic (seeded generator)",
        "config": {"workload": desc, "atoms": int(len(Z)), "nao": int(n), "slices": args.slices,
                   "parallelism": f"replicas x{ws}", "l2": "n^2 matrices above L2; no flush"},
        "fp64_mode": {"value": 1e3 / f.phase_ms[-1], "unit": "single points/s"},
        "error_vs_fp64": err,
        "e2e": {"value": ws * args.steps / wall, "unit": "single points/s", "h2d_bytes_per_step": int(r.h2d_bytes),
                "d2h_bytes_per_step": int(r.d2h_bytes)},
        "gpu_launches": int(launches),
        "phase_ms_per_step": {k: round(float(v), 3) for k, v in zip(PHASES, per)},
        "roofline": {"bound": "fp64", "kernel": sytrd_form(n)[0], "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                     "frac": ach / peak if peak else None, "launch_ms": sy,
                     "traffic": sytrd_form(n)[1], "traffic_unit": "bytes per launch",
                     "note": "the tridiagonalisation stays FP64 and dominates; split products are C = X Z, "
                             "the density and the energy-weighted density (the back-transformation takes "
                             "the tuned form: FP64 column strips below the split chain's crossover)",
                     "peak_detail": peak_detail},
        "clocks": clk,
    }


# ------------------------------------------------------------------ batched 4096
def run_batch(args, ws, rank):
    from xtb_gb300 import interface as X
    from xtb_gb300 import workloads as W
    metric, desc = workload_spec(args)
    mols = W.mixed_batch(4096, seed=7)
    lib = X.load_library()
    b = X.Batch(mols)
    for _ in range(args.warmup):
        r = b.run(check=False)
    dist_barrier(ws)
    clocks = ClockSampler(0)
    clocks.start()
    runs = [b.run(check=False) for _ in range(args.steps)]
    dist_barrier(ws)
    clk = clocks.stop()
    dev = dist_max(sum(x.device_ms for x in runs) / 1e3, ws)
    wall = dist_max(sum(x.wall_ms for x in runs) / 1e3, ws)
    if rank != 0:
        return None
    r = runs[-1]
    flops = sum(sp_flops(b.nao[i], b.nao[i] // 2, r.iterations[i]) for i in range(len(mols)))
    ach = flops / (r.device_ms * 1e-3) / 1e12
    peak, peak_detail = fp64_peak(lib)
    idx = np.random.default_rng(0).choice(len(mols), 32, replace=False)
    pw = pd = 0.0
    dE = 0.0
    for i in idx:
        t0 = time.perf_counter()
        p = X.Calculator(*mols[i], keep_orbitals=False).singlepoint()
        pw += time.perf_counter() - t0
        pd += p.phase_ms[-1] / 1e3
        dE = max(dE, abs(p.energy - r.energy[i]))
    n = len(mols)
    out = {
        "metric": metric,
        "value": ws * args.steps * n / dev, "unit": "single points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators)",
        "config": {"workload": desc, "nao_mean": float(np.mean(b.nao)), "nao_max": int(np.max(b.nao)),
                   "parallelism": f"replicas x{ws}", "l2": "6+ GB resident state, far above L2; no flush"},
        "e2e": {"value": ws * args.steps * n / wall, "unit": "single points/s",
                "h2d_bytes_per_step": int(r.h2d_bytes), "d2h_bytes_per_step": int(r.d2h_bytes)},
        "gpu_launches": int(sum(x.launches for x in runs)),
        "plain": {"value": len(idx) / pd, "e2e": len(idx) / pw, "unit": "single points/s",
                  "sample": "32 random molecules of the set, xtb_singlepoint one after another"},
        "parity": {"vs": "plain engine on 32 random molecules of the set", "max_abs_dE": dE,
                   "failed": int(np.sum(r.status != 0))},
        "roofline": {"bound": "fp64", "kernel": "batched step (all kernels)", "achieved": ach, "peak": peak,
                     "unit": "TFLOP/s", "frac": ach / peak if peak else None, "traffic": None,
                     "note": "algorithmic FP64 flops of all SCC iterations / CUDA-event time of the launch set",
                     "peak_detail": peak_detail},
        "clocks": clk,
    }
    if not args.no_cpu_baseline and ws == 1:
        out["cpu_baseline"] = cpu_baseline(args, workload_requests(args))
    return out


# ------------------------------------------------------------------ CPU: the reference's algorithm
def blas_info():
    try:
        import scipy
        b = scipy.show_config(mode="dicts")["Build Dependencies"]["lapack"]
        return f"{b.get('name')} {b.get('version')}"
    except Exception:   # noqa: BLE001 -- a description only
        return "SciPy's bundled OpenBLAS"


def cpu_threads():
    return int(os.environ.get("OMP_NUM_THREADS", "0") or 0) or os.cpu_count()


def twin_run(reqs):
    """The C++/OpenMP + LAPACK restatement on `reqs`, one after another; (seconds, count)."""
    from oracle import twin
    spent = 0.0
    for r in reqs:
        t0 = time.perf_counter()
        twin.singlepoint(np.asarray(r["numbers"]), np.asarray(r["positions"], dtype=float))
        spent += time.perf_counter() - t0
    return spent, len(reqs)


def cpu_desc(sample):
    return (f"{sample}; C++/OpenMP restatement of the reference's algorithm (oracle/twin.cpp: dpotrf once, "
            f"dsygst + dsyevd + dtrsm per SCC iteration, the density as a full dgemm, OpenMP loops elsewhere) with "
            f"{cpu_threads()} OpenMP threads and {blas_info()} on all cores of {host_info()}; the reference binary "
            "itself cannot be built here (no Fortran compiler, no meson)")


def cpu_baseline(args, reqs):
    """The reference's CPU algorithm on the same requests as the GPU arm, each once."""
    from oracle import twin
    twin.build()
    twin.singlepoint(np.asarray(reqs[0]["numbers"]), np.asarray(reqs[0]["positions"], dtype=float))   # load
    if args.workload == "batch4096":
        reqs = reqs[:args.cpu_batch_sample]
        what = f"the first {len(reqs)} molecules of the 4096-molecule set"
    else:
        what = "every request of the workload once"
    t, n = twin_run(reqs)
    return {"value": n / t, "unit": "single points/s", "cores": cpu_threads(), "kind": "port",
            "sample": cpu_desc(f"{n} single points ({what}) in {t:.1f} s")}


def run_reference(args, ws, rank):
    """The reference arm: the reference's CPU algorithm on the host cores, on this arm's workload.
    The K timed steps partition the workload's requests (request j goes to step j mod K), so the
    run covers every request once; warm-up steps run the smallest request."""
    if rank != 0:
        return None
    from oracle import twin
    twin.build()
    metric, wdesc = workload_spec(args)
    reqs = workload_requests(args)
    if args.workload == "batch4096":
        reqs = reqs[:args.cpu_batch_sample]
    small = min(reqs, key=lambda r: len(r["numbers"]))
    for _ in range(max(1, args.warmup)):
        twin_run([small])
    K = args.steps
    parts = [reqs[s::K] for s in range(K)] if len(reqs) >= K else [[reqs[s % len(reqs)]] for s in range(K)]
    tot_t, tot_n = 0.0, 0
    for part in parts:
        t, n = twin_run(part)
        tot_t += t
        tot_n += n
    value = tot_n / tot_t
    what = ("every request of the workload once, split over the timed steps" if args.workload != "batch4096"
            else f"the first {args.cpu_batch_sample} molecules of the 4096-molecule set")
    return {"metric": metric, "impl": "reference", "value": value, "unit": "single points/s", "n_gpus": ws,
            "steps": K, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the same seeded requests as the GPU arm)",
            "config": {"workload": wdesc},
            "cpu_baseline": {"value": value, "unit": "single points/s", "cores": cpu_threads(), "kind": "port",
                             "sample": cpu_desc(f"{tot_n} single points ({what}) in {tot_t:.1f} s")},
            "e2e": {"value": value, "unit": "single points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="served",
                    choices=["served", "batch4096"] + sorted(PLAIN_WORKLOADS) + sorted(SPLIT_WORKLOADS))
    ap.add_argument("--slices", type=int, default=5, help="split workloads: digits per operand")
    ap.add_argument("--served-precision", default="split", choices=["split", "fp64"],
                    help="served: precision of the plain-engine workers' products")
    ap.add_argument("--requests", type=int, default=64, help="served: requests per pass")
    ap.add_argument("--seed", type=int, default=11, help="served: stream seed")
    ap.add_argument("--rate", type=float, default=None, help="served: Poisson arrival rate (default: saturation)")
    ap.add_argument("--workers", type=int, default=None, help="served: plain-engine workers (default: autotuned)")
    ap.add_argument("--iters-per-step", type=int, default=None,
                    help="served: SCC iterations per pool step (default: autotuned)")
    ap.add_argument("--pool-gib", type=float, default=24.0, help="served: HBM budget of the resident pool")
    ap.add_argument("--pool-max-nao", type=int, default=None,
                    help="served: largest molecule (AOs) of the resident pool (default: autotuned)")
    ap.add_argument("--coop-blocks", type=int, default=None,
                    help="served: most blocks of a worker's cooperative tridiagonalisation, 0 = all SMs, "
                         "-D = one per D AOs of the request (default: autotuned)")
    ap.add_argument("--cpu-batch-sample", type=int, default=512,
                    help="batch4096: molecules of the set the CPU restatement runs")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forms", default=None,
                    help="pin the kernel forms instead of autotuning: sytrd_sym_min,blocked_min_fp64,blocked_min_split")
    ap.add_argument("--no-configs", action="store_true", help="served: skip the three other configurations")
    args = ap.parse_args()
    ws, rank, _ = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
    else:
        dist_init(ws)
        run = {"served": run_served, "batch4096": run_batch}.get(args.workload)
        if run is None:
            run = run_split if args.workload in SPLIT_WORKLOADS else run_plain
        out = run(args, ws, rank)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
