#!/usr/bin/env python
"""GFN2-xTB single-point throughput on GB300 (plain per-molecule FP64 GPU path).

One step = one complete single point (EEQ guess, integrals, SCC to convergence,
energy + Mulliken charges + analytic gradient) of the seeded (H2O)_300 cluster
(900 atoms, 1800 AOs) through the engine's C ABI.  Prints one JSON line.

  value : single points/s from the device time of each step (CUDA events on the
          engine stream, summed over the timed steps)
  e2e   : single points/s wall clock through xtb_singlepoint with host buffers
          (geometry in, energy/gradient/charges out, all copies inside the timing)

--impl reference times the CPU restatement of the reference (oracle/, NumPy +
SciPy LAPACK on all host cores) on the same workload, one single point per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (generator, description)
    "h2o300": (lambda: __import__("xtb_gb300.workloads", fromlist=["w"]).water_cluster(300, seed=1),
               "(H2O)300 seeded water cluster, 900 atoms, 1800 AOs, plain FP64 GPU single point"),
    "c10h22": (lambda: __import__("xtb_gb300.workloads", fromlist=["w"]).alkane(10, 0.02, seed=1),
               "C10H22 seeded n-decane, 32 atoms, 62 AOs, plain FP64 GPU single point"),
}

PHASES = ("setup", "integrals", "cholesky", "hbuild", "stdform", "sytrd", "trieig", "backtransform", "density",
          "popmix", "gradient", "total")


def flop_model(nao, nocc):
    """Algorithmic FP64 flops per SCC iteration and phase (dense kernels as executed)."""
    n3 = float(nao) ** 3
    return {"stdform": 4.0 * n3, "sytrd": 4.0 / 3.0 * n3, "backtransform": 4.0 * n3, "density": 2.0 * n3}


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

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
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

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


def dist_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def run_gpu(args, ws, rank):
    import numpy as np

    from xtb_gb300 import interface as X

    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    Z, xyz = WORKLOADS[args.workload][0]()
    lib = X.load_library()
    calc = X.Calculator(Z, xyz, keep_orbitals=False)
    for _ in range(args.warmup):
        r = calc.singlepoint()
    nao, nocc = r.nao, int(round(np.sum(r.focc) / 2))
    iters = r.iterations
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
    value = ws * args.steps / dev_s
    e2e = ws * args.steps / wall_s
    # roofline of the dominant FP64 phase
    per_step = phase / args.steps
    fl = flop_model(nao, nocc)
    dom = max(fl, key=lambda k: per_step[PHASES.index(k)])
    dom_ms = per_step[PHASES.index(dom)]
    achieved = fl[dom] * iters / (dom_ms * 1e-3) / 1e12
    peak = lib.xtbgb_fp64PeakTflops()
    out = {
        "metric": "GFN2-xTB single points/s (energy + Mulliken charges + gradient), plain FP64 GPU SCC",
        "value": value,
        "unit": "single points/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generator, no public suite exists for this path)",
        "config": {"workload": WORKLOADS[args.workload][1], "atoms": int(len(Z)), "nao": int(nao),
                   "scc_iterations": int(iters), "parallelism": f"replicas x{ws}",
                   "l2": "working set > L2 (n^2 matrices of ~26 MB each), no flush needed"},
        "e2e": {"value": e2e, "unit": "single points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "phase_ms_per_step": {k: round(float(v), 3) for k, v in zip(PHASES, per_step)},
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "peak_source": "measured FP64 FMA probe on this GPU (MEASURED_PEAKS.json has no FP64 figure)"},
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
    return out


def cpu_baseline(args):
    """Oracle (CPU restatement, NumPy/SciPy LAPACK, all host threads) on one step of the workload."""
    from oracle import gfn2
    Z, xyz = WORKLOADS[args.cpu_workload or args.workload][0]()
    t0 = time.perf_counter()
    r = gfn2.singlepoint(Z, xyz)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "single points/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"one full single point of {args.cpu_workload or args.workload} ({len(Z)} atoms, "
                      f"{r.iterations} SCC iterations) in {dt:.1f} s"}


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    from oracle import gfn2
    Z, xyz = WORKLOADS[args.workload][0]()
    for _ in range(min(args.warmup, 1)):
        gfn2.singlepoint(Z, xyz)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        gfn2.singlepoint(Z, xyz)
        times.append(time.perf_counter() - t0)
    value = args.steps / sum(times)
    return {"metric": "GFN2-xTB single points/s (energy + Mulliken charges + gradient), plain FP64 GPU SCC",
            "impl": "reference", "value": value, "unit": "single points/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload][1], "atoms": len(Z)},
            "cpu_baseline": {"value": value, "unit": "single points/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{args.steps} full single points on the CPU restatement"},
            "e2e": {"value": value, "unit": "single points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="h2o300", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-workload", default=None, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    ws, rank, _ = dist_setup()
    out = run_reference(args, ws, rank) if args.impl == "reference" else run_gpu(args, ws, rank)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
