"""Benchmark of the GB300 RHF-CCSD amplitude engine.

Metric: CCSD seconds per iteration and TFLOP/s at no=40, nv=300 (synthetic Hamiltonian,
seed 2), mixed precision vs plain FP64 on one GB300.  A "step" is one full CCSD iteration
of ``solve_cc`` (residual + Jacobi update + energy + DIIS) on device-resident amplitudes and
integrals.  TFLOP/s uses the pinned per-iteration count of the reference formulation,
F_iter = 2 o^2 v^4 + 18 o^3 v^3 + 10 o^2 v^3 + 4 o^4 v^2.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CCSD s/iter & TFLOP/s (no=40,nv=300): mixed vs FP64 on GB300 at 1e-6 Eh"


def f_iter(o, v):
    return 2 * o**2 * v**4 + 18 * o**3 * v**3 + 10 * o**2 * v**3 + 4 * o**4 * v**2


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[3:7]):
                if val.lower() == "active":
                    reasons.add(name)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_reference(args, world, rank):
    """The reference arm: the oracle port's CCSD iteration on the host cores."""
    import numpy as np
    if rank != 0:
        return None
    from oracle import ccsd as oc
    from pycc_gb300.synth import SyntheticFactors
    ncores = os.cpu_count() or 1
    o_s, v_s, seed = 20, 180, 1
    fac = SyntheticFactors(o_s, v_s, seed)
    F, ERI, L = fac.hamiltonian()
    o, v = slice(0, o_s), slice(o_s, o_s + v_s)
    t1, t2 = oc.mp2_guess(F, ERI, o_s)
    Dia, Dijab = oc.denominators(F, o_s)
    diis = oc.DIIS(t1, t2, 8)

    def step(t1, t2):
        r1, r2 = oc.residuals(o, v, F, ERI, L, t1, t2)
        t1 = t1 + r1 / Dia
        t2 = t2 + r2 / Dijab
        oc.cc_energy(o, v, F, L, t1, t2)
        diis.add_error_vector(t1, t2)
        return diis.extrapolate(t1, t2)

    for _ in range(args.warmup):
        t1, t2 = step(t1, t2)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1, t2 = step(t1, t2)
    dt = (time.perf_counter() - t0) / args.steps
    tf = f_iter(o_s, v_s) / dt / 1e12
    return dt, tf, ncores, "oracle CCSD iteration at no=%d,nv=%d (seed %d), %d threads" % (
        o_s, v_s, seed, ncores)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no", type=int, default=40)
    ap.add_argument("--nv", type=int, default=300)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--precision", default="DP")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        res = cpu_reference(args, world, rank)
        if res is None:
            return
        dt, tf, ncores, sample = res
        line = {"metric": METRIC, "value": tf, "unit": "TFLOP/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": "RHF-CCSD iteration, synthetic Hamiltonian",
                           "no": 20, "nv": 180, "seed": 1},
                "cpu_baseline": {"value": tf, "unit": "TFLOP/s", "cores": ncores,
                                 "kind": "port", "sample": sample},
                "e2e": {"value": tf, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    import pycc_gb300 as pg
    from pycc_gb300 import _lib
    dev = torch.device("cuda:%d" % local)
    torch.cuda.set_device(dev)
    fac = pg.SyntheticFactors(args.no, args.nv, args.seed)
    t0 = time.time()
    H = pg.Hamiltonian.from_factors(fac, device=dev)
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    w = pg.CCwfn(H, precision=args.precision)
    from pycc_gb300.diis import DIIS
    diis = DIIS(w._amps, 8)
    o, v = w.o, w.v

    def step():
        r1, r2 = w.residuals(H.F, w.t1, w.t2)
        w.update_amplitudes(r1, r2)
        w.cc_energy(o, v, H.F, H.L, w.t1, w.t2)
        diis.add_error_vector(w._amps)
        w._amps.copy_(diis.extrapolate(w._amps))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    tf = f_iter(args.no, args.nv) / (ms * 1e-3) / 1e12
    line = {"metric": METRIC, "value": tf, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "DP" else "bf16", "data": "synthetic",
            "config": {"workload": "RHF-CCSD iteration, synthetic Hamiltonian", "no": args.no,
                       "nv": args.nv, "seed": args.seed, "precision": args.precision,
                       "l2": "inputs larger than L2"},
            "setup_s": setup_s, "clocks": clocks}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
