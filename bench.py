"""Benchmark: TD-CCSD RK4 steps/s on one GB300 (replicas across GPUs).

One "step" is the reference's propagation loop body (CCSD_Helper.py:1206-1240):
16 right-hand sides (block-frozen RK4 over T1, T2, L1, L2), the rounded state
update and the dipole trace.  Workload: synthetic TD-CCSD at o=10, v=38
(Q=144 seeded density-fitting integrals), dt=0.005, E(t)=0.002 sin(0.923 t).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|mixed|auto] [--workload NAME] [--method CCSD|CC2]

Prints one JSON line (rank 0).  The reference arm (--impl reference) times the
CPU oracle (the numpy restatement of the reference, all host cores) on the
same workload; the reference itself cannot be shipped to the GPU host.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CCSD RK4 steps/s (T+L RHS) mixed vs FP64 GPU at |Δμ|≤1e-8 au; grad/fwd cost"
DT, A, W0 = 0.005, 0.002, 0.923


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    p.add_argument("--workload", default="ccsd_o10_v38")
    p.add_argument("--method", default="CCSD", choices=["CCSD", "CC2"])
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def start_state(sysm):
    """MP2-guess start: t1 = 0, t2 = <ij||ab>/D, lambda = t (complex128)."""
    from python_code_to_check_c_gb300.system import mp2_guess
    t2 = mp2_guess(sysm.tei(), sysm.eps(), sysm.o).astype(np.complex128)
    t1 = np.zeros((sysm.o, sysm.v), dtype=np.complex128)
    return (t1, t2, t1.copy(), t2.copy())


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_oracle_rate(sysm, method, state, budget_s=12.0, max_steps=50):
    """Oracle (numpy restatement of the reference) RK4 steps/s on the host cores."""
    from oracle.cc_oracle import CCOracle, sin_field
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    Vt = sin_field(A, W0, sysm.mu[2])
    t = 0.0
    s = state
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        t += DT
        s = orc.rk4_step(method, t, DT, s, sysm.fock, Vt, 15)
        orc.dipole_moment(*s)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return n / el, n, el


def run_reference(args, rank, world):
    if rank != 0:
        return
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    wl = WORKLOADS[args.workload]
    sysm = synthetic_system(**wl)
    st = start_state(sysm)
    cores = os.cpu_count()
    # warm-up: one step; timed: a bounded sample of the workload's steps
    cpu_oracle_rate(sysm, args.method, st, budget_s=0.0, max_steps=1)
    rate, n, el = cpu_oracle_rate(sysm, args.method, st, budget_s=90.0, max_steps=max(1, args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": world,
        "steps": n, "warmup": 1, "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded DF integrals, MP2-guess start)",
        "config": {"workload": args.workload, "method": args.method, "o": sysm.o, "v": sysm.v, "nq": sysm.nq,
                   "dt": DT, "field": f"{A} sin({W0} t)", "parallelism": "replicas"},
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": f"{n} RK4 steps (+dipole) of {args.workload} in {el:.1f} s, numpy complex128, "
                                   f"BLAS threads = all {cores} host cores"},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    from python_code_to_check_c_gb300 import _lib
    from python_code_to_check_c_gb300.engine import CCEngine, launch_count, profile_step
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    wl = WORKLOADS[args.workload]
    sysm = synthetic_system(**wl)
    st = start_state(sysm)
    eng = CCEngine.from_system(sysm)
    prec = args.precision
    if prec == "auto":
        prec = "fp64"
        try:
            eng.set_precision("mixed", 5)
            prec = "mixed"
        except _lib.TdccError:
            eng.set_precision("fp64")
    else:
        eng.set_precision(prec, 5)
    field = _lib.make_field("sin", A, W0)
    dst = [torch.as_tensor(x, device=dev) for x in st]

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up (captures the step graphs)
    eng.propagate(args.method, dst, 0.0, DT, max(args.warmup, 3), field)
    torch.cuda.synchronize()

    # ---- timed region: K device-resident steps ----
    barrier()
    torch.cuda.synchronize()
    n0 = launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record()
        final, traj = eng.propagate(args.method, dst, 0.0, DT, args.steps, field)
        e1.record()
        torch.cuda.synchronize()
    barrier()
    launches = launch_count() - n0
    ms = e0.elapsed_time(e1)
    t_max = ms
    if world > 1:
        tt = torch.tensor([ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_max = float(tt.item())
    value = world * args.steps / (t_max / 1e3)
    finite = bool(torch.isfinite(torch.view_as_real(traj)).all().item())
    eng.check_errors()

    # ---- the plain FP64 form on the same start state (ratio and |d mu|) ----
    fp64 = None
    if prec == "mixed":
        k64 = max(1, min(args.steps, 30))
        eng.set_precision("fp64")
        eng.propagate(args.method, dst, 0.0, DT, 3, field)
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record()
        _, traj64 = eng.propagate(args.method, dst, 0.0, DT, k64, field)
        g1.record()
        torch.cuda.synchronize()
        v64 = k64 / (g0.elapsed_time(g1) / 1e3)
        dmu = float((traj[:k64] - traj64).abs().max().item())
        fp64 = {"value": world * v64, "steps": k64, "mixed_over_fp64": value / (world * v64),
                "max_dmu_vs_fp64_au": dmu, "slices": 5}
        eng.set_precision("mixed", 5)
        eng.propagate(args.method, dst, 0.0, DT, 1, field)

    # ---- end-to-end through the C ABI with host buffers ----
    ke = max(1, min(args.e2e_steps, args.steps))
    hst = [torch.as_tensor(x).pin_memory() for x in st]
    hmu = torch.empty(1, dtype=torch.complex128).pin_memory()
    h2d = sum(x.numel() * x.element_size() for x in hst)
    d2h = h2d + hmu.numel() * hmu.element_size()
    barrier()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    t_e2e = 0.0
    for i in range(ke):
        d = [x.to(dev, non_blocking=True) for x in hst]
        new, tr = eng.propagate(args.method, d, t_e2e, DT, 1, field)
        for h, x in zip(hst, new):
            h.copy_(x, non_blocking=True)
        hmu.copy_(tr[-1:], non_blocking=True)
        t_e2e += DT
    f1.record()
    torch.cuda.synchronize()
    e2e_ms = f0.elapsed_time(f1)
    if world > 1:
        tt = torch.tensor([e2e_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(tt.item())
    e2e = {"value": world * ke / (e2e_ms / 1e3), "unit": "steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ke}

    if rank != 0:
        return

    # ---- roofline of the dominant kernel (CUDA events per launch) ----
    recs = profile_step(eng, args.method, dst, 0.0, DT, field)
    by = {}
    for r in recs:
        k = (r["tag"], r["backend"])
        a = by.setdefault(k, {"ms": 0.0, "n": 0, "flops": 0.0, "bytes": 0.0, "kind": r["kind"]})
        a["ms"] += r["ms"]
        a["n"] += 1
        a["flops"] += r["flops"]
        a["bytes"] += r["bytes"]
    tot = sum(a["ms"] for a in by.values())
    (tag, backend), dom = max(by.items(), key=lambda kv: kv[1]["ms"])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    if dom["kind"] == 0 and backend == 1:
        achieved = dom["flops"] / (dom["ms"] / 1e3) / 1e12
        peak = peaks.get("bf16_tflops", 1900.0)
        roof = {"bound": "tensor", "unit": "TFLOP/s", "peak_source": "measured bf16 (MEASURED_PEAKS.json)"}
    elif dom["kind"] == 0:
        achieved = dom["flops"] / (dom["ms"] / 1e3) / 1e12
        peak = 1.25
        roof = {"bound": "fp64", "unit": "TFLOP/s", "peak_source": "nominal GB300 FP64 (no measured FP64 peak)"}
    else:
        achieved = dom["bytes"] / (dom["ms"] / 1e3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "unit": "GB/s", "peak_source": "measured HBM copy (MEASURED_PEAKS.json)"}
    roof.update({"kernel": tag, "achieved": achieved, "peak": peak, "frac": achieved / peak,
                 "traffic": None, "launches_per_step": dom["n"], "share_of_step": dom["ms"] / tot,
                 "avg_launch_ms": dom["ms"] / dom["n"]})
    top = sorted(by.items(), key=lambda kv: -kv[1]["ms"])[:6]
    breakdown = [{"kernel": k[0], "tc": k[1], "share": a["ms"] / tot, "launches": a["n"]} for k, a in top]

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        rate, n, el = cpu_oracle_rate(sysm, args.method, st, budget_s=12.0, max_steps=20)
        cpu = {"value": rate, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} RK4 steps (+dipole) of {args.workload} in {el:.1f} s, numpy complex128 oracle, "
                         f"BLAS threads = all host cores"}
    ws = eng.workspace_bytes()
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == "fp64" else "bf16x5-split+f64",
        "data": "synthetic (seeded DF integrals, MP2-guess start state)",
        "config": {"workload": args.workload, "method": args.method, "o": sysm.o, "v": sysm.v, "nq": sysm.nq,
                   "dt": DT, "field": f"{A} sin({W0} t)", "precision": prec, "parallelism": f"replicas x{world}",
                   "l2": f"per-step working set {ws / 2**20:.0f} MiB workspace + "
                         f"{sysm.n ** 4 * 8 / 2**20:.0f} MiB integrals (> 129 MB L2), no flush"},
        "roofline": roof, "kernel_breakdown": breakdown, "cpu_baseline": cpu, "e2e": e2e,
        "fp64_form": fp64,
        "gpu_launches": launches, "launches_per_step": launches / args.steps, "clocks": clk.summary(),
        "finite": finite,
    }
    print(json.dumps(line), flush=True)
    eng.close()


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
