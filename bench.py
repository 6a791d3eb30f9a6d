"""Benchmark: TD-CCSD RK4 steps/s on one GB300 (replicas across GPUs).

One RK4 "step" of one trajectory is the reference's propagation loop body
(CCSD_Helper.py:1206-1240): 16 right-hand sides (block-frozen RK4 over T1,
T2, L1, L2), the rounded state update and the dipole trace.

Headline workload (``value``): the mixed-precision batched form at o=10,
v=38 (Q=144 seeded density-fitting integrals), 24 trajectories advanced
together -- 3 polarisations x A in {0.001, 0.002, 0.005, 0.01} x w0 in
{0.5, 0.923}, E(t) = A sin(w0 t), dt = 0.005 -- from the converged ground
state (device DIIS, 8 vectors, max residual 1e-10), 4 BF16 slices per
operand (--slices).  ``value`` counts trajectory-steps per second.  The same
line reports the plain FP64 GPU form on the same 24 trajectories (and on one
trajectory), the mixed form on one trajectory, |d mu| against the FP64 form,
the end-to-end rate with host buffers, the roofline of the dominant kernel,
the achieved flop rates under the reference's flop count and the engine's,
the cost of a pulse gradient by reverse mode relative to the forward
(``adjoint``, FP64, --adjoint-steps steps) and the CPU oracle on the host
cores (one single-thread process per core, each on its own trajectory).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|mixed|auto] [--workload NAME] [--method CCSD|CC2] [--nb 24]

Prints one JSON line (rank 0).  The reference arm (--impl reference) times the
CPU oracle (the numpy restatement of the reference) on the host cores for
the same workload: one single-thread process per core, each advancing its
own trajectory of the batch, as independent runs of the reference would.
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
DT = 0.005
AMPS = (0.001, 0.002, 0.005, 0.01)
W0S = (0.5, 0.923)
POLS = (0, 1, 2)
REF_TRAJ = (2, 0.002, 0.923)  # the single-trajectory configuration (z, A, w0)
# DRAM traffic of the slice-product kernels against their algorithmic bytes (packed operands
# read once, output written once): 460.9 MB over 403.8 MB for four launches of the T2 program
# (ladder, 24 batched products, two long-K products), a one-pass ncu capture (dram__bytes_read.sum,
# dram__bytes_write.sum) of `bench_cases/profile_case.py --block T2 --precision mixed --slices 4
# --nb 24`; the roofline's traffic per launch is this ratio times the step's algorithmic bytes per
# slice-product launch.
TRAFFIC_RATIO = {"ozaki_kernel": 460.9 / 403.8}
TRAFFIC_SOURCE = ("ncu DRAM bytes / algorithmic bytes of four slice-product launches of the T2 program "
                  "(1.14), times the step's algorithmic bytes per launch")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    p.add_argument("--workload", default="ccsd_o10_v38")
    p.add_argument("--method", default="CCSD", choices=["CCSD", "CC2"])
    p.add_argument("--nb", type=int, default=24, help="trajectories advanced together (24 = 3 pol x 4 A x 2 w0)")
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--slices", type=int, default=4, help="BF16 slices per operand in the mixed form (4: |d mu| <= 1e-8 over 2000 steps, tests/test_gpu_long.py)")
    p.add_argument("--fp64-batch-steps", type=int, default=4, help="timed steps of the batched FP64 form")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--adjoint-steps", type=int, default=100, help="pulse-gradient cost measurement (0: skip)")
    return p.parse_args()


def trajectories(nb):
    full = [(p, a, w) for p in POLS for a in AMPS for w in W0S]
    return [full[k % len(full)] for k in range(nb)]


def mp2_state(sysm):
    """MP2-guess state: t1 = 0, t2 = <ij||ab>/D, lambda = t (complex128)."""
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


def cpu_oracle_rate(sysm, method, state, budget_s=12.0, max_steps=50, traj=REF_TRAJ):
    """Oracle (numpy restatement of the reference) RK4 steps/s on the host cores
    for one trajectory (default: z / A=0.002 / w0=0.923)."""
    from oracle.cc_oracle import CCOracle, sin_field
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    Vt = sin_field(traj[1], traj[2], sysm.mu[traj[0]])
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


_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS")


def _one_thread_child(workload, method, state, budget_s, max_steps, warmup, q, traj, barrier):
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    sysm = synthetic_system(**WORKLOADS[workload], all_dipoles=True)
    if warmup > 0:
        cpu_oracle_rate(sysm, method, state, budget_s=0.0, max_steps=warmup, traj=traj)
    barrier.wait(timeout=1800)  # every process starts its timed loop at once
    q.put(cpu_oracle_rate(sysm, method, state, budget_s=budget_s, max_steps=max_steps, traj=traj))


def _spawn_one_thread(nproc, workload, method, state, budget_s, max_steps, warmup=1):
    """`nproc` spawned processes (numpy with one BLAS thread each, no GPU use),
    process k advancing trajectory k of the batch after `warmup` untimed
    steps; returns their (steps/s, steps, seconds)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    barrier = ctx.Barrier(nproc)
    trajs = trajectories(nproc)
    saved = {k: os.environ.get(k) for k in _THREAD_VARS}
    procs = []
    try:
        for k in _THREAD_VARS:
            os.environ[k] = "1"
        for k in range(nproc):
            pr = ctx.Process(target=_one_thread_child,
                             args=(workload, method, state, budget_s, max_steps, warmup, q, trajs[k], barrier))
            pr.start()
            procs.append(pr)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    try:
        res = [q.get(timeout=budget_s * 10 + 1800) for _ in range(nproc)]
    finally:
        for pr in procs:
            pr.join(timeout=60)
    return res


def cpu_oracle_rate_one_thread(workload, method, state, budget_s=12.0, max_steps=20):
    """The oracle rate with one BLAS thread: a spawned process whose numpy
    starts with the thread variables set to 1 (no GPU use there)."""
    return _spawn_one_thread(1, workload, method, state, budget_s, max_steps)[0]


def cpu_oracle_throughput(workload, method, state, budget_s=12.0, max_steps=20, warmup=1):
    """Throughput of the host cores: one single-thread oracle process per
    core, each on its own trajectory, all timed at once; trajectory-steps/s
    is the sum of the processes' rates.  Returns (rate, processes, steps of
    all processes, longest timed loop in seconds)."""
    nproc = os.cpu_count() or 1
    res = _spawn_one_thread(nproc, workload, method, state, budget_s, max_steps, warmup)
    return sum(r[0] for r in res), nproc, sum(r[1] for r in res), max(r[2] for r in res)


def port_calibration(workload):
    """The reference's own loop body timed against the oracle on a host with
    the reference checkout (oracle/calibrate_port.py), if recorded."""
    try:
        with open(os.path.join(ROOT, "oracle", "port_calibration.json")) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return None
    out = {k: v for k, v in data.items() if k.split("/")[0] == workload}
    return out or None


def workload_config(args, sysm, world):
    """The `config` object of both arms' lines (identical for the same flags)."""
    return {"workload": f"{args.workload}_x{args.nb}", "method": args.method, "o": sysm.o, "v": sysm.v,
            "nq": sysm.nq, "dt": DT, "trajectories": args.nb,
            "fields": "A sin(w0 t), 3 pol x A {0.001,0.002,0.005,0.01} x w0 {0.5,0.923}",
            "value_counts": "trajectory-steps per second (all trajectories of all replicas)",
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (n^4 integrals and per-step workspace > 129 MB), no flush"}


def run_reference(args, rank, world):
    """The reference arm: the oracle (the numpy restatement of the reference;
    the reference's own source does not travel to the GPU host) on the host
    cores, at its best throughput: one single-thread process per core, each
    advancing its own trajectory of the batch, as independent reference runs
    would.  The single-trajectory all-cores rate is reported beside it."""
    if rank != 0:
        return
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    sysm = synthetic_system(**WORKLOADS[args.workload], all_dipoles=True)
    st = mp2_state(sysm)
    cores = os.cpu_count()
    warm = max(args.warmup, 1)
    rate, nproc, n, el = cpu_oracle_throughput(args.workload, args.method, st, budget_s=60.0,
                                               max_steps=max(1, args.steps), warmup=warm)
    cpu_oracle_rate(sysm, args.method, st, budget_s=0.0, max_steps=1)  # warm-up
    r16, n16, el16 = cpu_oracle_rate(sysm, args.method, st, budget_s=20.0, max_steps=max(1, args.steps))
    sample = (f"{nproc} single-thread processes (one per host core), each advancing its own trajectory of the "
              f"batch after {warm} untimed steps: {n} RK4 steps (+dipole) in all, timed loops of "
              f"{el:.1f} s; numpy complex128 oracle")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": world,
        "steps": n, "warmup": warm, "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded DF integrals; MP2-guess state: the cost of a step does not depend on it)",
        "config": workload_config(args, sysm, world),
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample,
                         "one_trajectory_all_cores": {"value": r16, "unit": "steps/s", "cores": cores,
                                                      "sample": f"{n16} RK4 steps of one trajectory in "
                                                                f"{el16:.1f} s, BLAS threads = {cores}"},
                         "reference_vs_port": port_calibration(args.workload)},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ground_state(sysm, method, dev):
    """Converged T and Lambda (device DIIS, 8 vectors, max residual 1e-10)."""
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import mp2_guess
    eng = CCEngine.from_system(sysm)
    t2 = mp2_guess(sysm.tei(), np.linalg.eigh(sysm.fock)[0], sysm.o)
    t1 = np.zeros((sysm.o, sysm.v))
    E, nt, t1, t2 = eng.ground_state(method, 0, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
    El, nl, l1, l2 = eng.ground_state(method, 1, t1, t2, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
    eng.close()
    return (t1, t2, l1, l2), {"E_corr": E, "pseudo_E": El, "t_iterations": nt, "l_iterations": nl}


def adjoint_cost(sysm, method, gs, nsteps):
    """Gradient of J = sum_n dt cos(0.8 t_n) Re mu_z(t_n) with respect to a 32-bump
    pulse (A = 0.003, w0 = 0.923, c_k ~ U(0.5, 1.5)), dt = 0.01, FP64, every step
    kept (with the forward intermediates the reverse-mode programs read):
    seconds of the reverse mode over seconds of the forward, and dJ/dA
    against a central difference (h = 1e-5)."""
    import torch

    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights, pulse_gradient
    eng = CCEngine.from_system(sysm)
    dt = 0.01
    rng = np.random.default_rng(4)
    spacing = nsteps * dt / 31
    pulse = Pulse(A=0.003, w0=0.923, c=rng.uniform(0.5, 1.5, 32), t_first=0.0, spacing=spacing, sigma=spacing)
    w = cosine_weights(0.0, dt, nsteps)

    def J_of(pu):
        _, traj = eng.propagate(method, gs, 0.0, dt, nsteps, pu.field(), precs=-1)
        return float(np.sum(w * traj.cpu().numpy().real))

    J_of(pulse)
    pulse_gradient(eng, method, gs, pulse, 0.0, dt, min(nsteps, 10), w[:min(nsteps, 10)], checkpoint=nsteps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = J_of(pulse)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    Jg, gA, gw, gc = pulse_gradient(eng, method, gs, pulse, 0.0, dt, nsteps, w, checkpoint=nsteps)
    t_grad = time.perf_counter() - t0
    h = 1e-5
    pp = Pulse(pulse.A + h, pulse.w0, pulse.c, pulse.t_first, pulse.spacing, pulse.sigma)
    pm = Pulse(pulse.A - h, pulse.w0, pulse.c, pulse.t_first, pulse.spacing, pulse.sigma)
    fd = (J_of(pp) - J_of(pm)) / (2 * h)
    eng.close()
    return {"steps": nsteps, "dt": dt, "bumps": 32, "precision": "fp64", "checkpoint": "every step kept",
            "reverse_reads": "forward intermediates recorded by the forward step graph (activation records)",
            "forward_s": t_fwd, "gradient_s": t_grad, "grad_over_fwd": t_grad / t_fwd, "J": J,
            "dJ_dA": gA, "dJ_dA_central_difference": fd, "rel_err": abs(gA - fd) / max(abs(fd), 1e-300)}


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest value over the ranks (the slowest replica's time); the
    tensor lives on `device` (CUDA under NCCL, CPU under gloo)."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, trajectories: int, steps: int, ms: float) -> float:
    """Trajectory-steps per second of all replicas together: every rank
    advances `trajectories` trajectories by `steps` steps; `ms` is the
    slowest rank's time."""
    return world * trajectories * steps / (ms / 1e3)


# Algorithmic flops of one trajectory-step in the reference's convention: the
# reference's own contract() calls of one loop body (16 right-hand sides and
# the dipole), each costed by opt_einsum.contract_path (about 2 x
# multiply-adds), x2 with one complex operand and x4 with two or more
# (oracle/calibrate_port.py records the count).  The engine's re-associated
# equations do fewer (HOISTED_FLOPS, the sum of its contractions' flops).
REF_FLOPS = {("ccsd_o10_v38", "CCSD"): 5.771e10}
HOISTED_FLOPS = {("ccsd_o10_v38", "CCSD"): 2.13e10}


def flops_note(args, value):
    """Achieved flop rates of the batched step under both conventions."""
    key = (args.workload, args.method)
    out = {}
    for name, table in (("reference_convention", REF_FLOPS), ("hoisted", HOISTED_FLOPS)):
        if key in table:
            out[name] = {"flops_per_trajectory_step": table[key], "achieved_tflops": value * table[key] / 1e12}
    return out or None


def timed(fn):
    import torch
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    out = fn()
    b.record()
    torch.cuda.synchronize()
    return out, a.elapsed_time(b)


def run_ours(args, rank, world, local_rank):
    import torch

    from python_code_to_check_c_gb300 import _lib
    from python_code_to_check_c_gb300.engine import CCEngine, launch_count, profile_step
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    sysm = synthetic_system(**WORKLOADS[args.workload], all_dipoles=True)
    gs, gs_info = ground_state(sysm, args.method, dev)
    nb = args.nb
    trajs = trajectories(nb)
    fields = [_lib.make_field("sin", a, w) for (_, a, w) in trajs]
    pols = [p for (p, _, _) in trajs]
    ref_k = trajs.index(REF_TRAJ) if REF_TRAJ in trajs else 0
    bstate = [x.unsqueeze(0).expand((nb,) + tuple(x.shape)).contiguous() for x in gs]

    eng = CCEngine.from_system(sysm, nb=nb)
    prec = args.precision
    if prec == "auto":
        prec = "fp64"
        try:
            eng.set_precision("mixed", args.slices)
            prec = "mixed"
        except _lib.TdccError:
            eng.set_precision("fp64")
    else:
        eng.set_precision(prec, args.slices)
    eng.set_fields(fields, pols)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up (captures the step graphs)
    eng.propagate(args.method, bstate, 0.0, DT, max(args.warmup, 3), None)
    torch.cuda.synchronize()

    # ---- timed region: K device-resident steps of all nb trajectories ----
    barrier()
    torch.cuda.synchronize()
    n0 = launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record()
        final, traj = eng.propagate(args.method, bstate, 0.0, DT, args.steps, None)
        e1.record()
        torch.cuda.synchronize()
    barrier()
    launches = launch_count() - n0
    t_max = max_over_ranks(e0.elapsed_time(e1), world, dev)
    value = whole_job_rate(world, nb, args.steps, t_max)
    finite = bool(torch.isfinite(torch.view_as_real(traj)).all().item())
    eng.check_errors()

    # ---- one trajectory: the plain FP64 form and the mixed form ----
    ref_field = _lib.make_field("sin", REF_TRAJ[1], REF_TRAJ[2])
    e1t = CCEngine.from_system(sysm)
    e1t.set_fields([ref_field], [REF_TRAJ[0]])
    k1 = max(1, min(args.steps, 30))
    e1t.set_precision("fp64")
    e1t.propagate(args.method, gs, 0.0, DT, 3, None)
    (_, traj64), ms64 = timed(lambda: e1t.propagate(args.method, gs, 0.0, DT, k1, None))
    v64 = k1 / (ms64 / 1e3)
    single_mixed = None
    if prec == "mixed":
        e1t.set_precision("mixed", args.slices)
        e1t.propagate(args.method, gs, 0.0, DT, 3, None)
        k1m = max(1, min(args.steps * 2, 100))
        (_, _), ms1m = timed(lambda: e1t.propagate(args.method, gs, 0.0, DT, k1m, None))
        single_mixed = {"value": k1m / (ms1m / 1e3), "unit": "steps/s", "steps": k1m}
        e1t.check_errors()
    e1t.close()
    dmu = float((traj[:k1, ref_k] - traj64[:k1]).abs().max().item())

    # ---- the same batch of trajectories in the plain FP64 form ----
    kb64 = max(1, min(args.steps, args.fp64_batch_steps))
    e64 = CCEngine.from_system(sysm, nb=nb)
    e64.set_precision("fp64")
    e64.set_fields(fields, pols)
    e64.propagate(args.method, bstate, 0.0, DT, 2, None)
    (_, trajb64), msb64 = timed(lambda: e64.propagate(args.method, bstate, 0.0, DT, kb64, None))
    e64.check_errors()
    e64.close()
    vb64 = whole_job_rate(world, nb, kb64, max_over_ranks(msb64, world, dev))
    dmu_b = float((traj[:kb64] - trajb64[:kb64]).abs().max().item())
    fp64 = {"value": vb64, "unit": "steps/s", "steps": kb64, "trajectories": nb,
            "batched_mixed_over_fp64": value / vb64,
            "max_dmu_vs_fp64_au": dmu_b, "dmu_steps": kb64, "dmu_trajectories": f"all {nb}",
            "one_trajectory": {"value": world * v64, "unit": "steps/s", "steps": k1,
                               "max_dmu_vs_fp64_au": dmu, "dmu_steps": k1,
                               "dmu_trajectory": "z, A=0.002, w0=0.923"},
            "slices": args.slices if prec == "mixed" else None}
    if single_mixed is not None:
        single_mixed["single_mixed_over_fp64"] = single_mixed["value"] / v64

    # ---- end-to-end through the public API with host buffers ----
    ke = max(1, min(args.e2e_steps, args.steps))
    hst = [x.cpu().pin_memory() for x in bstate]
    hmu = torch.empty(nb, dtype=torch.complex128).pin_memory()
    h2d = sum(x.numel() * x.element_size() for x in hst)
    d2h = h2d + hmu.numel() * hmu.element_size()
    eng.propagate(args.method, [x.to(dev) for x in hst], 0.0, DT, 1, None)
    barrier()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    t_e2e = 0.0
    for i in range(ke):
        d = [x.to(dev, non_blocking=True) for x in hst]
        new, tr = eng.propagate(args.method, d, t_e2e, DT, 1, None)
        for h, x in zip(hst, new):
            h.copy_(x, non_blocking=True)
        hmu.copy_(tr[-1], non_blocking=True)
        t_e2e += DT
    f1.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1), world, dev)
    e2e = {"value": whole_job_rate(world, nb, ke, e2e_ms), "unit": "steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ke, "trajectories": nb}

    if rank != 0:
        eng.close()
        return

    # ---- roofline of the dominant kernel (CUDA events per launch) ----
    # launches are grouped by kernel: the slice products (tensor cores), the
    # FP32-pipe slice products, FP64 contractions, operand packing and the
    # elementwise ops; the roofline line describes the kernel with the most time
    recs = profile_step(eng, args.method, bstate, 0.0, DT, fields[0])

    def kernel_of(r):
        if r["kind"] == 0:
            return {1: "ozaki_kernel", 2: "simt_slices_kernel"}.get(r["backend"], "gemm_f64_kernel")
        if r["tag"].endswith(":packA") or r["tag"].endswith(":packB"):
            return "pack_kernel"
        return "add_kernel" if r["kind"] == 1 else "rk4/trace kernels"

    by, by_tag = {}, {}
    for r in recs:
        for d, k in ((by, kernel_of(r)), (by_tag, (r["tag"], r["backend"]))):
            a = d.setdefault(k, {"ms": 0.0, "n": 0, "flops": 0.0, "bytes": 0.0})
            a["ms"] += r["ms"]
            a["n"] += 1
            a["flops"] += r["flops"]
            a["bytes"] += r["bytes"]
    tot = sum(a["ms"] for a in by.values())
    kern, dom = max(by.items(), key=lambda kv: kv[1]["ms"])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    pairs = args.slices * (args.slices + 1) // 2  # slice products per FP64 product (levels 2..S+1)
    if kern == "ozaki_kernel":
        achieved = dom["flops"] / (dom["ms"] / 1e3) / 1e12
        peak = peaks.get("bf16_tflops", 1900.0)
        roof = {"bound": "tensor", "unit": "TFLOP/s",
                "peak_source": "measured bf16 burst (MEASURED_PEAKS.json)" if "bf16_tflops" in peaks else "fallback",
                "achieved_is": "FP64-equivalent algorithmic flops of the step's slice products / their launch time",
                "tensor_work_frac": achieved * pairs / peak}
    elif kern in ("gemm_f64_kernel", "simt_slices_kernel"):
        achieved = dom["flops"] / (dom["ms"] / 1e3) / 1e12
        peak = 1.25
        roof = {"bound": "fp64", "unit": "TFLOP/s", "peak_source": "nominal GB300 FP64 (no measured FP64 peak)"}
    else:
        achieved = dom["bytes"] / (dom["ms"] / 1e3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "unit": "GB/s", "peak_source": "measured HBM copy (MEASURED_PEAKS.json)"}
    traffic = TRAFFIC_RATIO[kern] * dom["bytes"] / dom["n"] if kern in TRAFFIC_RATIO else None
    roof.update({"kernel": kern, "achieved": achieved, "peak": peak, "frac": achieved / peak,
                 "traffic": traffic,
                 "traffic_source": TRAFFIC_SOURCE if traffic else None,
                 "algorithmic_bytes_per_launch": dom["bytes"] / dom["n"],
                 "launches_per_step": dom["n"], "share_of_step": dom["ms"] / tot,
                 "avg_launch_ms": dom["ms"] / dom["n"]})
    breakdown = [{"kernel": k, "share": a["ms"] / tot, "launches": a["n"]}
                 for k, a in sorted(by.items(), key=lambda kv: -kv[1]["ms"])]
    top = sorted(by_tag.items(), key=lambda kv: -kv[1]["ms"])[:6]
    top_contractions = [{"op": k[0], "backend": k[1], "share": a["ms"] / tot, "launches": a["n"]} for k, a in top]

    adj = None
    if args.adjoint_steps > 0:
        adj = adjoint_cost(sysm, args.method, gs, args.adjoint_steps)

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        host_state = [x.cpu().numpy() for x in gs]
        rate, nproc, n, el = cpu_oracle_throughput(args.workload, args.method, host_state, budget_s=12.0,
                                                   max_steps=20, warmup=1)
        cpu = {"value": rate, "unit": "steps/s", "cores": nproc, "kind": "port",
               "sample": f"{nproc} single-thread oracle processes (one per host core), each advancing its own "
                         f"trajectory of the batch: {n} RK4 steps (+dipole) in all, timed loops of {el:.1f} s; "
                         f"numpy complex128"}
        r16, n16, el16 = cpu_oracle_rate(sysm, args.method, host_state, budget_s=12.0, max_steps=20)
        cpu["one_trajectory_all_cores"] = {
            "value": r16, "unit": "steps/s", "cores": os.cpu_count(),
            "sample": f"{n16} RK4 steps (+dipole) of one trajectory in {el16:.1f} s, BLAS threads = all host cores"}
        try:
            r1, n1, el1 = cpu_oracle_rate_one_thread(args.workload, args.method, host_state, budget_s=12.0)
            cpu["one_thread"] = {"value": r1, "unit": "steps/s", "cores": 1,
                                 "sample": f"{n1} RK4 steps (+dipole) in {el1:.1f} s, same oracle, one BLAS thread"}
        except Exception as ex:  # reported, not fatal: the throughput figure stands
            cpu["one_thread"] = {"unavailable": str(ex)[:200]}
        cpu["reference_vs_port"] = port_calibration(args.workload)
    ws = eng.workspace_bytes()
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == "fp64" else f"bf16x{args.slices}-split+f64",
        "data": "synthetic (seeded DF integrals, ground state by device DIIS)",
        "config": workload_config(args, sysm, world),
        "precision": prec, "ground_state": gs_info,
        "working_set": f"{ws / 2**30:.1f} GiB workspace + {sysm.n ** 4 * 8 / 2**20:.0f} MiB integrals",
        "flops": flops_note(args, value),
        "roofline": roof, "kernel_breakdown": breakdown, "top_contractions": top_contractions,
        "cpu_baseline": cpu, "e2e": e2e,
        "fp64_form": fp64, "single_trajectory_mixed": single_mixed, "adjoint": adj,
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
