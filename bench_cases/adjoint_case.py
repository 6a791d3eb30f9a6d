"""Gradient of a dipole-response objective with respect to pulse parameters, on
the GPU:  python bench_cases/adjoint_case.py
    [--workload ccsd_o10_v38] [--method CCSD] [--steps 500] [--dt 0.01] [--bumps 32]
    [--checkpoint 50] [--precision fp64|mixed] [--fd 3] [--fd-random 0] [--store -1|0|1]

Pulse E(t) = A sin(w0 t) sum_k c_k phi_k(t), 32 Gaussian bumps spread over the
propagation (sigma = spacing), c_k ~ U(0.5, 1.5) (seed 4), A = 0.003,
w0 = 0.923; objective J = sum_n dt cos(0.8 t_n) Re mu_z(t_n); start: the
ground state (device DIIS, 8 vectors, max residual 1e-10).  Prints one JSON
line: J, the forward time (captured step graphs), the reverse-mode time (its
own forward with checkpoints + the backward), their ratio, and central
differences (h = 1e-5) for the first --fd parameters (A, w0, c_0, ...), or,
with --fd-random K, for A, w0 and K envelope coefficients drawn at random
(seed 7, without replacement).
--store: the reverse pass reads the forward intermediates recorded per step
(1), runs each stage's forward ops again (0), or records them when they fit
in half the free device memory (-1, default)."""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import argparse
import json
import time

import numpy as np
import torch

from python_code_to_check_c_gb300.engine import CCEngine
from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights, pulse_gradient
from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="ccsd_o10_v38")
    p.add_argument("--method", default="CCSD")
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--dt", type=float, default=0.01)
    p.add_argument("--bumps", type=int, default=32)
    p.add_argument("--checkpoint", type=int, default=50)
    p.add_argument("--precision", default="fp64")
    p.add_argument("--fd", type=int, default=3)
    p.add_argument("--fd-random", type=int, default=0)
    p.add_argument("--store", type=int, default=-1)
    a = p.parse_args()
    sysm = synthetic_system(**WORKLOADS[a.workload])
    eng = CCEngine.from_system(sysm)
    t2 = mp2_guess(sysm.tei(), np.linalg.eigh(sysm.fock)[0], sysm.o)
    t1 = np.zeros((sysm.o, sysm.v))
    _, _, t1, t2 = eng.ground_state(a.method, 0, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
    _, _, l1, l2 = eng.ground_state(a.method, 1, t1, t2, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
    st = (t1, t2, l1, l2)
    if a.precision == "mixed":
        eng.set_precision("mixed", 5)
    eng.set_adjoint_store(a.store)
    T = a.steps * a.dt
    spacing = T / max(a.bumps - 1, 1)
    rng = np.random.default_rng(4)
    pulse = Pulse(A=0.003, w0=0.923, c=rng.uniform(0.5, 1.5, a.bumps), t_first=0.0, spacing=spacing, sigma=spacing)
    w = cosine_weights(0.0, a.dt, a.steps)

    def J_of(pu):
        _, traj = eng.propagate(a.method, st, 0.0, a.dt, a.steps, pu.field(), precs=-1)
        return float(np.sum(w * traj.cpu().numpy().real))

    J_of(pulse)  # warm-up: programs, graphs
    torch.cuda.synchronize()
    t_a = time.perf_counter()
    J = J_of(pulse)
    t_fwd = time.perf_counter() - t_a
    pulse_gradient(eng, a.method, st, pulse, 0.0, a.dt, min(a.steps, 2 * a.checkpoint), w[: min(a.steps, 2 * a.checkpoint)],
                   checkpoint=a.checkpoint)  # warm-up of the reverse-mode programs
    torch.cuda.synchronize()
    t_b = time.perf_counter()
    Jg, gA, gw, gc = pulse_gradient(eng, a.method, st, pulse, 0.0, a.dt, a.steps, w, checkpoint=a.checkpoint)
    t_grad = time.perf_counter() - t_b
    eng.check_errors()
    grads = [gA, gw] + list(gc)
    names = ["A", "w0"] + [f"c{k}" for k in range(a.bumps)]
    fd = []
    h = 1e-5
    picks = list(range(min(a.fd, len(names))))
    if a.fd_random > 0:
        ks = np.random.default_rng(7).choice(a.bumps, size=min(a.fd_random, a.bumps), replace=False)
        picks = [0, 1] + sorted(int(k) + 2 for k in ks)
    for k in picks:
        pp = Pulse(pulse.A, pulse.w0, pulse.c.copy(), pulse.t_first, pulse.spacing, pulse.sigma)
        pm = Pulse(pulse.A, pulse.w0, pulse.c.copy(), pulse.t_first, pulse.spacing, pulse.sigma)
        if k == 0:
            pp.A += h
            pm.A -= h
        elif k == 1:
            pp.w0 += h
            pm.w0 -= h
        else:
            pp.c[k - 2] += h
            pm.c[k - 2] -= h
        d = (J_of(pp) - J_of(pm)) / (2 * h)
        fd.append({"param": names[k], "adjoint": grads[k], "central_difference": d,
                   "rel_err": abs(grads[k] - d) / max(abs(d), 1e-300)})
    print(json.dumps({
        "workload": a.workload, "method": a.method, "steps": a.steps, "dt": a.dt, "bumps": a.bumps,
        "checkpoint": a.checkpoint, "precision": a.precision, "store": a.store, "J": J, "J_from_adjoint_run": Jg,
        "forward_s": t_fwd, "gradient_s": t_grad, "grad_over_fwd": t_grad / t_fwd,
        "gradient_norm": float(np.linalg.norm(grads)), "fd_checks": fd}))
    eng.close()


if __name__ == "__main__":
    main()
