"""Batched trajectories over uneven systems on one GPU:
    python bench_cases/batch_case.py [--steps 20] [--check-steps 200] [--slices 4]
        [--systems o8_v30,ccsd_o10_v38,o14_v58,o18_v82] [--no-autotune] [--check-all o8_v30,ccsd_o10_v38]

Each system (seeded DF integrals, x/y/z dipoles) gets 24 trajectories -- 3
polarisations x A in {0.001, 0.002, 0.005, 0.01} x w0 in {0.5, 0.923}, E(t) =
A sin(w0 t), dt = 0.005 -- advanced together by one batched system in the
mixed-precision form (--slices BF16 slices), from its ground state (device DIIS, FP64,
8 vectors, max residual 1e-10; the MP2 guess where DIIS diverges).  Launch shapes come from the autotuner.  The
four systems run concurrently (one host thread and one stream each).  Prints
one JSON line: aggregate trajectory-steps/s over --steps graph replays, per
system rates, and the worst dipole error against the FP64 form over
--check-steps steps (scaled down for the larger systems by --check-budget-s)
of all 24 trajectories for the systems named by --check-all, of the three
A = 0.01, w0 = 0.923 trajectories for the others."""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import argparse
import json
import threading
import time

import numpy as np
import torch

from python_code_to_check_c_gb300._lib import make_field
from python_code_to_check_c_gb300.engine import CCEngine
from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system

AMPS = (0.001, 0.002, 0.005, 0.01)
W0S = (0.5, 0.923)
DT = 0.005


def ground_state(sysm):
    """Device DIIS; where it diverges (the seeded integrals grow with n: at
    o=18, v=82 the MP2 correlation energy is about -46 Eh) the MP2 guess
    (t1 = 0, lambda = t) is the start state instead, and the record says so."""
    eng = CCEngine.from_system(sysm)
    tei = sysm.tei()
    t2g = mp2_guess(tei, np.linalg.eigh(sysm.fock)[0], sysm.o)
    e_mp2 = 0.25 * float(np.sum(tei[: sysm.o, : sysm.o, sysm.o:, sysm.o:] * t2g))
    t1g = np.zeros((sysm.o, sysm.v))
    E, nt, t1, t2 = eng.ground_state("CCSD", 0, t1g, t2g, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
    ok = np.isfinite(E) and bool(torch.isfinite(torch.view_as_real(t2)).all())
    info = {"E_mp2": e_mp2}
    if ok:
        El, nl, l1, l2 = eng.ground_state("CCSD", 1, t1, t2, t1, t2, maxsize=8, maxiter=100, E_min=0.0,
                                          r_tol=1e-10)
        ok = np.isfinite(El) and bool(torch.isfinite(torch.view_as_real(l2)).all())
        info.update({"start": "DIIS ground state", "E_corr": E, "t_iter": nt, "l_iter": nl})
    if not ok:
        t1 = torch.zeros((sysm.o, sysm.v), dtype=torch.complex128, device="cuda")
        t2 = torch.as_tensor(t2g.astype(np.complex128), device="cuda")
        l1, l2 = t1.clone(), t2.clone()
        info["start"] = "MP2 guess (DIIS diverges on this seeded system)"
    eng.close()
    return (t1, t2, l1, l2), info


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--systems", default="o8_v30,ccsd_o10_v38,o14_v58,o18_v82")
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--check-steps", type=int, default=200)
    p.add_argument("--check-budget-s", type=float, default=40.0)
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--slices", type=int, default=4)
    p.add_argument("--check-all", default="", help="systems whose 24 trajectories are all compared with FP64")
    a = p.parse_args()
    trajs = [(pol, A, w) for pol in (0, 1, 2) for A in AMPS for w in W0S]
    nb = len(trajs)
    runs = []
    for name in a.systems.split(","):
        sysm = synthetic_system(**WORKLOADS[name], all_dipoles=True)
        t_gs = time.perf_counter()
        gs, info = ground_state(sysm)
        info["seconds"] = time.perf_counter() - t_gs
        eng = CCEngine.from_system(sysm, nb=nb)
        eng.set_precision("mixed", a.slices)
        eng.set_fields([make_field("sin", A, w) for (_, A, w) in trajs], [pol for (pol, _, _) in trajs])
        bstate = [x.unsqueeze(0).expand((nb,) + tuple(x.shape)).contiguous() for x in gs]
        tune = None
        if not a.no_autotune:
            n, before, after = eng.autotune("CCSD", bstate)
            tune = {"ops_changed": n, "contraction_ms_before": before, "contraction_ms_after": after}
        eng.propagate("CCSD", bstate, 0.0, DT, 3, None)  # graphs
        torch.cuda.synchronize()
        runs.append({"name": name, "sysm": sysm, "gs": gs, "info": info, "eng": eng, "state": bstate, "tune": tune})

    # per-system rates, one at a time
    for r in runs:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, traj = r["eng"].propagate("CCSD", r["state"], 0.0, DT, a.steps, None)
        torch.cuda.synchronize()
        r["alone_s"] = time.perf_counter() - t0
        r["traj"] = traj

    # all systems concurrently
    streams = [torch.cuda.Stream() for _ in runs]
    start = threading.Barrier(len(runs) + 1)
    done = [None] * len(runs)

    def work(i):
        r = runs[i]
        with torch.cuda.stream(streams[i]):
            start.wait()
            r["eng"].propagate("CCSD", r["state"], 0.0, DT, a.steps, None)
            streams[i].synchronize()
        done[i] = time.perf_counter()

    ths = [threading.Thread(target=work, args=(i,)) for i in range(len(runs))]
    for t in ths:
        t.start()
    torch.cuda.synchronize()
    start.wait()
    t0 = time.perf_counter()
    for t in ths:
        t.join()
    wall = max(done) - t0
    total = len(runs) * nb * a.steps

    # accuracy: the strongly driven trajectories against the FP64 form
    check_all = set(x for x in a.check_all.split(",") if x)
    for r in runs:
        strong = (list(range(nb)) if r["name"] in check_all
                  else [k for k, (pol, A, w) in enumerate(trajs) if A == 0.01 and w == 0.923])
        sysm = r["sysm"]
        e64 = CCEngine.from_system(sysm, nb=len(strong))
        e64.set_fields([make_field("sin", trajs[k][1], trajs[k][2]) for k in strong], [trajs[k][0] for k in strong])
        st3 = [x.unsqueeze(0).expand((len(strong),) + tuple(x.shape)).contiguous() for x in r["gs"]]
        e64.propagate("CCSD", st3, 0.0, DT, 2, None)
        torch.cuda.synchronize()
        t0c = time.perf_counter()
        e64.propagate("CCSD", st3, 0.0, DT, 2, None)
        torch.cuda.synchronize()
        per_step = (time.perf_counter() - t0c) / 2
        ncheck = int(max(2, min(a.check_steps, a.check_budget_s / max(per_step, 1e-6))))
        _, t64 = e64.propagate("CCSD", st3, 0.0, DT, ncheck, None)
        _, tmx = r["eng"].propagate("CCSD", r["state"], 0.0, DT, ncheck, None)
        d = (tmx[:, strong] - t64).abs().max().item()
        r["check"] = {"steps": ncheck, "trajectories": "all 24" if len(strong) == nb else "A=0.01, w0=0.923, x/y/z",
                      "max_dmu_au": d, "fp64_s_per_step": per_step}
        e64.close()
        r["eng"].check_errors()
    out = {
        "trajectories": len(runs) * nb, "steps": a.steps, "dt": DT, "precision": f"mixed ({a.slices} BF16 slices)",
        "aggregate_traj_steps_per_s": total / wall, "concurrent_wall_s": wall,
        "systems": [{"system": r["name"], "o": r["sysm"].o, "v": r["sysm"].v, "trajectories": nb,
                     "alone_traj_steps_per_s": nb * a.steps / r["alone_s"], "autotune": r["tune"],
                     "ground_state": r["info"], "workspace_gb": r["eng"].workspace_bytes() / 1e9,
                     "accuracy": r["check"]} for r in runs],
    }
    print(json.dumps(out))
    for r in runs:
        r["eng"].close()


if __name__ == "__main__":
    main()
