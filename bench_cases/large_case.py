"""Large TD-CCSD / TD-CC2 on one GPU:
    python bench_cases/large_case.py [--workload o24_v160] [--method CCSD]
        [--mixed-steps 10] [--fp64-steps 2] [--slices 4] [--also-slices 5] [--dt 0.005]

Seeded DF integrals (Q = 480 at o=24, v=160; <pq||rs> built on the device by
tdcc_tei_from_df, its time against the host numpy build reported with
--host-build), start t1 = 0, t2 = s x MP2
guess, lambda = t, dt = 0.005, E = 0.002 sin(0.923 t).  The seeded
integrals grow with n (at o=18, v=82 the MP2 correlation energy is already
about -46 Eh and the ground-state iteration diverges), so the state is
scaled (s = 1, 0.1, 0.01, ... until the measured steps stay finite; the
cost of a step does not depend on the state) and s is reported.  Prints one JSON line: steps/s of the mixed and FP64
forms (captured step graphs, CUDA events), |d mu| between them over the FP64
steps, and per-contraction rates of one mixed step from CUDA events around
every launch (the ladder and ring contractions with their tensor work
fraction: FP64-equivalent flops x slice products / time / measured BF16 peak)."""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import argparse
import json
import os
import time

import numpy as np
import torch

from python_code_to_check_c_gb300._lib import make_field
from python_code_to_check_c_gb300.engine import CCEngine, profile_step, tei_from_df_device
from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess_oovv, synthetic_system


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="o24_v160")
    p.add_argument("--method", default="CCSD")
    p.add_argument("--mixed-steps", type=int, default=10)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--host-build", action="store_true")
    p.add_argument("--slices", type=int, default=4, help="slices per operand in the mixed form")
    p.add_argument("--dt", type=float, default=0.005, help="time step (a step costs the same for any dt)")
    p.add_argument("--min-scale", type=float, default=1e-6, help="smallest state scale tried")
    p.add_argument("--also-slices", type=int, nargs="*", default=[], help="further slice counts timed and compared")
    a = p.parse_args()
    t_build = time.perf_counter()
    sysm = synthetic_system(**WORKLOADS[a.workload])
    host_build_s = None
    if a.host_build:
        t_h = time.perf_counter()
        sysm.tei()
        host_build_s = time.perf_counter() - t_h
    tei_from_df_device(sysm.B[:1, :2, :2])  # library load, first launch
    torch.cuda.synchronize()
    t_d = time.perf_counter()
    tei = tei_from_df_device(sysm.B)
    torch.cuda.synchronize()
    device_build_s = time.perf_counter() - t_d
    eng = CCEngine(tei, sysm.fock, sysm.mu, sysm.o)
    oovv = tei[: sysm.o, : sysm.o, sysm.o:, sysm.o:].cpu().numpy()
    del tei
    t2 = mp2_guess_oovv(oovv, sysm.eps(), sysm.o).astype(np.complex128)
    e_mp2 = 0.25 * float(np.real(np.sum(oovv * t2)))
    t1 = np.zeros((sysm.o, sysm.v), dtype=np.complex128)
    t2_dev = torch.as_tensor(t2, device="cuda")
    scale = 1.0
    st = [torch.as_tensor(x, device="cuda") for x in (t1, t2, t1.copy(), t2.copy())]
    build_s = time.perf_counter() - t_build
    f = make_field("sin", 0.002, 0.923)

    def timed(steps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, traj = eng.propagate(a.method, st, 0.0, a.dt, steps, f)
        e1.record()
        torch.cuda.synchronize()
        return traj, e0.elapsed_time(e1) / 1e3

    eng.set_precision("mixed", a.slices)
    while True:
        try:
            eng.propagate(a.method, st, 0.0, a.dt, 1, f)
            trmx, smx = timed(a.mixed_steps)
            break
        except Exception:
            if scale * 0.1 < a.min_scale:
                raise
            scale *= 0.1
            st[1] = t2_dev * scale
            st[3] = st[1].clone()
    eng.check_errors()
    recs = profile_step(eng, a.method, st, 0.0, a.dt, f)
    ws_mixed = eng.workspace_bytes()
    # further slice counts on the same state (rates and |d mu| against the same FP64 steps)
    more = {}
    for S2 in a.also_slices:
        eng.set_precision("mixed", S2)
        eng.propagate(a.method, st, 0.0, a.dt, 1, f)
        tr2, s2 = timed(a.mixed_steps)
        eng.check_errors()
        more[S2] = (tr2, a.mixed_steps / s2)
    eng.set_precision("fp64")
    eng.propagate(a.method, st, 0.0, a.dt, 1, f)
    tr64, s64 = timed(a.fp64_steps)
    k = min(a.fp64_steps, a.mixed_steps)
    dmu = float((trmx[:k] - tr64[:k]).abs().max().item())
    peak = 1886.4
    try:
        peak = json.load(open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                           "MEASURED_PEAKS.json")))["bf16_tflops"]
    except Exception:
        pass
    agg = {}
    for r in recs:
        if r["kind"] != 0:
            continue
        x = agg.setdefault((r["tag"], r["backend"]), [0.0, 0.0, 0])
        x[0] += r["ms"]
        x[1] += r["flops"]
        x[2] += 1
    tot = sum(r["ms"] for r in recs)
    pairs = a.slices * (a.slices + 1) // 2  # slice products per FP64 product
    top = sorted(agg.items(), key=lambda kv: -kv[1][0])[:8]
    contractions = [{"op": tag, "tensor_cores": bool(be), "launches": n, "share_of_step": ms / tot,
                     "fp64_equiv_tflops": fl / (ms / 1e3) / 1e12,
                     "tensor_work_frac": (fl * pairs / (ms / 1e3) / 1e12 / peak) if be == 1 else None}
                    for (tag, be), (ms, fl, n) in top]
    print(json.dumps({
        "workload": a.workload, "method": a.method, "o": sysm.o, "v": sysm.v, "nq": sysm.nq,
        "build_s": build_s, "tei_device_build_s": device_build_s, "tei_host_build_s": host_build_s,
        "E_mp2": e_mp2, "state_scale": scale,
        "mixed_steps_per_s": a.mixed_steps / smx, "mixed_steps": a.mixed_steps,
        "fp64_steps_per_s": a.fp64_steps / s64, "fp64_steps": a.fp64_steps,
        "mixed_over_fp64": (a.mixed_steps / smx) / (a.fp64_steps / s64), "max_dmu_au": dmu, "dmu_steps": k,
        "slices": a.slices, "dt": a.dt,
        "also": [{"slices": S2, "mixed_steps_per_s": r2, "mixed_over_fp64": r2 / (a.fp64_steps / s64),
                  "max_dmu_au": float((t2m[:k] - tr64[:k]).abs().max().item())} for S2, (t2m, r2) in more.items()], "mu_fp64_range": [float(tr64[:k].real.min().item()), float(tr64[:k].real.max().item())],
        "workspace_gb_mixed": ws_mixed / 1e9, "serial_step_ms_mixed": tot, "top_contractions": contractions}))
    eng.close()


if __name__ == "__main__":
    main()
