"""Times the reference's own loop body against the oracle port (TEST INFRASTRUCTURE ONLY).

The CPU baseline of ``bench.py`` runs the oracle (``oracle/cc_oracle.py``, a
numpy restatement of the reference), because the reference's source does
not travel to the GPU host.  This script measures, on a host that has the
reference checkout, how fast the reference's own functions advance the same
trajectory as the port does, so the port's rate can be read as the
reference's:

    python oracle/calibrate_port.py /path/to/reference [--threads N] [--steps 3]

One step is the propagation loop body of ``CCSD_Helper.py:1206-1240``
(``ft1``/``ft2``/``fL1``/``fL2`` from ``CCSD_Helper.py:1158-1187`` and
``dipole_moment`` from ``CCSD_Helper.py:1066-1092``), run through the
reference's ``CCSD_Helper`` (psi4/pandas replaced by empty stub modules, the
helper built with ``__new__`` and given the seeded integrals, the discarded
HF density stubbed), against ``CCOracle.rk4_step`` + ``dipole_moment`` on the
same state, field and integrals, both in complex128 with ``--threads`` BLAS
threads.  The two mu_z sequences are compared as a sanity check.  One
further, untimed reference step counts the algorithmic flops of the
reference's own contractions: every ``opt_einsum.contract`` call the loop
body makes is costed by ``opt_einsum.contract_path`` (its ``opt_cost``, about
2 x multiply-adds), times 2 when one operand is complex and 4 when two or
more are.  The result is merged into ``oracle/port_calibration.json`` under
the key ``<workload>/<threads>``.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("reference", help="path of the reference checkout (holds CCSD_Helper.py)")
    p.add_argument("--threads", type=int, default=os.cpu_count())
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--workload", default="ccsd_o10_v38")
    p.add_argument("--out", default=os.path.join(HERE, "port_calibration.json"))
    return p.parse_args()


ARGS = _args()
# BLAS threads are fixed before numpy loads
for _k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS"):
    os.environ[_k] = str(ARGS.threads)

import cmath  # noqa: E402

import numpy as np  # noqa: E402

sys.path.insert(0, ROOT)
from oracle.cc_oracle import CCOracle  # noqa: E402
from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system  # noqa: E402


def load_reference(ref_dir):
    stub_dir = tempfile.mkdtemp(prefix="refstubs_")
    for name in ("psi4", "pandas"):
        with open(os.path.join(stub_dir, name + ".py"), "w") as f:
            f.write("# empty stub: the reference's psi4/pandas uses are not exercised\n")
    sys.path.insert(0, stub_dir)
    sys.path.insert(1, ref_dir)
    sys.dont_write_bytecode = True
    import CCSD_Helper as mod
    return mod


def main():
    mod = load_reference(os.path.abspath(ARGS.reference))
    w = WORKLOADS[ARGS.workload]
    sysm = synthetic_system(**w)
    o, v, n = sysm.o, sysm.v, sysm.o + sysm.v
    tei = sysm.tei()
    mu = [np.asarray(m) for m in sysm.mu]
    F = sysm.fock
    h = mod.CCSD_Helper.__new__(mod.CCSD_Helper)
    h.occ, h.vir, h.TEI = slice(0, o), slice(o, n), tei
    h.Defd_dipole = lambda: mu
    h.Buildpho = lambda Fm: np.zeros((n, n))
    h.pholowdinbasis = lambda p: p
    orc = CCOracle(tei, o, mu=mu)

    t2 = mp2_guess(tei, sysm.eps(), o).astype(np.complex128)
    t1 = np.zeros((o, v), dtype=np.complex128)
    state0 = [t1, t2, t1.copy(), t2.copy()]
    A, w0, dt, precs = 0.002, 0.923, 0.005, 15
    mu_z = mu[2]

    def Vt(tt):  # the reference's own field form (CCSD_Helper.py:1196-1199)
        return -A * mu_z * cmath.exp(1j * w0 * 2 * np.pi * tt)

    def ref_step(st, tt):
        r = [np.around(x, decimals=precs) for x in st]
        d1 = -1j * h.ft1(tt, dt, st[0], st[1], F, Vt)
        d2 = -1j * h.ft2(tt, dt, st[0], st[1], F, Vt)
        e1 = 1j * h.fL1(tt, dt, st[0], st[1], st[2], st[3], F, Vt)
        e2 = 1j * h.fL2(tt, dt, st[0], st[1], st[2], st[3], F, Vt)
        st = [r[0] + d1, r[1] + d2, r[2] + e1, r[3] + e2]
        return st, h.dipole_moment(*st, F)[2]

    def port_step(st, tt):
        st = orc.rk4_step("CCSD", tt, dt, st, F, Vt, precs)
        return st, orc.dipole_moment(*st)[2]

    res = {}
    for name, fn in (("reference", ref_step), ("port", port_step)):
        st, tt = [x.copy() for x in state0], 0.0
        fn(st, dt)  # warm-up (BLAS thread pool, opt_einsum path cache)
        mus, t0 = [], time.perf_counter()
        for _ in range(ARGS.steps):
            tt += dt
            st, m = fn(st, tt)
            mus.append(m)
        el = time.perf_counter() - t0
        res[name] = {"steps_per_s": ARGS.steps / el, "seconds": el, "mu_z": [complex(x) for x in mus]}
    dmu = max(abs(a - b) for a, b in zip(res["reference"]["mu_z"], res["port"]["mu_z"]))

    # algorithmic flops of one reference step: cost every contract() call
    import opt_einsum
    counted = {"flops": 0.0, "calls": 0}
    plain = mod.contract

    def costed(eq, *ops, **kw):
        arrs = [x for x in ops if hasattr(x, "dtype")]
        nc = sum(1 for x in arrs if np.iscomplexobj(x))
        counted["flops"] += float(opt_einsum.contract_path(eq, *ops)[1].opt_cost) * (1, 2, 4)[min(nc, 2)]
        counted["calls"] += 1
        return plain(eq, *ops, **kw)

    mod.contract = costed
    try:
        ref_step([x.copy() for x in state0], dt)
    finally:
        mod.contract = plain
    entry = {
        "workload": ARGS.workload, "o": o, "v": v, "threads": ARGS.threads, "steps": ARGS.steps,
        "host": f"{platform.machine()} {os.cpu_count()} cores", "numpy": np.__version__,
        "reference_steps_per_s": res["reference"]["steps_per_s"], "port_steps_per_s": res["port"]["steps_per_s"],
        "reference_over_port": res["reference"]["steps_per_s"] / res["port"]["steps_per_s"],
        "max_dmu_reference_vs_port_au": dmu,
        "reference_flops_per_step": counted["flops"], "reference_contract_calls_per_step": counted["calls"],
    }
    try:
        import opt_einsum
        entry["opt_einsum"] = opt_einsum.__version__
    except ImportError:
        pass
    data = {}
    if os.path.exists(ARGS.out):
        with open(ARGS.out) as f:
            data = json.load(f)
    data[f"{ARGS.workload}/{ARGS.threads}"] = entry
    with open(ARGS.out, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
    print(json.dumps(entry))


if __name__ == "__main__":
    main()
