"""Runs one right-hand side (or one RK4 step) of a named workload on the GPU,
for profilers:  python bench_cases/profile_case.py
    --workload o14_v58 --method CCSD --block T2 [--repeat 2] [--step] [--nb 8]
    [--precision mixed --slices 4]"""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import argparse

import numpy as np
import torch

from python_code_to_check_c_gb300 import _lib
from python_code_to_check_c_gb300.engine import CCEngine
from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="o14_v58")
    p.add_argument("--method", default="CCSD")
    p.add_argument("--block", default="T2", choices=["T1", "T2", "L1", "L2"])
    p.add_argument("--repeat", type=int, default=2)
    p.add_argument("--step", action="store_true", help="one RK4 step instead of one RHS")
    p.add_argument("--precision", default="fp64")
    p.add_argument("--slices", type=int, default=4, help="slices per operand in the mixed form")
    p.add_argument("--nb", type=int, default=1, help="trajectories advanced together")
    a = p.parse_args()
    sysm = synthetic_system(**WORKLOADS[a.workload])
    eng = CCEngine.from_system(sysm, nb=a.nb)
    eng.set_precision(a.precision, a.slices)
    t2 = mp2_guess(sysm.tei(), sysm.eps(), sysm.o).astype(np.complex128)
    t1 = np.full((sysm.o, sysm.v), 0.01 + 0.005j)
    st = (t1, t2, t1.copy(), t2.copy())
    if a.nb > 1:
        st = tuple(np.broadcast_to(x, (a.nb,) + x.shape).copy() for x in st)
    F = sysm.fock if a.nb == 1 else np.broadcast_to(sysm.fock, (a.nb, sysm.n, sysm.n)).copy()
    blk = {"T1": 0, "T2": 1, "L1": 2, "L2": 3}[a.block]
    for _ in range(a.repeat):
        if a.step:
            eng.rk4_step(a.method, st, 0.0, 0.005, _lib.make_field("sin", 0.002, 0.923))
        else:
            eng.rhs(a.method, blk, *st, F=F)
    torch.cuda.synchronize()
    print("ok", a.workload, a.method, a.block, "step" if a.step else "rhs")


if __name__ == "__main__":
    main()
