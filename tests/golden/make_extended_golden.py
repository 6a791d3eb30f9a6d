"""Fixture bounding the FP64 form against the reference's production
precision: the reference runs its propagation in numpy's extended type
(``t1 = zeros(longdouble)``, CC_Calculator.py:170; the state becomes
clongdouble at the first field add).  This script runs the reference's own
block-frozen RK4 functions (``ft1/ft2/fL1/fL2`` and the CC2 variants) in the
loop body of CCSD_Helper.py:1206-1240 twice -- clongdouble and complex128 --
from the golden o=4, v=8 ground states, with the reference's field
Vt(t) = -A mu_z exp(i 2 pi w0 t), 20 steps, precs = 15:

    python tests/golden/make_extended_golden.py /path/to/reference

Output: ``golden_o4_v8_extended.npz`` (mu_z(t) of both runs, CCSD and CC2).
"""
from __future__ import annotations

import cmath
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_golden as mg  # noqa: E402

STEPS, DT, A, W0, PRECS = 20, 0.01, 0.005, 0.968635, 15


def run(h, F, mu_z, st, method, dtype):
    def Vt(tt):
        return -A * mu_z * cmath.exp(1j * W0 * 2 * np.pi * tt)

    if method == "CCSD":
        f2, fl1, fl2 = h.ft2, h.fL1, h.fL2
    else:
        f2, fl1, fl2 = h.ft2_CC2, h.fL1_CC2, h.fL2_CC2
    st = [np.asarray(x, dtype=dtype) for x in st]
    tt = 0.0
    mus = [complex(h.dipole_moment(*st, F)[2])]
    for _ in range(STEPS):
        r = [np.around(x, decimals=PRECS) for x in st]
        tt += DT
        d1 = -1j * h.ft1(tt, DT, st[0], st[1], F, Vt)
        d2 = -1j * f2(tt, DT, st[0], st[1], F, Vt)
        e1 = 1j * fl1(tt, DT, st[0], st[1], st[2], st[3], F, Vt)
        e2 = 1j * fl2(tt, DT, st[0], st[1], st[2], st[3], F, Vt)
        st = [(r[0] + d1).astype(dtype), (r[1] + d2).astype(dtype), (r[2] + e1).astype(dtype),
              (r[3] + e2).astype(dtype)]
        mus.append(complex(h.dipole_moment(*st, F)[2]))
    return np.array(mus)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_extended_golden.py <path of the reference checkout>")
    ref_dir = sys.argv[1]
    mod = mg.load_reference(ref_dir)
    g = np.load(os.path.join(HERE, "golden_o4_v8.npz"))
    sysm = mg.synthetic_system(int(g["o"]), int(g["v"]), int(g["nq"]), int(g["seed"]))
    mu = [np.asarray(m) for m in sysm.mu]
    h = mg.make_helper(mod, sysm.tei(), sysm.o, mu)
    out = dict(steps=STEPS, dt=DT, A=A, w0=W0, precs=PRECS)
    for method, sfx in (("CCSD", ""), ("CC2", "_cc2")):
        st = [g["gs_" + k + sfx] for k in ("t1", "t2", "l1", "l2")]
        for name, dtype in (("c128", np.complex128), ("cld", np.clongdouble)):
            out[f"mu_{method}_{name}"] = run(h, sysm.fock, mu[2], st, method, dtype)
        d = np.abs(out[f"mu_{method}_c128"] - out[f"mu_{method}_cld"]).max()
        print(method, "max |mu(complex128) - mu(clongdouble)| =", d)
    path = os.path.join(HERE, "golden_o4_v8_extended.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
