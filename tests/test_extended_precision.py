"""The FP64 form against the reference's production precision (no GPU): the
reference propagates in numpy's extended type (clongdouble after the first
field add, CC_Calculator.py:170).  The fixture holds mu_z(t) of the
reference's own loop body (CCSD_Helper.py:1206-1240) over 20 steps at o=4,
v=8 run in clongdouble and in complex128 (tests/golden/make_extended_golden.py).
The oracle's complex128 run reproduces the reference's complex128 run, and
both stay within a few FP64 roundings of the extended run: the FP64 form
(pinned to the oracle at 1e-12 on the GPU) inherits that bound."""
import cmath
import os

import numpy as np
import pytest

from golden_util import load

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("method,sfx", [("CCSD", ""), ("CC2", "_cc2")])
def test_fp64_within_roundings_of_extended(method, sfx):
    from oracle.cc_oracle import CCOracle
    ext = np.load(os.path.join(HERE, "golden", "golden_o4_v8_extended.npz"))
    d, sysm = load("golden_o4_v8.npz")
    mu_z = sysm.mu[2]
    A, w0, dt, n, precs = float(ext["A"]), float(ext["w0"]), float(ext["dt"]), int(ext["steps"]), int(ext["precs"])

    def Vt(t):  # the reference's field, CCSD_Helper.py:1197-1200
        return -A * mu_z * cmath.exp(1j * w0 * 2 * np.pi * t)

    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    st = tuple(d["gs_" + k + sfx] + 0j for k in ("t1", "t2", "l1", "l2"))
    _, mus, _ = orc.propagate(method, sysm.fock, st, 0.0, dt, n, Vt, precs)
    c128, cld = ext[f"mu_{method}_c128"], ext[f"mu_{method}_cld"]
    scale = np.abs(cld).max()
    assert np.abs(mus - c128).max() <= 1e-14 * scale       # same arithmetic up to summation order
    assert np.abs(c128 - cld).max() <= 1e-14 * scale       # the reference: FP64 vs extended
    assert np.abs(mus - cld).max() <= 1e-14 * scale        # the oracle vs the production precision
