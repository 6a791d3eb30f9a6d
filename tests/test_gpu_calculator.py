"""``CC_Calculator`` end to end on the device: ground state, propagation,
timeout stop, restart -- against the oracle running the reference's loop."""
import numpy as np
import pytest

from golden_util import load
from python_code_to_check_c_gb300 import restart_io

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_tdcc_then_restart(tmp_path, method):
    from oracle.cc_oracle import CCOracle, reference_field
    from python_code_to_check_c_gb300.calculator import CC_Calculator
    d, sysm = load("golden_o4_v8.npz")
    w0, A, dt = 0.923, 0.002, 0.01
    calc = CC_Calculator(system=sysm, outdir=str(tmp_path), verbose=False, chunk=5,
                         w0=w0, A=A, t0=0.0, dt=dt, precs=15)
    # tf is 10.1; a zero time limit stops after the first chunk
    out = calc.TDCC(0.0, method)
    assert out["stopped"] and out["steps"] == 5
    sfx = "" if method == "CCSD" else "_cc2"
    st = [d["gs_" + k + sfx] + 0j for k in ("t1", "t2", "l1", "l2")]
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    Vt = reference_field(A, w0, sysm.mu[2])
    times, mus, _ = orc.propagate(method, sysm.fock, st, 0.0, dt, 5, Vt, 15)
    assert np.array_equal(out["times"], np.round(times[1:], 4))
    assert np.abs(out["mu"] - mus[1:]).max() < 1e-10
    p = restart_io.read_parameters(tmp_path / "Parameters.csv")
    assert p["CCSD_or_CC2"] == method and (p["i"], p["a"]) == (sysm.o, sysm.v)
    F, *saved = restart_io.load_restart(str(tmp_path), sysm.o, sysm.v)
    calc2 = CC_Calculator(system=sysm, outdir=str(tmp_path), verbose=False, chunk=5)
    out2 = calc2.TDCC_restart(0.0)
    assert out2["steps"] == 5
    times2, mus2, _ = orc.propagate(method, F, saved, p["t0"] + dt, dt, 5, Vt, 15)
    assert np.array_equal(out2["times"], np.round(times2[1:], 4))
    assert np.abs(out2["mu"] - mus2[1:]).max() < 1e-10
    assert len((tmp_path / "H2O.csv").read_text().splitlines()) == 11
    # timing.csv: per-step total, split between the four blocks by their device times
    rows = (tmp_path / "timing.csv").read_text().splitlines()
    assert rows[0] == ",total,t1,t2,l1,l2" and len(rows) == 11
    for r in rows[1:]:
        tot, *blk = (float(x) for x in r.split(",")[1:])
        assert tot > 0 and all(b > 0 for b in blk)
        assert abs(sum(blk) - tot) <= 1e-9 * tot
