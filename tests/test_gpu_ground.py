"""Ground-state DIIS on the device against the reference's own DIIS results
(golden, o=4 v=8) and the CPU oracle (o=10 v=14).  Energy bar 1e-10 Eh."""
import numpy as np
import pytest

from golden_util import load, rel_err

pytestmark = pytest.mark.gpu


def _np(x):
    return x.detach().cpu().numpy()


@pytest.fixture(scope="module")
def small():
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load("golden_o4_v8.npz")
    eng = CCEngine.from_system(sysm)
    yield d, sysm, eng
    eng.close()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_diis_matches_reference_golden(small, method):
    from python_code_to_check_c_gb300.system import mp2_guess
    d, sysm, eng = small
    sfx = "_ccsd" if method == "CCSD" else "_cc2"
    asfx = "" if method == "CCSD" else "_cc2"
    t2 = mp2_guess(sysm.tei(), np.linalg.eigh(sysm.fock)[0], sysm.o)
    t1 = np.zeros((sysm.o, sysm.v))
    E, t1, t2 = eng.DIIS_solver(t1, t2, maxsize=7, maxiter=40, E_min=1e-15, method=method)
    assert abs(E - float(d["gs_E" + sfx])) < 1e-10
    assert rel_err(_np(t1).real, d["gs_t1" + asfx]) < 1e-8
    assert rel_err(_np(t2).real, d["gs_t2" + asfx]) < 1e-8
    El, l1, l2 = eng.DIIS_solver_Lam(t1, t2, t1, t2, maxsize=7, maxiter=30, E_min=1e-15, method=method)
    assert abs(El - float(d["gs_pseudo" + sfx])) < 1e-10
    assert rel_err(_np(l1).real, d["gs_l1" + asfx]) < 1e-8
    assert rel_err(_np(l2).real, d["gs_l2" + asfx]) < 1e-8


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_diis_matches_oracle_o10_v14(method):
    from oracle.cc_oracle import CCOracle
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    sysm = synthetic_system(**WORKLOADS["ccsd_o10_v14"])
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    F = sysm.fock
    t2 = orc.MP2_guess(F)
    t1 = np.zeros((sysm.o, sysm.v))
    E, t1r, t2r = orc.DIIS_solver(t1, t2, F, 7, 40, 1e-15, method=method)
    El, l1r, l2r = orc.DIIS_solver_Lam(t1r, t2r, t1r, t2r, F, 7, 30, 1e-15, method=method)
    eng = CCEngine.from_system(sysm)
    try:
        Eg, t1g, t2g = eng.DIIS_solver(t1, t2, method=method)
        Elg, l1g, l2g = eng.DIIS_solver_Lam(t1g, t2g, t1g, t2g, method=method)
        assert abs(Eg - E) < 1e-10
        assert abs(Elg - El) < 1e-10
        assert rel_err(_np(l2g).real, l2r) < 1e-8
    finally:
        eng.close()


def test_residual_tolerance_and_mixed_precision():
    """r_tol stops on the residual; the mixed-precision contractions give the
    same converged energy."""
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system
    sysm = synthetic_system(**WORKLOADS["ccsd_o10_v14"])
    t2 = mp2_guess(sysm.tei(), np.linalg.eigh(sysm.fock)[0], sysm.o)
    t1 = np.zeros((sysm.o, sysm.v))
    eng = CCEngine.from_system(sysm)
    try:
        E0, n0, _, _ = eng.ground_state("CCSD", 0, t1, t2, maxiter=40, E_min=1e-15)
        E1, n1, _, _ = eng.ground_state("CCSD", 0, t1, t2, maxiter=60, E_min=0.0, r_tol=1e-11)
        assert abs(E1 - E0) < 1e-10 and n1 <= 60
        eng.set_precision("mixed", 5)
        eng.set_tc_policy(0, 1, 1)
        E2, _, _, _ = eng.ground_state("CCSD", 0, t1, t2, maxiter=40, E_min=1e-15)
        eng.check_errors()
        assert abs(E2 - E0) < 1e-10
    finally:
        eng.close()
