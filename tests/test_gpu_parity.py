"""GPU residuals, intermediates-driven RHS and dipole against the reference's
golden outputs and the CPU oracle (FP64 path; tolerance 1e-12 relative)."""
import numpy as np
import pytest

from golden_util import CASES, load, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, FP64 plain form vs the reference's numpy path


@pytest.fixture(scope="module", params=CASES)
def case(request):
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load(request.param)
    eng = CCEngine.from_system(sysm)
    yield d, sysm, eng
    eng.close()


def _np(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("name,fn,args", [
    ("T1", "T1eq_rhs", "t"), ("T2", "T2eq_rhs", "t"),
    ("L1", "lam_1eq_rhs", "l"), ("L2", "lam2eq_rhs", "l"),
    ("T2_CC2", "T2eq_rhs_CC2", "t"), ("L1_CC2", "L1eq_rhs_CC2", "l"), ("L2_CC2", "L2eq_rhs_CC2", "l"),
])
def test_residual_matches_reference(case, name, fn, args):
    d, sysm, eng = case
    a = (d["t1"], d["t2"]) if args == "t" else (d["t1"], d["t2"], d["l1"], d["l2"])
    got = _np(getattr(eng, fn)(*a, d["F"]))
    assert rel_err(got, d[name]) < TOL, name


def test_t1_block_of_cc2_is_ccsd_t1(case):
    from python_code_to_check_c_gb300.engine import TDCC_T1
    d, sysm, eng = case
    got = _np(eng.rhs("CC2", TDCC_T1, d["t1"], d["t2"], F=d["F"]))
    assert rel_err(got, d["T1"]) < TOL


def test_dipole_matches_reference(case):
    d, sysm, eng = case
    mu = _np(eng.dipole_moment(d["t1"], d["t2"], d["l1"], d["l2"]))
    assert np.abs(mu[2] - d["mu"][2]) < 1e-14
    assert np.abs(mu[:2]).max() == 0.0


def test_repeated_calls_are_stable(case):
    d, sysm, eng = case
    a = _np(eng.T2eq_rhs(d["t1"], d["t2"], d["F"]))
    b = _np(eng.T2eq_rhs(d["t1"], d["t2"], d["F"]))
    assert rel_err(a, b) < 1e-14


def test_real_fock_input(case):
    from oracle.cc_oracle import CCOracle
    d, sysm, eng = case
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    F = sysm.fock
    got = _np(eng.lam2eq_rhs(d["t1"], d["t2"], d["l1"], d["l2"], F))
    assert rel_err(got, orc.lam2eq_rhs(d["t1"], d["t2"], d["l1"], d["l2"], F)) < TOL
