"""Pins the CPU oracle to outputs of the reference's own code (golden
fixtures made by ``tests/golden/make_golden.py``).  CPU only."""
import math

import numpy as np
import pytest

from golden_util import CASES, load, rel_err
from oracle.cc_oracle import CCOracle, reference_field

TOL = 1e-12


@pytest.fixture(scope="module", params=CASES)
def case(request):
    d, sysm = load(request.param)
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    return d, sysm, orc


def test_residuals_match_reference(case):
    d, sysm, orc = case
    t1, t2, l1, l2, F = d["t1"], d["t2"], d["l1"], d["l2"], d["F"]
    assert rel_err(orc.T1eq_rhs(t1, t2, F), d["T1"]) < TOL
    assert rel_err(orc.T2eq_rhs(t1, t2, F), d["T2"]) < TOL
    assert rel_err(orc.lam_1eq_rhs(t1, t2, l1, l2, F), d["L1"]) < TOL
    assert rel_err(orc.lam2eq_rhs(t1, t2, l1, l2, F), d["L2"]) < TOL
    assert rel_err(orc.T2eq_rhs_CC2(t1, t2, F), d["T2_CC2"]) < TOL
    assert rel_err(orc.L1eq_rhs_CC2(t1, t2, l1, l2, F), d["L1_CC2"]) < TOL
    assert rel_err(orc.L2eq_rhs_CC2(t1, t2, l1, l2, F), d["L2_CC2"]) < TOL


def test_density_and_dipole_match_reference(case):
    d, sysm, orc = case
    t1, t2, l1, l2 = d["t1"], d["t2"], d["l1"], d["l2"]
    assert rel_err(orc.Dij(t1, t2, l1, l2), d["Dij"]) < TOL
    assert rel_err(orc.Dab(t1, t2, l1, l2), d["Dab"]) < TOL
    assert rel_err(orc.Dai(t1, t2, l1, l2), d["Dai"]) < TOL
    mu = np.array(orc.dipole_moment(t1, t2, l1, l2))
    assert abs(mu[2] - d["mu"][2]) < 1e-14


def test_intermediates_match_reference():
    d, sysm = load("golden_o4_v8.npz")
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    t1, t2, l1, l2, F = d["t1"], d["t2"], d["l1"], d["l2"], d["F"]
    for name in ("Fae", "Fmi", "Fme", "Wmnij", "Wabef", "Wmbej", "LRFea", "LRFim",
                 "LSWieam", "LRWefam", "LRWibjm", "LSWmnij", "LSWabef", "Wmnij_2", "Wabef_2"):
        got = getattr(orc, name)(t1, t2, F)
        assert rel_err(got, d["I_" + name]) < TOL, name
    assert rel_err(orc.Gfe(t2, l2), d["I_Gfe"]) < TOL
    assert rel_err(orc.Gmn(t2, l2), d["I_Gmn"]) < TOL
    assert rel_err(orc.LWfiea(t1), d["I_LWfiea"]) < TOL
    assert rel_err(orc.LWmina(t1), d["I_LWmina"]) < TOL


def test_rk4_blocks_match_reference():
    d, sysm = load("golden_o4_v8.npz")
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    A, w0, dt = float(d["traj_A"]), float(d["traj_w0"]), float(d["traj_dt"])
    Vt = reference_field(A, w0, sysm.mu[2])
    F = sysm.fock
    t1, t2, l1, l2 = d["t1"], d["t2"], d["l1"], d["l2"]
    t = dt
    assert rel_err(orc.ft1(t, dt, t1, t2, F, Vt), d["rk_ft1"]) < TOL
    assert rel_err(orc.ft2(t, dt, t1, t2, F, Vt), d["rk_ft2"]) < TOL
    assert rel_err(orc.fL1(t, dt, t1, t2, l1, l2, F, Vt), d["rk_fL1"]) < TOL
    assert rel_err(orc.fL2(t, dt, t1, t2, l1, l2, F, Vt), d["rk_fL2"]) < TOL
    assert rel_err(orc.ft2_CC2(t, dt, t1, t2, F, Vt), d["rk_ft2_CC2"]) < TOL
    assert rel_err(orc.fL1_CC2(t, dt, t1, t2, l1, l2, F, Vt), d["rk_fL1_CC2"]) < TOL
    assert rel_err(orc.fL2_CC2(t, dt, t1, t2, l1, l2, F, Vt), d["rk_fL2_CC2"]) < TOL


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_trajectory_matches_reference(method):
    d, sysm = load("golden_o4_v8.npz")
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    A, w0, dt = float(d["traj_A"]), float(d["traj_w0"]), float(d["traj_dt"])
    Vt = reference_field(A, w0, sysm.mu[2])
    sfx = "" if method == "CCSD" else "_cc2"
    st = tuple(d["gs_" + k + sfx] + 0j for k in ("t1", "t2", "l1", "l2"))
    times, mus, st = orc.propagate(method, sysm.fock, st, 0.0, dt, 6, Vt, precs=15)
    ref = d["traj_mu_" + method]
    assert np.abs(mus - ref).max() < 1e-12
    assert rel_err(st[1], d["traj_final_t2_" + method]) < 1e-10


def test_ground_state_diis_matches_reference():
    d, sysm = load("golden_o4_v8.npz")
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    F = sysm.fock
    t2 = orc.MP2_guess(F)
    t1 = np.zeros((sysm.o, sysm.v))
    E, t1, t2 = orc.DIIS_solver(t1, t2, F, 7, 40, 1e-15)
    assert abs(E - float(d["gs_E_ccsd"])) < 1e-10
    El, l1, l2 = orc.DIIS_solver_Lam(t1, t2, t1, t2, F, 7, 30, 1e-15)
    assert abs(El - float(d["gs_pseudo_ccsd"])) < 1e-10
    t2 = orc.MP2_guess(F)
    t1 = np.zeros((sysm.o, sysm.v))
    Ec, t1, t2 = orc.DIIS_solver(t1, t2, F, 7, 40, 1e-15, method="CC2")
    assert abs(Ec - float(d["gs_E_cc2"])) < 1e-10
    Elc, l1, l2 = orc.DIIS_solver_Lam(t1, t2, t1, t2, F, 7, 30, 1e-15, method="CC2")
    assert abs(Elc - float(d["gs_pseudo_cc2"])) < 1e-10
    assert math.isfinite(E)
