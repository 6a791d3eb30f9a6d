"""Block-frozen RK4 propagation on the GPU against the reference's own
trajectory (golden) and the CPU oracle.  FP64 path.

Tolerances: one step 1e-12 relative on the state; mu_z(t) 1e-10 a.u.
absolute over 200 steps (o=10, v=14, dt=0.01, E(t) = 0.002 sin(0.923 t))."""
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
def test_one_step_matches_oracle(small, method):
    from oracle.cc_oracle import CCOracle, reference_field
    from python_code_to_check_c_gb300._lib import make_field
    d, sysm, eng = small
    A, w0, dt = float(d["traj_A"]), float(d["traj_w0"]), float(d["traj_dt"])
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    st = (d["t1"], d["t2"], d["l1"], d["l2"])
    ref = orc.rk4_step(method, 0.0 + dt, dt, st, sysm.fock, reference_field(A, w0, sysm.mu[2]), 15)
    new, mu = eng.rk4_step(method, st, 0.0, dt, make_field("reference", A, w0), precs=15)
    for a, b in zip(new, ref):
        assert rel_err(_np(a), b) < 1e-12
    assert abs(_np(mu)[2] - orc.dipole_moment(*ref)[2]) < 1e-14


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_trajectory_matches_reference_golden(small, method):
    """6 steps of the reference's own loop body (golden) from its ground state."""
    from python_code_to_check_c_gb300._lib import make_field
    d, sysm, eng = small
    A, w0, dt = float(d["traj_A"]), float(d["traj_w0"]), float(d["traj_dt"])
    sfx = "" if method == "CCSD" else "_cc2"
    st = tuple(d["gs_" + k + sfx] + 0j for k in ("t1", "t2", "l1", "l2"))
    final, traj = eng.propagate(method, st, 0.0, dt, 6, make_field("reference", A, w0), precs=15)
    ref = d["traj_mu_" + method]
    assert np.abs(_np(traj) - ref[1:]).max() < 1e-12
    assert rel_err(_np(final[1]), d["traj_final_t2_" + method]) < 1e-10


def test_graph_propagation_equals_step_loop(small):
    from python_code_to_check_c_gb300._lib import make_field
    d, sysm, eng = small
    f = make_field("sin", 0.002, 0.923)
    st = (d["t1"], d["t2"], d["l1"], d["l2"])
    final, traj = eng.propagate("CCSD", st, 0.0, 0.01, 5, f, precs=15)
    s = st
    t = 0.0
    mus = []
    for _ in range(5):
        s, mu = eng.rk4_step("CCSD", s, t, 0.01, f, precs=15)
        t += 0.01
        mus.append(_np(mu)[2])
    assert np.abs(_np(traj) - np.array(mus)).max() < 1e-15
    for a, b in zip(final, s):
        assert rel_err(_np(a), _np(b)) < 1e-15


@pytest.fixture(scope="module")
def water_size():
    """o=10, v=14 synthetic system with its CCSD / CC2 ground states (oracle DIIS, 8 vectors)."""
    from oracle.cc_oracle import CCOracle
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    sysm = synthetic_system(**WORKLOADS["ccsd_o10_v14"])
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    F = sysm.fock
    gs = {}
    for method in ("CCSD", "CC2"):
        t1 = np.zeros((sysm.o, sysm.v))
        E, t1, t2 = orc.DIIS_solver(t1, orc.MP2_guess(F), F, 8, 40, 1e-15, method=method)
        El, l1, l2 = orc.DIIS_solver_Lam(t1, t2, t1, t2, F, 8, 30, 1e-15, method=method)
        gs[method] = tuple(x + 0j for x in (t1, t2, l1, l2))
    return sysm, orc, gs


@pytest.mark.parametrize("method,nsteps", [("CCSD", 200), ("CC2", 200)])
def test_200_step_dipole_matches_oracle(water_size, method, nsteps):
    from oracle.cc_oracle import sin_field
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    sysm, orc, gs = water_size
    dt, A, w0 = 0.01, 0.002, 0.923
    _, mus_ref, st_ref = orc.propagate(method, sysm.fock, gs[method], 0.0, dt, nsteps,
                                       sin_field(A, w0, sysm.mu[2]), precs=15)
    eng = CCEngine.from_system(sysm)
    try:
        final, traj = eng.propagate(method, gs[method], 0.0, dt, nsteps, make_field("sin", A, w0), precs=15)
    finally:
        pass
    err = np.abs(_np(traj) - mus_ref[1:]).max()
    assert err < 1e-10, err
    assert rel_err(_np(final[1]), st_ref[1]) < 1e-9
    eng.close()
