"""Parity against the CPU oracle at the benchmark sizes: o=10, v=38 (Q=144,
seed 1038) and o=10, v=14 (Q=72, seed 1014).

At v=38 the contractions take the launch shapes the golden sizes never
reach: several output tiles per product, split K, tensor-core slice
products whose K (v^2 = 1444 for the ladders) crosses several 512-wide
chunks with partial sums parked in TMEM, and the FP32-pipe slice products
for K = o and K = v.  Every residual of both methods is compared with the
oracle (numpy complex128, CCSD_Helper.py:177-648, CC2_Helper.py:12-175) on
seeded complex amplitudes and a complex dressed Fock matrix; then 20 steps
of the reference loop body (CCSD_Helper.py:1206-1240) from the device-DIIS
ground state.

Tolerances (written here):
  FP64 form   residuals 1e-12 relative (max |diff| / max |ref|); dipole
              1e-14 a.u.; mu_z(t) over 20 steps 1e-10 a.u.
  mixed form  5 slices per operand: residuals 1e-9 relative; 4 slices:
              residuals 1e-7 relative; mu_z(t) over 20 steps 1e-8 a.u. with
              either
"""
import numpy as np
import pytest

from golden_util import rel_err

pytestmark = pytest.mark.gpu

RES_FP64 = 1e-12
RES_MIXED = 1e-9
RES_MIXED4 = 1e-7
MU_FP64 = 1e-10
MU_MIXED = 1e-8

RESIDUALS = [
    ("CCSD", "T1eq_rhs", "t"), ("CCSD", "T2eq_rhs", "t"),
    ("CCSD", "lam_1eq_rhs", "l"), ("CCSD", "lam2eq_rhs", "l"),
    ("CC2", "T2eq_rhs_CC2", "t"), ("CC2", "L1eq_rhs_CC2", "l"), ("CC2", "L2eq_rhs_CC2", "l"),
]


def _np(x):
    return x.detach().cpu().numpy()


def _state(o, v, seed):
    """Complex amplitudes of ground-state magnitude with phases, as a
    propagation produces them."""
    rng = np.random.default_rng(seed)

    def c(shape, s):
        return s * (rng.standard_normal(shape) + 0.5j * rng.standard_normal(shape))

    return c((o, v), 0.02), c((o, o, v, v), 0.01), c((o, v), 0.02), c((o, o, v, v), 0.01)


def _system(name):
    from oracle.cc_oracle import CCOracle
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    sysm = synthetic_system(**WORKLOADS[name])
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    # dressed Fock of a field sample: complex, as in the reference's F + Vt
    F = sysm.fock + (-0.004 + 0.003j) * sysm.mu[2]
    return sysm, orc, F


@pytest.fixture(scope="module", params=["ccsd_o10_v38", "ccsd_o10_v14"])
def sized(request):
    sysm, orc, F = _system(request.param)
    st = _state(sysm.o, sysm.v, 38)
    refs = {}
    for method, fn, args in RESIDUALS:
        a = st[:2] if args == "t" else st
        refs[fn] = getattr(orc, fn)(*a, F)
    refs["mu"] = orc.dipole_moment(*st)
    return request.param, sysm, orc, F, st, refs


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed4"])
def test_every_residual_matches_oracle(sized, precision):
    from python_code_to_check_c_gb300.engine import CCEngine
    name, sysm, orc, F, st, refs = sized
    eng = CCEngine.from_system(sysm)
    errs = {}
    try:
        if precision != "fp64":
            eng.set_precision("mixed", 4 if precision == "mixed4" else 5)
        for method, fn, args in RESIDUALS:
            a = st[:2] if args == "t" else st
            errs[fn] = rel_err(_np(getattr(eng, fn)(*a, F)), refs[fn])
        eng.check_errors()
    finally:
        eng.close()
    tol = {"fp64": RES_FP64, "mixed": RES_MIXED, "mixed4": RES_MIXED4}[precision]
    print(name, precision, {k: f"{e:.2e}" for k, e in errs.items()})
    bad = {k: e for k, e in errs.items() if not e < tol}
    assert not bad, bad


def test_dipole_matches_oracle(sized):
    from python_code_to_check_c_gb300.engine import CCEngine
    name, sysm, orc, F, st, refs = sized
    eng = CCEngine.from_system(sysm)
    try:
        mu = _np(eng.dipole_moment(*st))
    finally:
        eng.close()
    assert np.abs(mu[2] - refs["mu"][2]) < 1e-14


def test_mixed_residuals_with_every_contraction_on_the_tensor_cores():
    """o=10, v=38 with every contraction of at least 4096 multiply-adds and
    K >= 16 routed to the tensor-core slice products (no FP32-pipe path):
    the one-K-block and multi-chunk launches of every residual."""
    from python_code_to_check_c_gb300.engine import CCEngine
    sysm, orc, F = _system("ccsd_o10_v38")
    st = _state(sysm.o, sysm.v, 39)
    eng = CCEngine.from_system(sysm)
    errs = {}
    try:
        eng.set_precision("mixed", 5)
        eng.set_tc_policy(1 << 12, 16, 1)
        eng.set_simt_policy(0, 0)
        for method, fn, args in RESIDUALS:
            a = st[:2] if args == "t" else st
            errs[fn] = rel_err(_np(getattr(eng, fn)(*a, F)), getattr(orc, fn)(*a, F))
        eng.check_errors()
    finally:
        eng.close()
    print({k: f"{e:.2e}" for k, e in errs.items()})
    bad = {k: e for k, e in errs.items() if not e < RES_MIXED}
    assert not bad, bad


@pytest.fixture(scope="module")
def ground_o10_v38():
    """FP64 device-DIIS ground states (8 vectors, max residual 1e-10) of both
    methods at o=10, v=38; the device DIIS itself is pinned to the oracle and
    the reference's golden energies elsewhere."""
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import mp2_guess
    sysm, orc, _ = _system("ccsd_o10_v38")
    eng = CCEngine.from_system(sysm)
    gs = {}
    try:
        t2 = mp2_guess(sysm.tei(), np.linalg.eigh(sysm.fock)[0], sysm.o)
        t1 = np.zeros((sysm.o, sysm.v))
        for method in ("CCSD", "CC2"):
            _, _, t1g, t2g = eng.ground_state(method, 0, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
            _, _, l1g, l2g = eng.ground_state(method, 1, t1g, t2g, t1g, t2g, maxsize=8, maxiter=100, E_min=0.0,
                                              r_tol=1e-10)
            gs[method] = tuple(_np(x) for x in (t1g, t2g, l1g, l2g))
    finally:
        eng.close()
    return sysm, orc, gs


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_20_step_dipole_trace_matches_oracle(ground_o10_v38, method):
    """mu_z(t) of 20 steps (dt = 0.005, E(t) = 0.002 sin(0.923 t) along z)
    from the ground state: FP64 and mixed forms against the oracle's loop."""
    from oracle.cc_oracle import sin_field
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    sysm, orc, gs = ground_o10_v38
    nsteps, dt, A, w0 = 20, 0.005, 0.002, 0.923
    _, mus_ref, st_ref = orc.propagate(method, sysm.fock, gs[method], 0.0, dt, nsteps,
                                       sin_field(A, w0, sysm.mu[2]), precs=15)
    eng = CCEngine.from_system(sysm)
    try:
        f = make_field("sin", A, w0)
        fin64, mu64 = eng.propagate(method, gs[method], 0.0, dt, nsteps, f)
        eng.set_precision("mixed", 5)
        finmx, mumx = eng.propagate(method, gs[method], 0.0, dt, nsteps, f)
        eng.set_precision("mixed", 4)
        _, mum4 = eng.propagate(method, gs[method], 0.0, dt, nsteps, f)
        eng.check_errors()
    finally:
        eng.close()
    e64 = np.abs(_np(mu64) - mus_ref[1:]).max()
    emx = np.abs(_np(mumx) - mus_ref[1:]).max()
    em4 = np.abs(_np(mum4) - mus_ref[1:]).max()
    print(f"{method}: max|dmu| fp64 {e64:.2e}, mixed {emx:.2e}, mixed (4 slices) {em4:.2e} a.u.; "
          f"t2 rel fp64 {rel_err(_np(fin64[1]), st_ref[1]):.2e}, mixed {rel_err(_np(finmx[1]), st_ref[1]):.2e}")
    assert e64 < MU_FP64
    assert emx < MU_MIXED
    assert em4 < MU_MIXED
    assert rel_err(_np(fin64[1]), st_ref[1]) < 1e-10
