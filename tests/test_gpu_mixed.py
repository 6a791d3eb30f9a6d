"""Mixed-precision form: contractions on the tensor cores as BF16 slice
products (FP32 accumulate), everything else FP64.  Checked against the
reference's golden residuals and against the FP64 GPU form.

Tolerances (written here, met with S = 5 slices per operand):
  residuals      relative 1e-9 (max |diff| / max |ref|); 1e-7 with S = 4
  mu_z(t)        |d mu| <= 1e-8 a.u. over the propagation vs the FP64 form
"""
import numpy as np
import pytest

from golden_util import CASES, load, rel_err

pytestmark = pytest.mark.gpu

RES_TOL = 1e-9
RES_TOL4 = 1e-7
MU_TOL = 1e-8


def _np(x):
    return x.detach().cpu().numpy()


@pytest.fixture(scope="module", params=CASES[:2])
def case(request):
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load(request.param)
    eng = CCEngine.from_system(sysm)
    eng.set_precision("mixed", 5)
    eng.set_tc_policy(0, 1, 1)  # every contraction on the tensor cores at these small sizes
    yield d, sysm, eng
    eng.close()


@pytest.mark.parametrize("name,fn,args", [
    ("T1", "T1eq_rhs", "t"), ("T2", "T2eq_rhs", "t"),
    ("L1", "lam_1eq_rhs", "l"), ("L2", "lam2eq_rhs", "l"),
    ("T2_CC2", "T2eq_rhs_CC2", "t"), ("L1_CC2", "L1eq_rhs_CC2", "l"), ("L2_CC2", "L2eq_rhs_CC2", "l"),
])
def test_mixed_residual_close_to_reference(case, name, fn, args):
    d, sysm, eng = case
    a = (d["t1"], d["t2"]) if args == "t" else (d["t1"], d["t2"], d["l1"], d["l2"])
    got = _np(getattr(eng, fn)(*a, d["F"]))
    eng.check_errors()
    err = rel_err(got, d[name])
    assert err < RES_TOL, (name, err)


def test_slices_control_the_error():
    """More slices, smaller error (until FP64 round-off)."""
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load("golden_o6_v10.npz")
    eng = CCEngine.from_system(sysm)
    errs = []
    eng.set_tc_policy(0, 1, 1)
    try:
        for S in (3, 4, 5, 6):
            eng.set_precision("mixed", S)
            got = _np(eng.lam2eq_rhs(d["t1"], d["t2"], d["l1"], d["l2"], d["F"]))
            eng.check_errors()
            errs.append(rel_err(got, d["L2"]))
    finally:
        eng.close()
    assert errs[0] > errs[2] and errs[1] > errs[2], errs
    assert errs[3] < 1e-10, errs


def test_mixed_large_contractions_use_tensor_cores():
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine, profile_step
    from python_code_to_check_c_gb300.system import synthetic_system
    sysm = synthetic_system(10, 38, 144, seed=1038)
    eng = CCEngine.from_system(sysm)
    try:
        eng.set_precision("mixed", 5)
        o, v = sysm.o, sysm.v
        rng = np.random.default_rng(3)
        st = (0.01 * rng.standard_normal((o, v)) + 0j, 0.01 * rng.standard_normal((o, o, v, v)) + 0j,
              0.01 * rng.standard_normal((o, v)) + 0j, 0.01 * rng.standard_normal((o, o, v, v)) + 0j)
        recs = profile_step(eng, "CCSD", st, 0.0, 0.005, make_field("sin", 0.002, 0.923))
        tc = [r for r in recs if r["backend"] == 1 and r["kind"] == 0]
        f64 = [r for r in recs if r["backend"] == 0 and r["kind"] == 0]
        assert tc, "no tensor-core contraction in the mixed step"
        assert sum(r["flops"] for r in tc) > 20 * sum(r["flops"] for r in f64)
        eng.check_errors()
    finally:
        eng.close()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_mixed_trajectory_o10_v14(method):
    """200 steps (dt 0.01, E = 0.002 sin(0.923 t)) from a converged ground state."""
    from oracle.cc_oracle import CCOracle
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import WORKLOADS, synthetic_system
    sysm = synthetic_system(**WORKLOADS["ccsd_o10_v14"])
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    F = sysm.fock
    t1 = np.zeros((sysm.o, sysm.v))
    E, t1, t2 = orc.DIIS_solver(t1, orc.MP2_guess(F), F, 8, 40, 1e-15, method=method)
    El, l1, l2 = orc.DIIS_solver_Lam(t1, t2, t1, t2, F, 8, 30, 1e-15, method=method)
    gs = tuple(x + 0j for x in (t1, t2, l1, l2))
    f = make_field("sin", 0.002, 0.923)
    eng = CCEngine.from_system(sysm)
    try:
        _, mu64 = eng.propagate(method, gs, 0.0, 0.01, 200, f)
        eng.set_precision("mixed", 5)
        _, mumx = eng.propagate(method, gs, 0.0, 0.01, 200, f)
        eng.check_errors()
    finally:
        eng.close()
    err = np.abs(_np(mumx) - _np(mu64)).max()
    assert err < MU_TOL, err


@pytest.mark.parametrize("fn,name,args", [("T2eq_rhs", "T2", "t"), ("lam_1eq_rhs", "L1", "l"),
                                          ("lam2eq_rhs", "L2", "l"), ("L1eq_rhs_CC2", "L1_CC2", "l")])
def test_short_contractions_on_the_fp32_pipe(fn, name, args):
    """Slice products on the FP32 pipe (tensor cores off, every contraction
    with K <= 64 on the SIMT path): the residuals meet the same bar, the
    error shrinks with more slices, and the path is really taken."""
    from python_code_to_check_c_gb300.engine import CCEngine, profile_step
    from python_code_to_check_c_gb300._lib import make_field
    d, sysm = load("golden_o6_v10.npz")
    eng = CCEngine.from_system(sysm)
    try:
        eng.set_tc_policy(1 << 62, 1 << 30, 1)  # nothing on the tensor cores
        eng.set_simt_policy(64, 0)
        a = (d["t1"], d["t2"]) if args == "t" else (d["t1"], d["t2"], d["l1"], d["l2"])
        errs = []
        for S in (4, 5, 6):  # the FP32-pipe path takes 4, 5 or 6 slices
            eng.set_precision("mixed", S)
            got = _np(getattr(eng, fn)(*a, d["F"]))
            errs.append(rel_err(got, d[name]))
        assert errs[0] < RES_TOL4, errs
        assert errs[1] < RES_TOL, errs
        assert errs[0] > errs[1] > errs[2], errs
        st = [d["t1"] + 0j, d["t2"] + 0j, d["l1"] + 0j, d["l2"] + 0j]
        recs = profile_step(eng, "CCSD", st, 0.0, 0.01, make_field("sin", 0.002, 0.923))
        assert sum(1 for r in recs if r["kind"] == 0 and r["backend"] == 2) >= 10
    finally:
        eng.close()


def test_simt_path_keeps_trajectories():
    """Default routing (tensor cores for the large contractions, the FP32
    pipe for the short ones) against the same without the FP32-pipe path."""
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load("golden_o6_v10.npz")
    st = [d["t1"] + 0j, d["t2"] + 0j, d["l1"] + 0j, d["l2"] + 0j]
    out = []
    for max_k in (64, 0):
        eng = CCEngine.from_system(sysm)
        try:
            eng.set_precision("mixed", 5)
            eng.set_tc_policy(1 << 16, 32, 1)
            eng.set_simt_policy(max_k, 0)
            _, traj = eng.propagate("CCSD", st, 0.0, 0.01, 20, make_field("sin", 0.005, 0.923))
            eng.check_errors()
            out.append(_np(traj))
        finally:
            eng.close()
    assert np.abs(out[0] - out[1]).max() < MU_TOL
