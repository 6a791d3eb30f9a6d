"""Long-run accuracy of the mixed-precision form (TD-CCSD and TD-CC2 at
o=10, v=38, Q=144): 2000 RK4 steps, dt = 0.005, E(t) = 0.002 sin(0.923 t)
along z, from the device-DIIS ground state (8 vectors, max residual 1e-10).

Bars (written here): |mu_mixed(t) - mu_fp64(t)| <= 1e-8 a.u. at every step,
with 5 and with 4 slices per operand;
a ground state converged with the mixed-precision contractions within
1e-8 Eh of the FP64 one (the FP64 form is what the parity bar of 1e-10 Eh
applies to; propagation starts from the FP64 ground state).  The final
||t2_mixed - t2_fp64|| and |dE| are printed with the other numbers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NSTEPS = 2000


def _np(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_mixed_2000_steps_o10_v38(method):
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system
    sysm = synthetic_system(**WORKLOADS["ccsd_o10_v38"])
    eng = CCEngine.from_system(sysm)
    try:
        t2 = mp2_guess(sysm.tei(), np.linalg.eigh(sysm.fock)[0], sysm.o)
        t1 = np.zeros((sysm.o, sysm.v))
        E64, _, t1g, t2g = eng.ground_state(method, 0, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
        El64, _, l1g, l2g = eng.ground_state(method, 1, t1g, t2g, t1g, t2g, maxsize=8, maxiter=100, E_min=0.0,
                                             r_tol=1e-10)
        gs = (t1g, t2g, l1g, l2g)
        f = make_field("sin", 0.002, 0.923)
        fin64, mu64 = eng.propagate(method, gs, 0.0, 0.005, NSTEPS, f)
        eng.set_precision("mixed", 4)
        _, mum4 = eng.propagate(method, gs, 0.0, 0.005, NSTEPS, f)
        eng.set_precision("mixed", 5)
        Emx, _, _, _ = eng.ground_state(method, 0, t1, t2, maxsize=8, maxiter=100, E_min=0.0, r_tol=1e-10)
        finmx, mumx = eng.propagate(method, gs, 0.0, 0.005, NSTEPS, f)
        eng.check_errors()
    finally:
        eng.close()
    dmu4 = np.abs(_np(mum4) - _np(mu64))
    print(f"{method} (4 slices): max|dmu| {dmu4.max():.3e} a.u. (at step {int(dmu4.argmax()) + 1})")
    assert np.isfinite(dmu4).all()
    assert dmu4.max() <= 1e-8
    dmu = np.abs(_np(mumx) - _np(mu64))
    dt2 = float(np.linalg.norm(_np(finmx[1]) - _np(fin64[1])))
    print(f"{method}: max|dmu| {dmu.max():.3e} a.u. (at step {int(dmu.argmax()) + 1}), final ||dt2|| {dt2:.3e}, "
          f"|dE| {abs(Emx - E64):.3e} Eh, E_corr {E64:.12f}, pseudo-E {El64:.12f}")
    assert np.isfinite(dmu).all()
    assert dmu.max() <= 1e-8
    assert abs(Emx - E64) <= 1e-8
