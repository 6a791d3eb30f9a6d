"""Reverse mode on the device: gradients of J = sum_n dt cos(0.8 t_n) Re mu_z(t_n)
with respect to the pulse parameters (A, w0, envelope coefficients c_k)
against central finite differences of the forward propagation (h = 1e-5,
relative 1e-6), and dJ/d(initial state) against a directional difference.
Small system (o=4, v=8), no rounding (precs < 0: the map is smooth)."""
import numpy as np
import pytest

from golden_util import load

pytestmark = pytest.mark.gpu

H = 1e-5


def _J(eng, method, st, pulse, t0, dt, n, w):
    _, traj = eng.propagate(method, st, t0, dt, n, pulse.field(), precs=-1)
    return float(np.sum(w * traj.detach().cpu().numpy().real))


@pytest.mark.parametrize("method,checkpoint", [("CCSD", 5), ("CC2", 5), ("CCSD", 1000)])
def test_pulse_gradient_matches_finite_differences(method, checkpoint):
    """checkpoint 5: segments recomputed from checkpoints; 1000 >= the step
    count: every step kept by the forward pass."""
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights, pulse_gradient
    d, sysm = load("golden_o4_v8.npz")
    sfx = "" if method == "CCSD" else "_cc2"
    st = tuple(d["gs_" + k + sfx] + 0j for k in ("t1", "t2", "l1", "l2"))
    rng = np.random.default_rng(4)
    n, dt, t0 = 24, 0.01, 0.0
    pulse = Pulse(A=0.03, w0=0.923, c=rng.uniform(0.5, 1.5, 4), t_first=0.0, spacing=n * dt / 3, sigma=n * dt / 3)
    w = cosine_weights(t0, dt, n)
    eng = CCEngine.from_system(sysm)
    try:
        J, gA, gw, gc = pulse_gradient(eng, method, st, pulse, t0, dt, n, w, checkpoint=checkpoint)
        assert abs(J - _J(eng, method, st, pulse, t0, dt, n, w)) < 1e-13
        fd = []
        for name in ["A", "w0"] + [f"c{k}" for k in range(len(pulse.c))]:
            pp, pm = (Pulse(pulse.A, pulse.w0, pulse.c.copy(), pulse.t_first, pulse.spacing, pulse.sigma)
                      for _ in range(2))
            if name == "A":
                pp.A += H
                pm.A -= H
            elif name == "w0":
                pp.w0 += H
                pm.w0 -= H
            else:
                k = int(name[1:])
                pp.c[k] += H
                pm.c[k] -= H
            fd.append((_J(eng, method, st, pp, t0, dt, n, w) - _J(eng, method, st, pm, t0, dt, n, w)) / (2 * H))
        ours = np.array([gA, gw] + list(gc))
        fd = np.array(fd)
        assert np.abs(ours - fd).max() <= 1e-6 * np.abs(fd).max(), (ours, fd)
    finally:
        eng.close()


def test_state_gradient_matches_directional_difference():
    from python_code_to_check_c_gb300.engine import CCEngine, adjoint
    from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights
    d, sysm = load("golden_o4_v8.npz")
    st = [d["gs_" + k] + 0j for k in ("t1", "t2", "l1", "l2")]
    rng = np.random.default_rng(9)
    dx = [1e-2 * (rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape)) for x in st]
    n, dt = 16, 0.01
    pulse = Pulse(A=0.02, w0=0.923, c=np.array([1.0]), t_first=0.08, spacing=1.0, sigma=0.1)
    w = cosine_weights(0.0, dt, n)
    eng = CCEngine.from_system(sysm)
    try:
        J, gE, a = adjoint(eng, "CCSD", st, 0.0, dt, n, w, field=pulse.field(), checkpoint=4, want_state_grad=True)
        # conjugated adjoint: dJ = Re(sum a * dx)
        lhs = sum(float(np.real(np.sum(x.detach().cpu().numpy() * v))) for x, v in zip(a, dx))
        h = 1e-4
        jp = _J(eng, "CCSD", [x + h * v for x, v in zip(st, dx)], pulse, 0.0, dt, n, w)
        jm = _J(eng, "CCSD", [x - h * v for x, v in zip(st, dx)], pulse, 0.0, dt, n, w)
        assert abs(lhs - (jp - jm) / (2 * h)) <= 1e-6 * abs(lhs) + 1e-12
    finally:
        eng.close()


@pytest.mark.parametrize("method,checkpoint", [("CCSD", 5), ("CC2", 1000), ("CCSD", 1000)])
def test_activation_records_match_recomputation(method, checkpoint):
    """Reverse mode bound to the forward step's stored intermediates gives the
    gradients of reverse mode that runs each stage's forward ops again."""
    from python_code_to_check_c_gb300.engine import CCEngine, adjoint
    from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights
    d, sysm = load("golden_o4_v8.npz")
    sfx = "" if method == "CCSD" else "_cc2"
    st = [d["gs_" + k + sfx] + 0j for k in ("t1", "t2", "l1", "l2")]
    n, dt = 14, 0.01
    pulse = Pulse(A=0.02, w0=0.923, c=np.array([1.0, 0.7]), t_first=0.02, spacing=0.06, sigma=0.05)
    w = cosine_weights(0.0, dt, n)
    eng = CCEngine.from_system(sysm)
    try:
        out = []
        for mode in (1, 0):
            eng.set_adjoint_store(mode)
            J, gE, a = adjoint(eng, method, st, 0.0, dt, n, w, field=pulse.field(), checkpoint=checkpoint,
                               want_state_grad=True)
            out.append((J, np.asarray(gE), [x.detach().cpu().numpy() for x in a]))
        (J1, g1, a1), (J0, g0, a0) = out
        assert np.abs(J1 - J0).max() <= 1e-14 * max(1.0, np.abs(J0).max())
        assert np.abs(g1 - g0).max() <= 1e-12 * np.abs(g0).max()
        for x, y in zip(a1, a0):
            assert np.abs(x - y).max() <= 1e-12 * max(np.abs(y).max(), 1e-30)
    finally:
        eng.close()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_state_gradient_matches_torch_autograd_o6_v12(method):
    """dJ/d(initial state) of the device reverse mode against torch autograd
    through the oracle's reference-style einsum right-hand sides and the
    block-frozen RK4 loop (no rounding), o=6, v=12, 6 steps."""
    torch = pytest.importorskip("torch")
    import math

    from oracle.cc_oracle import CCOracle
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine, adjoint
    from python_code_to_check_c_gb300.system import mp2_guess, synthetic_system
    sysm = synthetic_system(6, 12, 72, seed=612)
    tei = sysm.tei()
    o = sysm.o
    rng = np.random.default_rng(13)
    t2 = mp2_guess(tei, sysm.eps(), o) + 1e-3 * rng.standard_normal((o, o, sysm.v, sysm.v))
    t1 = 1e-2 * (rng.standard_normal((o, sysm.v)) + 1j * rng.standard_normal((o, sysm.v)))
    st = [t1, t2 + 0j, 0.5 * t1, 0.7 * t2 + 0j]
    n, dt, A, w0 = 6, 0.01, 0.02, 0.923
    w = np.cos(0.8 * dt * np.arange(1, n + 1)) * dt
    eng = CCEngine.from_system(sysm)
    try:
        J, _, a = adjoint(eng, method, st, 0.0, dt, n, w, field=make_field("sin", A, w0), checkpoint=4,
                          want_state_grad=True)
        a = [x.detach().cpu().numpy() for x in a]
    finally:
        eng.close()

    mu_z = torch.as_tensor(sysm.mu[2]).to(torch.complex128)
    orc = CCOracle(torch.as_tensor(tei).to(torch.complex128), o)
    F = torch.as_tensor(sysm.fock).to(torch.complex128)
    x = [torch.as_tensor(s).clone().requires_grad_(True) for s in st]
    Vt = lambda t: -(A * math.sin(w0 * t)) * mu_z  # noqa: E731

    def dipole(t1, t2, l1, l2):
        rho = torch.cat([torch.cat([orc.Dij(t1, t2, l1, l2), l1], 1),
                         torch.cat([orc.Dai(t1, t2, l1, l2), orc.Dab(t1, t2, l1, l2)], 1)], 0)
        return torch.sum(mu_z * rho)

    t1, t2, l1, l2 = x
    t = 0.0
    Jt = 0.0
    for k in range(n):
        t += dt
        d1 = -1j * orc.ft1(t, dt, t1, t2, F, Vt)
        if method == "CCSD":
            d2 = -1j * orc.ft2(t, dt, t1, t2, F, Vt)
            e1 = 1j * orc.fL1(t, dt, t1, t2, l1, l2, F, Vt)
            e2 = 1j * orc.fL2(t, dt, t1, t2, l1, l2, F, Vt)
        else:
            d2 = -1j * orc.ft2_CC2(t, dt, t1, t2, F, Vt)
            e1 = 1j * orc.fL1_CC2(t, dt, t1, t2, l1, l2, F, Vt)
            e2 = 1j * orc.fL2_CC2(t, dt, t1, t2, l1, l2, F, Vt)
        t1, t2, l1, l2 = t1 + d1, t2 + d2, l1 + e1, l2 + e2
        Jt = Jt + w[k] * dipole(t1, t2, l1, l2).real
    assert abs(float(Jt.detach()) - float(J[0])) <= 1e-12 * max(1.0, abs(float(J[0])))
    grads = torch.autograd.grad(Jt, x)
    for ours, g in zip(a, grads):
        ref = np.conj(g.numpy())  # torch's gradient of a real J is dJ/dRe z + i dJ/dIm z
        assert np.abs(ours - ref).max() <= 1e-10 * np.abs(ref).max(), np.abs(ours - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_pulse_gradient_100_steps_o6_v12(method):
    """o=6, v=12 (Q=72, seed 612), 100 steps of dt = 0.01 from the MP2-guess
    state, a pulse of 8 Gaussian envelope bumps, checkpoints every 10 steps:
    dJ/dA, dJ/dw0 and all eight dJ/dc_k against central differences
    (h = 1e-5), relative 1e-6 of the largest."""
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights, pulse_gradient
    from python_code_to_check_c_gb300.system import WORKLOADS, mp2_guess, synthetic_system
    sysm = synthetic_system(**WORKLOADS["o6_v12"])
    t2 = mp2_guess(sysm.tei(), sysm.eps(), sysm.o).astype(np.complex128)
    t1 = np.zeros((sysm.o, sysm.v), dtype=np.complex128)
    st = (t1, t2, t1.copy(), t2.copy())
    rng = np.random.default_rng(12)
    n, dt, t0 = 100, 0.01, 0.0
    spacing = n * dt / 7
    pulse = Pulse(A=0.03, w0=0.923, c=rng.uniform(0.5, 1.5, 8), t_first=0.0, spacing=spacing, sigma=spacing)
    w = cosine_weights(t0, dt, n)
    eng = CCEngine.from_system(sysm)
    try:
        J, gA, gw, gc = pulse_gradient(eng, method, st, pulse, t0, dt, n, w, checkpoint=10)
        assert abs(J - _J(eng, method, st, pulse, t0, dt, n, w)) < 1e-13
        fd = []
        for name in ["A", "w0"] + [f"c{k}" for k in range(len(pulse.c))]:
            pp, pm = (Pulse(pulse.A, pulse.w0, pulse.c.copy(), pulse.t_first, pulse.spacing, pulse.sigma)
                      for _ in range(2))
            if name == "A":
                pp.A += H
                pm.A -= H
            elif name == "w0":
                pp.w0 += H
                pm.w0 -= H
            else:
                k = int(name[1:])
                pp.c[k] += H
                pm.c[k] -= H
            fd.append((_J(eng, method, st, pp, t0, dt, n, w) - _J(eng, method, st, pm, t0, dt, n, w)) / (2 * H))
        ours = np.array([gA, gw] + list(gc))
        fd = np.array(fd)
        print(method, "max |adjoint - FD| / max |FD|:", np.abs(ours - fd).max() / np.abs(fd).max())
        assert np.abs(ours - fd).max() <= 1e-6 * np.abs(fd).max(), (ours, fd)
    finally:
        eng.close()
