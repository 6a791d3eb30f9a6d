"""Host logic of ``CC_Calculator.Runge_Kutta_solver`` (chunking, stop tests,
save / restart) with a CPU stand-in for the device engine.  The stand-in
follows the engine's call contract; its arithmetic is either the oracle's
loop body or a counter that makes the stop step predictable."""
import numpy as np
import torch

from golden_util import load
from python_code_to_check_c_gb300 import restart_io
from python_code_to_check_c_gb300.calculator import USAGE, CC_Calculator


class OracleEngine:
    """propagate / rk4_step / dipole_moment over the oracle (reference field)."""

    def __init__(self, sysm, A, w0):
        from oracle.cc_oracle import CCOracle, reference_field
        self.orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
        self.F = sysm.fock
        self.Vt = reference_field(A, w0, sysm.mu[2])
        self.calls = []

    def dipole_moment(self, *st):
        return torch.as_tensor(np.asarray(self.orc.dipole_moment(*[np.asarray(x) for x in st])))

    def rk4_step(self, method, state, t_prev, dt, field, precs=15):
        self.calls.append(("step", t_prev))
        st = [np.asarray(x) for x in state]
        new = self.orc.rk4_step(method, t_prev + dt, dt, st, self.F, self.Vt, precs)
        return tuple(torch.as_tensor(x) for x in new), self.dipole_moment(*new)

    def block_times(self, method, state, t_prev, dt, field, precs=15):
        return [1.0, 4.0, 2.0, 3.0]

    def propagate(self, method, state, t0, dt, n, field, precs=15):
        self.calls.append(("prop", t0, n))
        _, mus, st = self.orc.propagate(method, self.F, [np.asarray(x) for x in state], t0, dt, n, self.Vt, precs)
        return tuple(torch.as_tensor(x) for x in st), torch.as_tensor(mus[1:])


class CounterEngine:
    """Each step maps the state x to round(x) + 1; mu_z = 30 * t1[0, 0]."""

    def _mu(self, st):
        return torch.tensor([0j, 0j, 30.0 * complex(st[0][0, 0])])

    def dipole_moment(self, *st):
        return self._mu(st)

    def block_times(self, method, state, t_prev, dt, field, precs=15):
        return [1.0, 4.0, 2.0, 3.0]

    def rk4_step(self, method, state, t_prev, dt, field, precs=15):
        new = tuple(torch.round(x.real) + 1 + 0j for x in state)
        return new, self._mu(new)

    def propagate(self, method, state, t0, dt, n, field, precs=15):
        mus = []
        for _ in range(n):
            state, mu = self.rk4_step(method, state, t0, dt, field, precs)
            mus.append(mu[-1])
        return state, torch.stack(mus) if mus else torch.zeros(0, dtype=torch.complex128)


def _calc(sysm, tmp_path, eng, **kw):
    c = CC_Calculator(system=sysm, outdir=str(tmp_path), verbose=False, w0=0.923, A=0.002, t0=0.0,
                      dt=0.01, precs=15, **kw)
    c.engine = lambda F=None: eng
    return c


def test_usage_message(capsys):
    _, sysm = load("golden_o3_v5.npz")
    c = CC_Calculator(system=sysm, verbose=False)
    assert c.TDCC(1.0, "CCSDT") is None
    assert capsys.readouterr().out.strip() == USAGE


def test_missing_keywords_are_ignored():
    _, sysm = load("golden_o3_v5.npz")
    c = CC_Calculator(system=sysm, verbose=False, w0=1.0)
    assert c.w0 == 1.0 and not hasattr(c, "dt") and c.tf == 10.1


def test_mp2_energy_matches_oracle():
    from oracle.cc_oracle import CCOracle
    _, sysm = load("golden_o4_v8.npz")
    orc = CCOracle(sysm.tei(), sysm.o, mu=sysm.mu)
    t2 = orc.MP2_guess(sysm.fock)
    e2 = 0.25 * np.sum(sysm.tei()[: sysm.o, : sysm.o, sysm.o:, sysm.o:] * t2)
    c = CC_Calculator(system=sysm, verbose=False)
    assert abs(c.test_MP2() - e2) < 1e-14


def test_chunked_loop_equals_plain_loop(tmp_path):
    d, sysm = load("golden_o3_v5.npz")
    eng = OracleEngine(sysm, 0.002, 0.923)
    st = tuple(d[k] + 0j for k in ("t1", "t2", "l1", "l2"))
    c = _calc(sysm, tmp_path, eng, chunk=3)
    out = c.Runge_Kutta_solver(sysm.fock, *st, 0.923, 0.002, 0.0, 0.07, 0.01, None, 15)
    times, mus, _ = eng.orc.propagate("CCSD", sysm.fock, list(st), 0.0, 0.01, 7, eng.Vt, 15)
    assert out["steps"] == 7 and not out["stopped"]
    assert np.array_equal(out["times"], np.round(times[1:], 4))
    assert np.array_equal(out["mu"], mus[1:])
    assert list(tmp_path.iterdir()) == []          # reaching tf saves nothing


def test_divergence_stop_saves_previous_state(tmp_path):
    _, sysm = load("golden_o3_v5.npz")
    o, v = sysm.o, sysm.v
    st = (np.zeros((o, v)), np.zeros((o, o, v, v)), np.zeros((o, v)), np.zeros((o, o, v, v)))
    c = _calc(sysm, tmp_path, CounterEngine(), chunk=6)
    out = c.Runge_Kutta_solver(sysm.fock, *st, 0.923, 0.002, 0.0, 10.0, 0.01, None, 15)
    # mu_z after step k is 30 k: step 4 is the first above 100
    assert out["stopped"] and out["steps"] == 4
    assert np.allclose(out["mu"].real, [30, 60, 90, 120])
    rows = (tmp_path / "H2O.csv").read_text().splitlines()
    assert rows[0] == ",time,mu_real,mu_imag" and len(rows) == 5
    p = restart_io.read_parameters(tmp_path / "Parameters.csv")
    assert p["t0"] == 0.01 + 0.01 + 0.01 + 0.01 - 0.01 and (p["i"], p["a"]) == (o, v)
    _, t1, t2, l1, l2 = restart_io.load_restart(str(tmp_path), o, v)
    assert np.all(t1 == 3) and np.all(l2 == 3)     # the state before the stopping step
    # timing.csv: the block columns split each step's time 1 : 4 : 2 : 3 and sum to total
    rows = (tmp_path / "timing.csv").read_text().splitlines()
    assert rows[0] == ",total,t1,t2,l1,l2" and len(rows) == 5
    for r in rows[1:]:
        tot, *blk = (float(x) for x in r.split(",")[1:])
        assert abs(sum(blk) - tot) <= 1e-12 * max(tot, 1e-300)
        assert np.allclose(np.array(blk) / tot, [0.1, 0.4, 0.2, 0.3])


def test_timeout_stop_and_restart(tmp_path):
    d, sysm = load("golden_o3_v5.npz")
    eng = OracleEngine(sysm, 0.002, 0.923)
    st = tuple(d[k] + 0j for k in ("t1", "t2", "l1", "l2"))
    c = _calc(sysm, tmp_path, eng, chunk=4)
    out = c.Runge_Kutta_solver(sysm.fock, *st, 0.923, 0.002, 0.0, 10.0, 0.01, 0.0, 15, method="CC2")
    assert out["stopped"] and out["steps"] == 4     # the limit is checked after each chunk
    assert eng.calls == [("prop", 0.0, 3), ("step", 0.01 + 0.01 + 0.01)]
    p = restart_io.read_parameters(tmp_path / "Parameters.csv")
    assert p["CCSD_or_CC2"] == "CC2"
    t_saved = p["t0"]
    F, *saved = restart_io.load_restart(str(tmp_path), sysm.o, sysm.v)
    # restart: starts at t_saved + dt from the saved (rounded) state, appends rows
    eng2 = OracleEngine(sysm, 0.002, 0.923)
    c2 = _calc(sysm, tmp_path, eng2, chunk=4)
    out2 = c2.TDCC_restart(0.0)
    assert out2["steps"] == 4
    times, mus, _ = eng2.orc.propagate("CC2", sysm.fock, saved, t_saved + 0.01, 0.01, 4, eng2.Vt, 15)
    assert np.array_equal(out2["times"], np.round(times[1:], 4))
    assert np.abs(out2["mu"] - mus[1:]).max() < 1e-14
    rows = (tmp_path / "H2O.csv").read_text().splitlines()
    assert len(rows) == 1 + 4 + 4 and rows[5].startswith("1,")


def test_psi4_construction_path(tmp_path):
    """CC_Calculator(psi4) as the reference's scripts call it: the system comes
    from the psi4 integral adapter (here the psi4 stand-in), and the loop runs
    on it."""
    import fake_psi4
    from python_code_to_check_c_gb300.system import system_from_psi4
    psi4 = fake_psi4.make()
    c = CC_Calculator(psi4, outdir=str(tmp_path), verbose=False, w0=0.923, A=0.002, t0=0.0, dt=0.01, precs=15)
    ref = system_from_psi4(fake_psi4.make())
    assert (c.system.o, c.system.v, c.ndocc) == (ref.o, ref.v, ref.o // 2)
    np.testing.assert_array_equal(c.system.fock, ref.fock)
    eng = OracleEngine(c.system, 0.002, 0.923)
    c.engine = lambda F=None: eng
    o, v = c.system.o, c.system.v
    rng = np.random.default_rng(2)
    st = (0.01 * rng.standard_normal((o, v)) + 0j, np.zeros((o, o, v, v)) + 0j,
          0.01 * rng.standard_normal((o, v)) + 0j, np.zeros((o, o, v, v)) + 0j)
    out = c.Runge_Kutta_solver(c.system.fock, *st, 0.923, 0.002, 0.0, 0.05, 0.01, None, 15)
    _, mus, _ = eng.orc.propagate("CCSD", c.system.fock, list(st), 0.0, 0.01, 5, eng.Vt, 15)
    assert out["steps"] == 5 and np.array_equal(out["mu"], mus[1:])
