"""Trajectory batching on the device: nb trajectories advanced by one batched
system equal nb single-trajectory runs (same fields, polarisations and
starting states).  FP64 to 1e-12 (summation order differs between the
batched and single GEMM shapes); the mixed mode to 1e-10."""
import numpy as np
import pytest

from golden_util import load, rel_err

pytestmark = pytest.mark.gpu

NB = 4


def _np(x):
    return x.detach().cpu().numpy()


def _inputs(d, nb, seed=3):
    rng = np.random.default_rng(seed)
    states = []
    for z in range(nb):
        st = []
        for k in ("gs_t1", "gs_t2", "gs_l1", "gs_l2"):
            x = d[k].astype(np.complex128)
            if z:
                x = x * (1 + 0.05 * rng.standard_normal(x.shape)) + 1e-3j * rng.standard_normal(x.shape)
            st.append(x)
        states.append(st)
    return states


def _fields(nb):
    from python_code_to_check_c_gb300._lib import make_field
    amps = [0.001, 0.002, 0.005, 0.01]
    w0s = [0.5, 0.923]
    fl = [make_field("sin", amps[z % 4], w0s[z % 2]) for z in range(nb)]
    pol = [z % 3 for z in range(nb)]
    return fl, pol


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_propagation_equals_single_runs(method, precision):
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.system import synthetic_system
    d, _ = load("golden_o4_v8.npz")
    sysm = synthetic_system(4, 8, int(d["nq"]), int(d["seed"]))
    # x and y dipoles too, so every polarisation couples
    rng = np.random.default_rng(11)
    mus = []
    for _ in range(2):
        M = rng.standard_normal((sysm.n, sysm.n))
        M = 0.5 * (M + M.T)
        mus.append(M / np.linalg.norm(M))
    sysm.mu = [mus[0], mus[1], sysm.mu[2]]
    states = _inputs(d, NB)
    fields, pol = _fields(NB)
    dt, nsteps = 0.01, 12
    eb = CCEngine.from_system(sysm, nb=NB)
    if precision == "mixed":
        eb.set_precision("mixed", 5)
        eb.set_tc_policy(0, 1, 1)
    eb.set_fields(fields, pol)
    batch_state = [np.stack([s[k] for s in states]) for k in range(4)]
    fin_b, traj_b = eb.propagate(method, batch_state, 0.0, dt, nsteps, None, precs=15)
    eb.check_errors()
    traj_b = _np(traj_b)
    assert traj_b.shape == (nsteps, NB)
    for z in range(NB):
        es = CCEngine.from_system(sysm)
        if precision == "mixed":
            es.set_precision("mixed", 5)
            es.set_tc_policy(0, 1, 1)
        es.set_fields([fields[z]], [pol[z]])
        fin_s, traj_s = es.propagate(method, states[z], 0.0, dt, nsteps, None, precs=15)
        tol = 1e-12 if precision == "fp64" else 1e-10
        assert np.abs(traj_b[:, z] - _np(traj_s)).max() < tol, z
        for a, b in zip(fin_b, fin_s):
            assert rel_err(_np(a)[z], _np(b)) < 1e2 * tol, z
        es.close()
    eb.close()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
def test_batched_rhs_and_dipole(method):
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load("golden_o4_v8.npz")
    states = _inputs(d, NB)
    rng = np.random.default_rng(2)
    Fs = [d["F"] + 0.01 * rng.standard_normal(d["F"].shape) * (z > 0) for z in range(NB)]
    eb = CCEngine.from_system(sysm, nb=NB)
    es = CCEngine.from_system(sysm)
    bst = [np.stack([s[k] for s in states]) for k in range(4)]
    F = np.stack(Fs).astype(np.complex128)
    for block in range(4):
        out = _np(eb.rhs(method, block, bst[0], bst[1], bst[2], bst[3], F))
        for z in range(NB):
            ref = _np(es.rhs(method, block, *states[z], Fs[z]))
            assert rel_err(out[z], ref) < 1e-12, (block, z)
    mu = _np(eb.dipole_moment(*bst))
    for z in range(NB):
        assert np.abs(mu[z] - _np(es.dipole_moment(*states[z]))).max() < 1e-13
    eb.close()
    es.close()
