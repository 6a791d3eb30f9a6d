"""CPU check of the reverse-mode (vector-Jacobian product) programs the engine
generates from its equation programs.  The op lists (tdcc_program_json /
tdcc_adjoint_program_json, no GPU) are interpreted with numpy and compared
with (a) central finite differences of the forward programs and (b) torch
autograd through the oracle's reference-style einsum right-hand sides.

Adjoints are carried conjugated: for cotangent w of the output, the program
returns a_x = J^T w, so sum(w * df) = sum(a_x * dx) for every direction dx
(bilinear, no conjugation), and torch's grad with grad_outputs = conj(w) is
conj(a_x)."""
import numpy as np
import pytest

from golden_util import load, rel_err
from program_emulator import S_F, S_L1, S_L2, S_MU, S_OUT, S_RES, S_T1, S_T2, S_TEI, Emulator

INPUTS = (S_F, S_T1, S_T2, S_L1, S_L2)
NAMES = {S_F: "F", S_T1: "t1", S_T2: "t2", S_L1: "l1", S_L2: "l2"}


def _inputs(sysm, nb, seed):
    rng = np.random.default_rng(seed)
    o, v, n = sysm.o, sysm.v, sysm.n
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    x = {}
    x[S_F] = np.stack([sysm.fock + 0.05 * c(n, n) for _ in range(nb)])
    x[S_T1] = 0.05 * c(nb, o, v)
    x[S_T2] = 0.05 * c(nb, o, o, v, v)
    x[S_L1] = 0.05 * c(nb, o, v)
    x[S_L2] = 0.05 * c(nb, o, o, v, v)
    return x


def _forward(sysm, tei, method, block, x, nb):
    from python_code_to_check_c_gb300._lib import program_json
    o, v = sysm.o, sysm.v
    prog = program_json(o, v, method, block, 3, nb)
    e = Emulator(prog, o, v, share=False)
    e.bind(S_TEI, tei)
    e.bind(S_MU, np.stack(sysm.mu))
    for s in INPUTS:
        e.bind(s, x[s])
    e.bind(S_OUT, np.zeros(nb * o * o * v * v, dtype=np.complex128))
    e.bind(S_RES, np.zeros(nb * 3, dtype=np.complex128))
    e.run("all")
    return e, prog


def _out(e, block, sysm, nb):
    o, v = sysm.o, sysm.v
    if block == 4:
        return e.bufs[S_RES][: nb * 3].copy()
    n1 = o * v if block in (0, 2) else o * o * v * v
    return e.bufs[S_OUT][: nb * n1].copy()


def _adjoint(sysm, tei, method, block, x, w, nb, ef=None):
    """Returns {input slot: a_x} for cotangent w of the output."""
    from python_code_to_check_c_gb300._lib import adjoint_program_json
    o, v = sysm.o, sysm.v
    if ef is None:
        ef, _ = _forward(sysm, tei, method, block, x, nb)
    adj = adjoint_program_json(o, v, method, block, 3, nb)
    ea = Emulator(adj, o, v, zero=True)
    for s, b in ef.bufs.items():
        if s < adj["nfwd"]:
            ea.bufs[s] = b
    aof = adj["adj_of"]
    for s, a in enumerate(aof):
        if a >= 0 and adj["slots"][a]["fixed"]:
            ea.bufs[a] = np.zeros(adj["slots"][a]["numel"], dtype=np.complex128)
    tgt = aof[S_RES] if block == 4 else aof[S_OUT]
    ea.bufs[tgt][: w.size] = w
    ea.run("all")
    return {s: ea.bufs[aof[s]].copy() for s in INPUTS if aof[s] >= 0}, adj


@pytest.fixture(scope="module")
def small():
    d, sysm = load("golden_o3_v5.npz")
    return sysm, sysm.tei()


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
@pytest.mark.parametrize("block", [0, 1, 2, 3, 4])
def test_adjoint_matches_finite_differences(small, method, block):
    sysm, tei = small
    nb = 1
    x = _inputs(sysm, nb, 1)
    dx = _inputs(sysm, nb, 2)
    ef, _ = _forward(sysm, tei, method, block, x, nb)
    y = _out(ef, block, sysm, nb)
    rng = np.random.default_rng(3)
    w = rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)
    a, _ = _adjoint(sysm, tei, method, block, x, w, nb, ef)
    lhs = sum(np.sum(a[s] * dx[s].reshape(-1)) for s in a)
    h = 1e-4
    xp = {s: x[s] + h * dx[s] for s in INPUTS}
    xm = {s: x[s] - h * dx[s] for s in INPUTS}
    yp = _out(_forward(sysm, tei, method, block, xp, nb)[0], block, sysm, nb)
    ym = _out(_forward(sysm, tei, method, block, xm, nb)[0], block, sysm, nb)
    rhs = np.sum(w * (yp - ym)) / (2 * h)
    assert abs(lhs - rhs) <= 1e-7 * max(abs(rhs), 1e-12), (lhs, rhs)


@pytest.mark.parametrize("method,block", [("CCSD", 0), ("CCSD", 1), ("CCSD", 2), ("CCSD", 3),
                                          ("CC2", 1), ("CC2", 2), ("CC2", 3)])
def test_adjoint_matches_torch_autograd_o6_v12(method, block):
    """Against torch autograd through the oracle's einsum right-hand sides
    (reference-style contractions), o=6, v=12."""
    torch = pytest.importorskip("torch")
    from oracle.cc_oracle import CCOracle
    from python_code_to_check_c_gb300.system import synthetic_system
    sysm = synthetic_system(6, 12, 72, seed=612)
    tei = sysm.tei()
    x = _inputs(sysm, 1, 7)
    ef, _ = _forward(sysm, tei, method, block, x, 1)
    y = _out(ef, block, sysm, 1)
    rng = np.random.default_rng(8)
    w = rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)
    a, _ = _adjoint(sysm, tei, method, block, x, w, 1, ef)
    orc = CCOracle(torch.as_tensor(tei).to(torch.complex128), sysm.o)  # torch.einsum wants one dtype
    tx = {s: torch.as_tensor(x[s][0]).clone().requires_grad_(True) for s in INPUTS}
    F, t1, t2, l1, l2 = (tx[s] for s in (S_F, S_T1, S_T2, S_L1, S_L2))
    fn = {("CCSD", 0): lambda: orc.T1eq_rhs(t1, t2, F), ("CCSD", 1): lambda: orc.T2eq_rhs(t1, t2, F),
          ("CCSD", 2): lambda: orc.lam_1eq_rhs(t1, t2, l1, l2, F),
          ("CCSD", 3): lambda: orc.lam2eq_rhs(t1, t2, l1, l2, F),
          ("CC2", 1): lambda: orc.T2eq_rhs_CC2(t1, t2, F),
          ("CC2", 2): lambda: orc.L1eq_rhs_CC2(t1, t2, l1, l2, F),
          ("CC2", 3): lambda: orc.L2eq_rhs_CC2(t1, t2, l1, l2, F)}[(method, block)]
    out = fn()
    assert rel_err(out.detach().numpy().reshape(-1), y) < 1e-12
    grads = torch.autograd.grad(out, [tx[s] for s in INPUTS], grad_outputs=torch.as_tensor(np.conj(w).reshape(out.shape)),
                                allow_unused=True)
    for s, gr in zip(INPUTS, grads):
        ours = a.get(s, np.zeros(x[s].size, dtype=np.complex128))
        ref = np.zeros(x[s].size, dtype=np.complex128) if gr is None else np.conj(gr.numpy().reshape(-1))
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(ours - ref).max() <= 1e-12 * scale + 1e-14, (NAMES[s], np.abs(ours - ref).max(), scale)


def test_batched_adjoint_equals_single(small):
    sysm, tei = small
    nb = 3
    x = _inputs(sysm, nb, 4)
    ef, _ = _forward(sysm, tei, "CCSD", 3, x, nb)
    y = _out(ef, 3, sysm, nb)
    rng = np.random.default_rng(5)
    w = rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)
    a, _ = _adjoint(sysm, tei, "CCSD", 3, x, w, nb, ef)
    n1 = y.size // nb
    for z in range(nb):
        xz = {s: x[s][z:z + 1] for s in INPUTS}
        az, _ = _adjoint(sysm, tei, "CCSD", 3, xz, w[z * n1:(z + 1) * n1], 1)
        for s in az:
            k = az[s].size
            assert rel_err(a[s][z * k:(z + 1) * k], az[s]) < 1e-13, (NAMES[s], z)


@pytest.mark.parametrize("method,block", [("CCSD", 1), ("CCSD", 2), ("CC2", 3)])
def test_adjoint_phase_split(small, method, block):
    """What the propagator does: the forward prologue once, then per stage the
    forward stage and the stage adjoint (cotangent w_s, stage inputs Y_s,
    F_s), then the prologue adjoint once -- equals the sum of whole-program
    adjoints, for the adjoints of the frozen inputs."""
    from python_code_to_check_c_gb300._lib import adjoint_program_json, program_json
    sysm, tei = small
    o, v = sysm.o, sysm.v
    x = _inputs(sysm, 1, 11)
    vs = S_T1 + block
    stages = []
    rng = np.random.default_rng(12)
    for k in range(2):
        ys = _inputs(sysm, 1, 20 + k)
        xs = dict(x)
        xs[vs] = ys[vs]
        xs[S_F] = ys[S_F]
        stages.append(xs)
    n1 = o * v if block in (0, 2) else o * o * v * v
    ws = [rng.standard_normal(n1) + 1j * rng.standard_normal(n1) for _ in stages]
    ref = {}
    for xs, w in zip(stages, ws):
        a, _ = _adjoint(sysm, tei, method, block, xs, w, 1)
        for s in a:
            ref[s] = ref.get(s, 0) + a[s]
    # phased run
    fwd = program_json(o, v, method, block, 3, 1)
    adj = adjoint_program_json(o, v, method, block, 3, 1)
    ef = Emulator(fwd, o, v, share=False)
    ef.bind(S_TEI, tei)
    ef.bind(S_MU, np.stack(sysm.mu))
    for s in INPUTS:
        ef.bind(s, x[s])
    ef.bind(S_OUT, np.zeros(o * o * v * v, dtype=np.complex128))
    ef.bind(S_RES, np.zeros(3, dtype=np.complex128))
    ef.run("setup")
    ef.run("prologue")
    ea = Emulator(adj, o, v, zero=True)
    aof = adj["adj_of"]
    for s, a in enumerate(aof):
        if a >= 0 and adj["slots"][a]["fixed"]:
            ea.bufs[a] = np.zeros(adj["slots"][a]["numel"], dtype=np.complex128)
    got = {s: np.zeros(x[s].size, dtype=np.complex128) for s in INPUTS}
    for xs, w in zip(stages, ws):
        ef.bind(vs, xs[vs])
        ef.bind(S_F, xs[S_F])
        ef.run("stage")
        for s, b in ef.bufs.items():
            if s < adj["nfwd"]:
                ea.bufs[s] = b
        ea.bufs[aof[S_OUT]][:n1] = w
        ea.run("stage")
        for s in (vs, S_F):  # per-stage inputs: read out and clear
            got[s] += ea.bufs[aof[s]][: x[s].size]
            ea.bufs[aof[s]][:] = 0
    ea.run("prologue")
    for s in INPUTS:
        if s in (vs, S_F) or aof[s] < 0:
            continue
        got[s] += ea.bufs[aof[s]][: x[s].size]
    for s in INPUTS:
        if s in ref:
            assert rel_err(got[s], ref[s]) < 1e-12, NAMES[s]
