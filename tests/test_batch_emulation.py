"""CPU check of the trajectory-batched programs: the op lists libtdcc launches
for nb trajectories (read through tdcc_program_json, no GPU) are interpreted
with numpy; every trajectory's result must equal the single-trajectory
program's on that trajectory's inputs, and trajectory 0 the reference's
golden output."""
import numpy as np
import pytest

from golden_util import load, rel_err
from program_emulator import S_F, S_L1, S_L2, S_MU, S_OUT, S_RES, S_T1, S_T2, S_TEI, Emulator

GOLD = {("CCSD", 0): "T1", ("CCSD", 1): "T2", ("CCSD", 2): "L1", ("CCSD", 3): "L2",
        ("CC2", 0): "T1", ("CC2", 1): "T2_CC2", ("CC2", 2): "L1_CC2", ("CC2", 3): "L2_CC2"}
NB = 3


@pytest.fixture(scope="module")
def case():
    d, sysm = load("golden_o3_v5.npz")
    rng = np.random.default_rng(5)
    trajs = [{k: d[k].astype(np.complex128) for k in ("F", "t1", "t2", "l1", "l2")}]
    for _ in range(NB - 1):
        t = {}
        for k in ("F", "t1", "t2", "l1", "l2"):
            x = d[k].astype(np.complex128)
            t[k] = x * (1 + 0.1 * rng.standard_normal(x.shape)) + 0.01j * rng.standard_normal(x.shape)
        trajs.append(t)
    return d, sysm, sysm.tei(), trajs


def _run(sysm, tei, method, block, trajs, nb, phases=("all",)):
    from python_code_to_check_c_gb300._lib import program_json
    o, v = sysm.o, sysm.v
    prog = program_json(o, v, method, block, 3, nb)
    e = Emulator(prog, o, v)
    e.bind(S_TEI, tei)
    e.bind(S_MU, np.stack(sysm.mu))
    for slot, k in ((S_F, "F"), (S_T1, "t1"), (S_T2, "t2"), (S_L1, "l1"), (S_L2, "l2")):
        e.bind(slot, np.concatenate([t[k].reshape(-1) for t in trajs[:nb]]))
    e.bind(S_OUT, np.zeros(nb * o * o * v * v, dtype=np.complex128))
    e.bind(S_RES, np.zeros(nb * 3, dtype=np.complex128))
    for ph in phases:
        e.run(ph)
    return e, prog


@pytest.mark.parametrize("method,block", sorted(GOLD))
def test_batched_program_equals_single(case, method, block):
    d, sysm, tei, trajs = case
    o, v = sysm.o, sysm.v
    eb, prog = _run(sysm, tei, method, block, trajs, NB)
    n1 = o * v if block in (0, 2) else o * o * v * v
    outb = eb.bufs[S_OUT]
    for z in range(NB):
        es, _ = _run(sysm, tei, method, block, [trajs[z]], 1)
        ref = es.bufs[S_OUT][:n1]
        got = outb[z * n1:(z + 1) * n1]
        assert rel_err(got, ref) < 1e-13, z
    gold = d[GOLD[(method, block)]]
    assert rel_err(outb[:n1].reshape(gold.shape), gold) < 1e-12


def test_batched_program_uses_folded_and_batched_products(case):
    """Contractions with the integrals fold the trajectories into one GEMM
    (a mode of extent nb in the M or N group); products of two per-trajectory
    operands run as batched GEMMs."""
    d, sysm, tei, trajs = case
    from python_code_to_check_c_gb300._lib import program_json
    prog = program_json(sysm.o, sysm.v, "CCSD", 1, 3, NB)
    folded = batched = 0
    for op in prog["ops"]:
        if op["kind"] != "gemm":
            continue
        if op["nb"] > 1:
            batched += 1
        elif NB in op["gm"]["dim"][:1] or NB in op["gn"]["dim"][:1]:
            folded += 1
    assert folded > 0 and batched > 0
    slots = prog["slots"]
    assert not slots[S_TEI]["batched"] and slots[S_T2]["batched"]
    assert all(s["numel"] == s["numel1"] * (NB if s["batched"] else 1) for s in slots if not s["fixed"])


@pytest.mark.parametrize("method,block", [("CCSD", 1), ("CCSD", 3), ("CC2", 2)])
def test_batched_prologue_split(case, method, block):
    """setup + prologue with the varying inputs poisoned, then the stages,
    give the same result as the whole program (batched)."""
    d, sysm, tei, trajs = case
    o, v = sysm.o, sysm.v
    ref, _ = _run(sysm, tei, method, block, trajs, NB)
    from python_code_to_check_c_gb300._lib import program_json
    prog = program_json(o, v, method, block, 3, NB)
    e = Emulator(prog, o, v)
    e.bind(S_TEI, tei)
    e.bind(S_MU, np.stack(sysm.mu))
    for slot, k in ((S_F, "F"), (S_T1, "t1"), (S_T2, "t2"), (S_L1, "l1"), (S_L2, "l2")):
        e.bind(slot, np.concatenate([t[k].reshape(-1) for t in trajs]))
    e.bind(S_OUT, np.zeros(NB * o * o * v * v, dtype=np.complex128))
    e.bind(S_RES, np.zeros(NB * 3, dtype=np.complex128))
    vs = S_T1 + block
    good_v, good_f = e.bufs[vs].copy(), e.bufs[S_F].copy()
    e.bufs[vs] = np.full_like(good_v, np.nan)
    e.bufs[S_F] = np.full_like(good_f, np.nan)
    e.run("setup")
    e.run("prologue")
    e.bufs[vs], e.bufs[S_F] = good_v, good_f
    e.run("stage")
    assert np.isfinite(e.bufs[S_OUT]).all()
    assert rel_err(e.bufs[S_OUT], ref.bufs[S_OUT]) < 1e-13


def test_batched_density(case):
    d, sysm, tei, trajs = case
    eb, _ = _run(sysm, tei, "CCSD", 4, trajs, NB)
    for z in range(NB):
        es, _ = _run(sysm, tei, "CCSD", 4, [trajs[z]], 1)
        assert np.abs(eb.bufs[S_RES][3 * z:3 * z + 3] - es.bufs[S_RES][:3]).max() < 1e-14
    assert abs(eb.bufs[S_RES][2] - d["mu"][2]) < 1e-14
