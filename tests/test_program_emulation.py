"""CPU check of the engine's equation programs: the op lists libtdcc would
launch (read through tdcc_program_json, no GPU) are interpreted with numpy and
compared with the reference's golden outputs.  Also checks that every op the
RK4 prologue runs once per step is independent of the block's varying inputs
(the amplitude being advanced and the field-dressed Fock matrix)."""
import numpy as np
import pytest

from golden_util import CASES, load, rel_err
from program_emulator import S_F, S_L1, S_L2, S_MU, S_OUT, S_RES, S_T1, S_T2, S_TEI, Emulator

BLOCKS = {"T1": 0, "T2": 1, "L1": 2, "L2": 3}
GOLD = {("CCSD", 0): "T1", ("CCSD", 1): "T2", ("CCSD", 2): "L1", ("CCSD", 3): "L2",
        ("CC2", 0): "T1", ("CC2", 1): "T2_CC2", ("CC2", 2): "L1_CC2", ("CC2", 3): "L2_CC2"}


@pytest.fixture(scope="module", params=CASES)
def case(request):
    d, sysm = load(request.param)
    return d, sysm, sysm.tei()


def _emu(d, sysm, tei, method, block, F=None):
    from python_code_to_check_c_gb300._lib import program_json
    o, v = sysm.o, sysm.v
    prog = program_json(o, v, method, block, 3)
    e = Emulator(prog, o, v)
    e.bind(S_TEI, tei)
    e.bind(S_F, (d["F"] if F is None else F).astype(np.complex128))
    e.bind(S_T1, d["t1"])
    e.bind(S_T2, d["t2"])
    e.bind(S_L1, d["l1"])
    e.bind(S_L2, d["l2"])
    e.bind(S_OUT, np.zeros(o * o * v * v, dtype=np.complex128))
    e.bind(S_MU, np.stack(sysm.mu))
    e.bind(S_RES, np.zeros(3, dtype=np.complex128))
    return e, prog


@pytest.mark.parametrize("method,block", sorted(GOLD))
def test_program_matches_reference(case, method, block):
    d, sysm, tei = case
    e, _ = _emu(d, sysm, tei, method, block)
    e.run("all")
    ref = d[GOLD[(method, block)]]
    got = e.bufs[S_OUT][: ref.size].reshape(ref.shape)
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("method,block", sorted(GOLD))
def test_prologue_independent_of_varying_inputs(case, method, block):
    d, sysm, tei = case
    e, prog = _emu(d, sysm, tei, method, block)
    vslot = S_T1 + block
    good_v = e.bufs[vslot].copy()
    good_f = e.bufs[S_F].copy()
    e.bufs[vslot] = np.full_like(good_v, np.nan)
    e.bufs[S_F] = np.full_like(good_f, np.nan)
    e.run("setup")
    e.run("prologue")
    e.bufs[vslot] = good_v
    e.bufs[S_F] = good_f
    e.run("stage")
    ref = d[GOLD[(method, block)]]
    got = e.bufs[S_OUT][: ref.size].reshape(ref.shape)
    assert np.isfinite(got).all()
    assert rel_err(got, ref) < 1e-12
    # the expensive contractions must leave the stage loop
    n_prologue = sum(1 for op in prog["ops"] if not op["varying"])
    if block in (1, 3) or method == "CCSD":
        assert n_prologue > 0


def test_density_program_matches_reference(case):
    d, sysm, tei = case
    e, _ = _emu(d, sysm, tei, "CCSD", 4)
    e.run("all")
    assert abs(e.bufs[S_RES][2] - d["mu"][2]) < 1e-14


def test_stage_flops_below_reference_step():
    """Per-step contraction flops of the hoisted programs vs the reference's
    16 full right-hand sides (o=10, v=38)."""
    from python_code_to_check_c_gb300._lib import program_json
    tot = 0
    for block in range(4):
        prog = program_json(10, 38, "CCSD", block, 3)
        for op in prog["ops"]:
            if op["kind"] == "gemm":
                tot += op["flops"] * (4 if op["varying"] else 1)
    assert tot < 5.76e10  # the reference step's flops at o=10, v=38
