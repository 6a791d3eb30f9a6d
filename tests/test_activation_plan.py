"""Reverse mode's activation records, planned on the host (no GPU): the
forward step graph keeps, per step, exactly the forward values the
reverse-mode programs read -- those written by prologue ops once per step,
those written by stage ops once per stage -- in non-overlapping, 256-byte
aligned entries.  The plan comes from the exported op lists
(tdcc_adjoint_program_json), the check re-derives it from the ops' read and
write slots and phase flags."""
import pytest

from python_code_to_check_c_gb300 import _lib

ELEM = {0: 8, 1: 16}


@pytest.mark.parametrize("method", ["CCSD", "CC2"])
@pytest.mark.parametrize("block", [0, 1, 2, 3])
@pytest.mark.parametrize("nb", [1, 3])
def test_activation_plan(method, block, nb):
    f = _lib.program_json(4, 8, method, block, 1, nb)
    a = _lib.adjoint_program_json(4, 8, method, block, 1, nb)
    nf = a["nfwd"]
    assert len(f["slots"]) == nf
    reads = {r for op in a["ops"] for r in op["reads"] if 0 <= r < nf}
    stage_w = {op["write"] for op in f["ops"] if op["write"] >= 0 and op["varying"]}
    pro_w = {op["write"] for op in f["ops"] if op["write"] >= 0 and not op["varying"] and not op["const"]}
    act = a["act"]
    got_stage = {s for s, st in zip(act["slots"], act["stage"]) if st}
    got_pro = {s for s, st in zip(act["slots"], act["stage"]) if not st}
    assert got_stage == reads & stage_w
    assert got_pro == (reads & pro_w) - stage_w
    assert not any(f["slots"][s]["fixed"] for s in act["slots"])  # integrals and inputs are bound, not kept
    for part, size in ((0, act["pro8"]), (1, act["stage8"])):
        ents = sorted((o, s) for s, st, o in zip(act["slots"], act["stage"], act["off8"]) if st == part)
        end = 0
        for off, s in ents:
            words = (f["slots"][s]["numel"] * ELEM[f["slots"][s]["dt"]] + 7) // 8
            assert off % 32 == 0 and off >= end
            end = off + words
        assert end <= size
    # the stage part holds the values of the varying amplitude's products
    if block in (1, 3) and method == "CCSD":
        assert got_stage
