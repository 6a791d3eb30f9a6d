"""Launch-shape and memory choices must not change results: workspace buffer
sharing forced on, the autotuner's picks, and the tensor-core kernel forms
(with 5 slices the 64- and 32-column tiles; with 4 the 128-column tile and
the persistent 64-column form as well), against the default configuration
(FP64 and mixed)."""
import numpy as np
import pytest

from golden_util import load, rel_err

pytestmark = pytest.mark.gpu


def _np(x):
    return x.detach().cpu().numpy()


def _run(method, prec, nb, sharing=None, tune=False, steps=8):
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    d, sysm = load("golden_o6_v10.npz")
    eng = CCEngine.from_system(sysm, nb=nb)
    try:
        if prec.startswith("mixed"):
            eng.set_precision("mixed", 4 if prec == "mixed4" else 5)
            eng.set_tc_policy(0, 1, 1)
        if sharing is not None:
            eng.set_memory_sharing(sharing)
        st = [d["t1"] + 0j, d["t2"] + 0j, d["l1"] + 0j, d["l2"] + 0j]
        if nb > 1:
            st = [np.stack([x * (1 + 0.1 * z) for z in range(nb)]) for x in st]
        eng.set_fields([make_field("sin", 0.002 * (1 + z), 0.923) for z in range(nb)], [2] * nb)
        if tune:
            eng.autotune(method, st)
        fin, traj = eng.propagate(method, st, 0.0, 0.01, steps, None)
        eng.check_errors()
        return _np(traj), [_np(x) for x in fin]
    finally:
        eng.close()


@pytest.mark.parametrize("method,prec,nb", [("CCSD", "fp64", 1), ("CCSD", "mixed", 3), ("CC2", "mixed", 2),
                                            ("CCSD", "mixed4", 3)])
def test_buffer_sharing_and_autotune_keep_results(method, prec, nb):
    ref_mu, ref_st = _run(method, prec, nb)
    for kw in ({"sharing": 0}, {"tune": True}, {"sharing": 0, "tune": True}):
        mu, stt = _run(method, prec, nb, **kw)
        tol = 1e-12 if prec == "fp64" else 1e-10
        assert np.abs(mu - ref_mu).max() < tol, kw
        for a, b in zip(stt, ref_st):
            assert rel_err(a, b) < 1e2 * tol, kw
