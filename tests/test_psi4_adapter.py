"""The psi4 integral adapter (``system_from_psi4``) against the reference's
own integral setup (``CCSD_Helper.__init__`` / ``TEI_MO`` / ``F_MO`` /
``Defd_dipole``, CCSD_Helper.py:26-93, 970-980), both driven by the same
deterministic psi4 stand-in (``tests/fake_psi4.py``); the reference's
outputs are the fixture ``tests/golden/psi4_adapter_fake.npz`` written by
``tests/golden/make_psi4_adapter_golden.py``.  No GPU."""
import os

import numpy as np

import fake_psi4

HERE = os.path.dirname(os.path.abspath(__file__))


def test_adapter_builds_the_reference_integrals():
    from python_code_to_check_c_gb300.system import system_from_psi4
    ref = np.load(os.path.join(HERE, "golden", "psi4_adapter_fake.npz"))
    psi4 = fake_psi4.make(nao=int(ref["nao"]), electrons=int(ref["electrons"]), seed=int(ref["seed"]))
    sysm = system_from_psi4(psi4)
    assert sysm.o == int(ref["o"]) and sysm.o + sysm.v == 2 * int(ref["nmo"])
    np.testing.assert_allclose(sysm.fock, ref["F"], rtol=0, atol=1e-13)
    for m, r in zip(sysm.mu, ref["mu"]):
        np.testing.assert_allclose(m, r, rtol=0, atol=1e-13)
    np.testing.assert_array_equal(sysm.tei_full, ref["tei"])
    assert sysm.scf_energy == float(ref["scf_e"])
    # spin structure: no alpha-beta coupling in the one-electron matrices
    sp = np.arange(sysm.o + sysm.v) % 2
    assert np.abs(sysm.fock[sp[:, None] != sp[None, :]]).max() == 0.0
