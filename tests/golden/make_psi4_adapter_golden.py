"""Fixture for the psi4 integral adapter (``system.system_from_psi4``): runs
the reference's own integral setup -- ``CCSD_Helper.__init__``, ``TEI_MO``,
``F_MO`` and ``Defd_dipole`` (CCSD_Helper.py:26-93, 970-980) -- with the
deterministic psi4 stand-in of ``tests/fake_psi4.py`` (psi4 is not installed
here) and stores what it builds:

    python tests/golden/make_psi4_adapter_golden.py /path/to/reference

Output: ``psi4_adapter_fake.npz`` with the spin-orbital Fock matrix, the three
dipole matrices, <pq||rs>, the occupied spin-orbital count and the SCF energy.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import fake_psi4  # noqa: E402

PARAMS = dict(nao=4, electrons=2, seed=11)


def main(ref_dir):
    sys.modules["psi4"] = fake_psi4.make(**PARAMS)
    sys.modules["pandas"] = types.ModuleType("pandas")  # used only by the CSV writers
    sys.path.insert(0, ref_dir)
    import CCSD_Helper  # noqa: E402  (the reference's module)
    h = CCSD_Helper.CCSD_Helper(None)
    F = np.asarray(h.F_MO())
    mu = np.stack([np.asarray(m) for m in h.Defd_dipole()])
    out = os.path.join(HERE, "psi4_adapter_fake.npz")
    np.savez(out, F=F, mu=mu, tei=np.asarray(h.TEI), o=2 * h.ndocc, nmo=h.nmo, scf_e=float(h.scf_e),
             **{k: v for k, v in PARAMS.items()})
    print("wrote", out, F.shape, mu.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_psi4_adapter_golden.py <path of the reference checkout>")
    main(sys.argv[1])
