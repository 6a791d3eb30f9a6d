"""A deterministic stand-in for the psi4 calls the integral setup makes
(TEST INFRASTRUCTURE).  psi4 is not installed here; this module answers the
same calls the reference's ``CCSD_Helper.__init__`` / ``TEI_MO`` / ``F_MO`` /
``Defd_dipole`` (CCSD_Helper.py:26-93, 970-980) and the package's
``system_from_psi4`` make, from seeded AO matrices:

* ``core.get_active_molecule()``: a molecule with ``natom()`` and ``Z(i)``;
* ``scf_helper('SCF', return_wfn=True)``: a wavefunction with ``nmo()``,
  ``Ca()`` (MO coefficients, ascending orbital energies), ``Ca_subset``,
  ``epsilon_a()`` and ``basisset()``;
* ``energy(name)``: a fixed number per method;
* ``core.MintsHelper(basis)``: ``ao_overlap()`` (with an in-place
  ``power``), ``ao_kinetic()``, ``ao_potential()``, ``so_dipole()`` and
  ``mo_spin_eri(C, C)`` -- the antisymmetrised spin-orbital integrals
  <PQ||RS> with spin interleaved (P = 2p + spin), built from seeded AO
  electron-repulsion integrals (pr|qs) = sum_Q B_Q,pr B_Q,qs.
"""
from __future__ import annotations

import types

import numpy as np


class _Mat:
    """A matrix with psi4's in-place ``power`` and ``print_out``."""

    def __init__(self, a):
        self.a = np.array(a, dtype=np.float64)

    def __array__(self, dtype=None, copy=None):
        return self.a if dtype is None else self.a.astype(dtype)

    def power(self, p, tol):
        w, v = np.linalg.eigh(self.a)
        w = np.where(w > tol, w, 0.0)
        self.a = (v * np.where(w > 0, w ** p, 0.0)) @ v.T

    def print_out(self):
        pass


def make(nao=4, electrons=2, seed=11):
    rng = np.random.default_rng(seed)

    def sym(scale):
        m = rng.standard_normal((nao, nao)) * scale
        return 0.5 * (m + m.T)

    S = np.eye(nao) + sym(0.05)
    T = sym(0.4) + np.diag(np.linspace(0.5, 2.0, nao))
    V = sym(0.3) - np.diag(np.linspace(2.0, 0.5, nao))
    B = rng.standard_normal((3 * nao, nao, nao)) * 0.1
    B = 0.5 * (B + B.transpose(0, 2, 1))
    eri = np.einsum("Qpr,Qqs->prqs", B, B)  # (pr|qs)
    dip = [sym(0.5) for _ in range(3)]
    # orthonormal MOs (S-metric) from the one-electron Hamiltonian, ascending
    s_half = np.linalg.inv(np.linalg.cholesky(S)).T
    w, u = np.linalg.eigh(s_half.T @ (T + V) @ s_half)
    C = s_half @ u
    eps = w

    def mo_spin_eri(C1, C2):
        Cm = np.asarray(C1)
        mo = np.einsum("prqs,pi,rj,qk,sl->ijkl", eri, Cm, Cm, Cm, Cm)  # (ij|kl), chemists'
        n = 2 * Cm.shape[1]
        g = np.zeros((n, n, n, n))
        sp = np.arange(n) % 2
        idx = np.arange(n) // 2
        # <PQ|RS> = (PR|QS) with spin conservation, then antisymmetrised
        phys = mo[idx[:, None, None, None], idx[None, None, :, None], idx[None, :, None, None],
                  idx[None, None, None, :]]
        spin = ((sp[:, None, None, None] == sp[None, None, :, None]) &
                (sp[None, :, None, None] == sp[None, None, None, :]))
        g = phys * spin
        return g - g.transpose(0, 1, 3, 2)

    class Mol:
        def natom(self):
            return 1

        def Z(self, i):
            return electrons

    class Wfn:
        def nmo(self):
            return nao

        def Ca(self):
            return C.copy()

        def Ca_subset(self, basis, space):
            return _Mat(C)

        def epsilon_a(self):
            return eps.copy()

        def basisset(self):
            return "fake-basis"

    class Mints:
        def __init__(self, basis):
            pass

        def ao_overlap(self):
            return _Mat(S)

        def ao_kinetic(self):
            return T.copy()

        def ao_potential(self):
            return V.copy()

        def so_dipole(self):
            return [d.copy() for d in dip]

        def mo_spin_eri(self, C1, C2):
            return mo_spin_eri(C1, C2)

    mod = types.ModuleType("psi4")
    mod.core = types.SimpleNamespace(get_active_molecule=lambda: Mol(), MintsHelper=Mints)
    mod.scf_helper = lambda name, return_wfn=True: Wfn()
    mod.energy = lambda name: {"scf": -1.25, "ccsd": -1.30}.get(name, 0.0)
    return mod
