"""Seeded synthetic molecular systems (integral provider).

The reference obtains its integrals from psi4 (``CCSD_Helper.py:26-93``:
``mo_spin_eri``, ``F_MO``; dipoles at ``CCSD_Helper.py:970-980``).  psi4 is not
available here, so systems are drawn from a seeded density-fitting model:

* ``B[Q,p,q] ~ 0.05 N(0,1)``, symmetrised in ``pq``;
* ``(pr|qs) = sum_Q B[Q,p,r] B[Q,q,s]`` and
  ``<pq||rs> = (pr|qs) - (ps|qr)`` (antisymmetrised physicist notation,
  occupied orbitals first, as ``mo_spin_eri`` returns them);
* canonical Fock: occupied diagonal ~ U[-1.5,-0.3], virtual diagonal
  ~ U[0.2,3.0], each sorted ascending (the reference's ``eigh`` denominators
  are sorted, ``CCSD_Helper.py:327``), off-diagonal zero;
* ``mu_z`` random symmetric with Frobenius norm 1 (x and y are zero unless
  ``all_dipoles``: then drawn the same way after mu_z).

The draw order is fixed (B, occupied energies, virtual energies, mu_z) so a
seed names a system on every platform (numpy's PCG64 streams are
platform-independent).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class System:
    o: int
    v: int
    nq: int
    seed: int
    B: np.ndarray          # (Q, n, n) float64 (None when tei_full is given)
    fock: np.ndarray       # (n, n) float64
    mu: list = field(default_factory=list)   # [mu_x, mu_y, mu_z], each (n, n)
    tei_full: np.ndarray = None              # explicit <pq||rs> (psi4 systems)
    scf_energy: float = 0.0

    @property
    def n(self) -> int:
        return self.o + self.v

    def tei(self) -> np.ndarray:
        """Antisymmetrised <pq||rs> as an (n,n,n,n) float64 array (host)."""
        if self.tei_full is not None:
            return self.tei_full
        return tei_from_df(self.B)

    def eps(self) -> np.ndarray:
        return np.diag(self.fock).copy()


def synthetic_system(o: int, v: int, nq: int, seed: int, all_dipoles: bool = False) -> System:
    """``all_dipoles``: also draw mu_x and mu_y (same distribution, drawn after
    mu_z, so mu_z and everything before it are unchanged) for runs over
    several polarisations."""
    rng = np.random.default_rng(seed)
    n = o + v
    B = rng.standard_normal((nq, n, n)) * 0.05
    B = 0.5 * (B + B.transpose(0, 2, 1))
    eo = np.sort(rng.uniform(-1.5, -0.3, o))
    ev = np.sort(rng.uniform(0.2, 3.0, v))

    def dipole():
        M = rng.standard_normal((n, n))
        M = 0.5 * (M + M.T)
        return M / np.linalg.norm(M)

    mu_z = dipole()
    fock = np.diag(np.concatenate([eo, ev]))
    if all_dipoles:
        mu_x, mu_y = dipole(), dipole()
    else:
        mu_x, mu_y = np.zeros((n, n)), np.zeros((n, n))
    return System(o=o, v=v, nq=nq, seed=seed, B=B, fock=fock, mu=[mu_x, mu_y, mu_z])


def tei_from_df(B: np.ndarray) -> np.ndarray:
    nq, n, _ = B.shape
    Bm = B.reshape(nq, n * n)
    # phys[p,q,r,s] = (pr|qs) = sum_Q B[Q,p,r] B[Q,q,s]
    J = (Bm.T @ Bm).reshape(n, n, n, n)          # J[p,r,q,s]
    phys = J.transpose(0, 2, 1, 3)               # [p,q,r,s]
    return np.ascontiguousarray(phys - phys.transpose(0, 1, 3, 2))


def system_from_psi4(psi4) -> System:
    """The integrals CCSD_Helper.__init__ builds from a psi4 SCF
    (CCSD_Helper.py:26-93, 970-980): spin-orbital <pq||rs> from
    ``mo_spin_eri``, the MO Fock matrix and the three dipole matrices, spin
    interleaved (each spatial index p becomes 2p, 2p+1)."""
    wfn = psi4.scf_helper("SCF", return_wfn=True)
    scf_e = float(psi4.energy("scf"))
    mints = psi4.core.MintsHelper(wfn.basisset())
    mol = psi4.core.get_active_molecule()
    nmo = wfn.nmo()
    ndocc = int(sum(mol.Z(a) for a in range(mol.natom())) / 2)
    C = wfn.Ca()
    Cn = np.asarray(C)
    H = np.asarray(mints.ao_kinetic()) + np.asarray(mints.ao_potential())
    tei = np.asarray(mints.mo_spin_eri(C, C))
    o = 2 * ndocc
    spin = lambda X: np.kron(X, np.eye(2))  # noqa: E731
    fock = spin(Cn.T @ H @ Cn) + np.einsum("pmqm->pq", tei[:, :o, :, :o])
    mu = [spin(Cn.T @ np.asarray(d) @ Cn) for d in mints.so_dipole()]
    return System(o=o, v=2 * nmo - o, nq=0, seed=-1, B=None, fock=fock, mu=mu, tei_full=tei,
                  scf_energy=scf_e)


def mp2_guess(tei: np.ndarray, eps: np.ndarray, o: int) -> np.ndarray:
    """t2 = <ij||ab> / (e_i + e_j - e_a - e_b) (``CCSD_Helper.py:102-124``)."""
    return mp2_guess_oovv(tei[:o, :o, o:, o:], eps, o)


def mp2_guess_oovv(oovv: np.ndarray, eps: np.ndarray, o: int) -> np.ndarray:
    """The same from the <ij||ab> block alone."""
    eo, ev = eps[:o], eps[o:]
    d = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
    return oovv / d


# Named workloads (sizes and generator parameters of the synthetic systems).
WORKLOADS = {
    "ccsd_o10_v14": dict(o=10, v=14, nq=72, seed=1014),
    "ccsd_o10_v38": dict(o=10, v=38, nq=144, seed=1038),
    "o8_v30": dict(o=8, v=30, nq=144, seed=830),
    "o14_v58": dict(o=14, v=58, nq=144, seed=1458),
    "o18_v82": dict(o=18, v=82, nq=144, seed=1882),
    "o24_v160": dict(o=24, v=160, nq=480, seed=24160),
    "o6_v12": dict(o=6, v=12, nq=72, seed=612),
}
