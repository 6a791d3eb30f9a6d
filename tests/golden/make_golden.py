"""Generates the golden fixtures by running the reference's own Python code.

Run in a container that has the reference checkout (read-only) and
opt_einsum; psi4 and pandas are replaced by empty stub modules because only
the integral setup and the CSV writers use them, and neither is exercised:

    python tests/golden/make_golden.py /path/to/reference

The helper objects are built with ``__new__`` (skipping the psi4 SCF in
``CCSD_Helper.__init__``) and given ``occ``/``vir``/``TEI`` from the seeded
synthetic system of ``python_code_to_check_c_gb300.system``.  Outputs:

* ``golden_o{o}_v{v}.npz`` -- for a random complex state: every T/L residual
  (CCSD and CC2), the Hbar intermediates, the density blocks and the dipole;
  for the smallest size also the ground-state DIIS energies/amplitudes, one
  block-frozen RK4 step (``ft1/ft2/fL1/fL2`` and CC2 variants) and a short
  mu_z(t) trajectory of the reference loop body.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from python_code_to_check_c_gb300.system import synthetic_system, mp2_guess  # noqa: E402


def load_reference(ref_dir):
    stub_dir = tempfile.mkdtemp(prefix="refstubs_")
    for name in ("psi4", "pandas"):
        with open(os.path.join(stub_dir, name + ".py"), "w") as f:
            f.write("# empty stub: the reference's psi4/pandas uses are not exercised\n")
    sys.path.insert(0, stub_dir)
    sys.path.insert(1, ref_dir)
    sys.dont_write_bytecode = True
    import CC2_Helper as cc2mod  # noqa: F401  (imports CCSD_Helper too)
    return cc2mod


def make_helper(mod, tei, o, mu):
    h = mod.CC2_Helper.__new__(mod.CC2_Helper)
    n = tei.shape[0]
    h.occ = slice(0, o)
    h.vir = slice(o, n)
    h.TEI = tei
    h.Defd_dipole = lambda: mu
    # The Hartree-Fock density built inside dipole_moment is discarded by the
    # reference (CCSD_Helper.py:1080-1088); stub it to avoid psi4 overlaps.
    h.Buildpho = lambda F: np.zeros((n, n))
    h.pholowdinbasis = lambda p: p
    return h


def random_state(rng, o, v, scale1=0.05, scale2=0.02):
    def c(shape, s):
        return s * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    t1 = c((o, v), scale1)
    l1 = c((o, v), scale1)
    t2 = c((o, o, v, v), scale2)
    l2 = c((o, o, v, v), scale2)
    t2 = 0.5 * (t2 - t2.transpose(1, 0, 2, 3))
    t2 = 0.5 * (t2 - t2.transpose(0, 1, 3, 2))
    l2 = 0.5 * (l2 - l2.transpose(1, 0, 2, 3))
    l2 = 0.5 * (l2 - l2.transpose(0, 1, 3, 2))
    return t1, t2, l1, l2


def residual_fixture(mod, o, v, nq, seed, full):
    sysm = synthetic_system(o, v, nq, seed)
    tei = sysm.tei()
    n = o + v
    mu = [np.asarray(m) for m in sysm.mu]
    h = make_helper(mod, tei, o, mu)
    rng = np.random.default_rng(seed + 7)
    t1, t2, l1, l2 = random_state(rng, o, v)
    # a complex, field-dressed Fock matrix (F + V(t) in the propagator)
    F = sysm.fock + (-0.002 * np.exp(0.37j)) * mu[2]
    out = dict(o=o, v=v, nq=nq, seed=seed, t1=t1, t2=t2, l1=l1, l2=l2, F=F)
    out["T1"] = h.T1eq_rhs(t1, t2, F)
    out["T2"] = h.T2eq_rhs(t1, t2, F)
    out["L1"] = h.lam_1eq_rhs(t1, t2, l1, l2, F)
    out["L2"] = h.lam2eq_rhs(t1, t2, l1, l2, F)
    out["T2_CC2"] = h.T2eq_rhs_CC2(t1, t2, F)
    out["L1_CC2"] = h.L1eq_rhs_CC2(t1, t2, l1, l2, F)
    out["L2_CC2"] = h.L2eq_rhs_CC2(t1, t2, l1, l2, F)
    out["Dij"] = h.Dij(t1, t2, l1, l2)
    out["Dab"] = h.Dab(t1, t2, l1, l2)
    out["Dai"] = h.Dai(t1, t2, l1, l2)
    out["mu"] = np.array(h.dipole_moment(t1, t2, l1, l2, F))
    if full:
        for name in ("Fae", "Fmi", "Fme", "Wmnij", "Wabef", "Wmbej", "LRFea", "LRFim",
                     "LSWieam", "LRWefam", "LRWibjm", "LSWmnij", "LSWabef"):
            out["I_" + name] = getattr(h, name)(t1, t2, F)
        out["I_Wmnij_2"] = h.Wmnij_2(t1, t2, F)
        out["I_Wabef_2"] = h.Wabef_2(t1, t2, F)
        out["I_Gfe"] = h.Gfe(t2, l2)
        out["I_Gmn"] = h.Gmn(t2, l2)
        out["I_LWfiea"] = h.LWfiea(t1)
        out["I_LWmina"] = h.LWmina(t1)
    return sysm, h, out


def ground_and_dynamics(mod, sysm, h, out):
    o = sysm.o
    F = sysm.fock.copy()
    mu_z = sysm.mu[2]
    tei = sysm.tei()
    t2 = mp2_guess(tei, sysm.eps(), o)
    t1 = np.zeros((o, sysm.v), dtype=np.longdouble)
    E, t1, t2 = h.DIIS_solver(t1, t2, F, 7, 40, 1e-15)
    El, l1, l2 = h.DIIS_solver_Lam(t1, t2, t1, t2, F, 7, 30, 1e-15)
    out["gs_E_ccsd"] = np.float64(E)
    out["gs_pseudo_ccsd"] = np.float64(El)
    out["gs_t1"], out["gs_t2"] = np.float64(t1), np.float64(t2)
    out["gs_l1"], out["gs_l2"] = np.float64(l1), np.float64(l2)
    t2c = mp2_guess(tei, sysm.eps(), o)
    t1c = np.zeros((o, sysm.v))
    Ec, t1c, t2c = h.DIIS_solver_CC2(t1c, t2c, F, 7, 40, 1e-15)
    Elc, l1c, l2c = h.DIIS_solver_Lam_CC2(t1c, t2c, t1c, t2c, F, 7, 30, 1e-15)
    out["gs_E_cc2"] = np.float64(Ec)
    out["gs_pseudo_cc2"] = np.float64(Elc)
    out["gs_t1_cc2"], out["gs_t2_cc2"] = t1c, t2c
    out["gs_l1_cc2"], out["gs_l2_cc2"] = l1c, l2c

    # One block-frozen RK4 step from the random complex state, with the
    # reference's own field Vt(t) = -A mu_z exp(i 2 pi w0 t).
    A, w0, dt, t = 0.005, 0.968635, 0.01, 0.01
    import cmath

    def Vt(tt):
        return -A * mu_z * cmath.exp(1j * w0 * 2 * np.pi * tt)

    s = (out["t1"], out["t2"], out["l1"], out["l2"])
    out["rk_ft1"] = h.ft1(t, dt, s[0], s[1], F, Vt)
    out["rk_ft2"] = h.ft2(t, dt, s[0], s[1], F, Vt)
    out["rk_fL1"] = h.fL1(t, dt, s[0], s[1], s[2], s[3], F, Vt)
    out["rk_fL2"] = h.fL2(t, dt, s[0], s[1], s[2], s[3], F, Vt)
    out["rk_ft2_CC2"] = h.ft2_CC2(t, dt, s[0], s[1], F, Vt)
    out["rk_fL1_CC2"] = h.fL1_CC2(t, dt, s[0], s[1], s[2], s[3], F, Vt)
    out["rk_fL2_CC2"] = h.fL2_CC2(t, dt, s[0], s[1], s[2], s[3], F, Vt)

    # mu_z(t) over the reference loop body (CCSD_Helper.py:1206-1240),
    # from the FP64 ground state, for CCSD and CC2, precs=15.
    for method in ("CCSD", "CC2"):
        if method == "CCSD":
            st = [out["gs_t1"] + 0j, out["gs_t2"] + 0j, out["gs_l1"] + 0j, out["gs_l2"] + 0j]
            f2, fl1, fl2 = h.ft2, h.fL1, h.fL2
        else:
            st = [t1c + 0j, t2c + 0j, l1c + 0j, l2c + 0j]
            f2, fl1, fl2 = h.ft2_CC2, h.fL1_CC2, h.fL2_CC2
        tt = 0.0
        mus = [h.dipole_moment(*st, F)[2]]
        precs = 15
        for _ in range(6):
            r = [np.around(x, decimals=precs) for x in st]
            tt += dt
            d1 = -1j * h.ft1(tt, dt, st[0], st[1], F, Vt)
            d2 = -1j * f2(tt, dt, st[0], st[1], F, Vt)
            e1 = 1j * fl1(tt, dt, st[0], st[1], st[2], st[3], F, Vt)
            e2 = 1j * fl2(tt, dt, st[0], st[1], st[2], st[3], F, Vt)
            st = [r[0] + d1, r[1] + d2, r[2] + e1, r[3] + e2]
            mus.append(h.dipole_moment(*st, F)[2])
        out["traj_mu_" + method] = np.array(mus)
        out["traj_final_t2_" + method] = st[1]
    out["traj_A"], out["traj_w0"], out["traj_dt"] = A, w0, dt


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the reference checkout>")
    ref_dir = sys.argv[1]
    mod = load_reference(ref_dir)
    cases = [(4, 8, 72, 48, True), (6, 10, 72, 610, False), (3, 5, 40, 35, False)]
    for o, v, nq, seed, full in cases:
        sysm, h, out = residual_fixture(mod, o, v, nq, seed, full)
        if full:
            ground_and_dynamics(mod, sysm, h, out)
        path = os.path.join(HERE, f"golden_o{o}_v{v}.npz")
        np.savez_compressed(path, **{k: np.asarray(x) for k, x in out.items()})
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
