"""CPU oracle for the TD-CCSD / TD-CC2 hot path (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The GPU engine in
``python_code_to_check_c_gb300`` never calls into it.

It restates, in numpy complex128, the spin-orbital CC equations of the
reference (yramis/python_code_to_check_C).  Every function cites the
reference ``file:line`` it follows.  The equations are the method itself, so
each term (index pattern, prefactor, antisymmetriser) is the same as the
reference's; the code around them (how operands are sliced, how terms are
grouped, how antisymmetrisers are written) is this project's own.

Parity pin: ``tests/golden/make_golden.py`` imports the reference's own
``CCSD_Helper``/``CC2_Helper`` (psi4/pandas stubbed) in the build container
and stores its outputs as fixtures; ``tests/test_oracle_golden.py`` checks
this oracle against them (relative 1e-12).

Conventions (reference quirks kept on purpose):

* ``g`` is the antisymmetrised physicist tensor ``<pq||rs>`` (n^4, real),
  occupied orbitals first (``CCSD_Helper.py:49-50``).
* ``F`` is the full n x n Fock matrix, complex once the field is added
  (``CCSD_Helper.py:1158-1187``: ``F + Vt(t)``).
* einsum index strings are positional, exactly like the reference's
  ``opt_einsum.contract`` calls (e.g. ``'ijab,eb->ijab'`` sums over ``e``).
"""
from __future__ import annotations

import math
import time

import numpy as np


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _ein(spec, *ops):
    # torch tensors (the autograd cross-check of the engine's reverse-mode
    # programs) go through torch.einsum; everything else is numpy
    if any(_is_torch(x) for x in ops):
        import torch
        return torch.einsum(spec, *ops)
    return np.einsum(spec, *ops, optimize=True)


def _pij(x):
    """x - x with (i,j) swapped, on axes (0,1)."""
    return x - x.swapaxes(0, 1)


def _pab(x):
    """x - x with (a,b) swapped, on axes (2,3)."""
    return x - x.swapaxes(2, 3)


def _pijab(x):
    """P(ij)P(ab) x as written at CCSD_Helper.py:298 / 636-639."""
    return x - x.swapaxes(2, 3) - x.swapaxes(0, 1) + x.swapaxes(0, 1).swapaxes(2, 3)


def _outer(x, y):
    """'ia,jb->ijab'."""
    return x[:, None, :, None] * y[None, :, None, :]


class CCOracle:
    """Residuals, Hbar intermediates, RK4 block propagator and density of the
    reference, on a system given by its integrals.

    ``g``  : (n,n,n,n) float64 antisymmetrised ``<pq||rs>``
    ``o``  : number of occupied spin orbitals
    ``mu`` : list of dipole matrices (n x n); the z component is ``mu[-1]``
    """

    def __init__(self, g, o, mu=None):
        self.g = g if _is_torch(g) else np.asarray(g)
        self.n = self.g.shape[0]
        self.o = int(o)
        self.v = self.n - self.o
        self.mu = mu

    # -- blocks --------------------------------------------------------
    def G(self, blk):
        o, n = self.o, self.n
        sl = [slice(0, o) if c == "o" else slice(o, n) for c in blk]
        return self.g[sl[0], sl[1], sl[2], sl[3]]

    def Fb(self, F, blk):
        o, n = self.o, self.n
        s0 = slice(0, o) if blk[0] == "o" else slice(o, n)
        s1 = slice(0, o) if blk[1] == "o" else slice(o, n)
        return F[s0, s1]

    # -- CCSD one-body intermediates (CCSD_Helper.py:136-170) -----------
    def Fae(self, t1, t2, F):
        tau = t2 + _outer(t1, t1)
        return (self.Fb(F, "vv")
                - 0.5 * _ein("me,ma->ae", self.Fb(F, "ov"), t1)
                + _ein("mafe,mf->ae", self.G("ovvv"), t1)
                - 0.5 * _ein("mnef,mnaf->ae", self.G("oovv"), tau))

    def Fmi(self, t1, t2, F):
        tau = t2 + _outer(t1, t1)
        return (self.Fb(F, "oo")
                + 0.5 * _ein("me,ie->mi", self.Fb(F, "ov"), t1)
                + _ein("mnie,ne->mi", self.G("ooov"), t1)
                + 0.5 * _ein("mnef,inef->mi", self.G("oovv"), tau))

    def Fme(self, t1, t2, F):
        return self.Fb(F, "ov") + _ein("mnef,nf->me", self.G("oovv"), t1)

    # -- T1 residual (CCSD_Helper.py:177-196) ---------------------------
    def T1eq_rhs(self, t1, t2, F):
        fae = self.Fae(t1, t2, F)
        fmi = self.Fmi(t1, t2, F)
        fme = self.Fme(t1, t2, F)
        return (self.Fb(F, "ov")
                + _ein("ae,ie->ia", fae, t1)
                - _ein("mi,ma->ia", fmi, t1)
                + _ein("me,imae->ia", fme, t2)
                - _ein("naif,nf->ia", self.G("ovov"), t1)
                - 0.5 * _ein("nmei,mnae->ia", self.G("oovo"), t2)
                - 0.5 * _ein("maef,imef->ia", self.G("ovvv"), t2))

    # -- two-body intermediates (CCSD_Helper.py:199-265) ----------------
    def Wmnij(self, t1, t2, F=None):
        x = _ein("mnie,je->mnij", self.G("ooov"), t1)
        tau = 0.25 * t2 + 0.5 * _outer(t1, t1) - 0.5 * _outer(t1, t1).swapaxes(2, 3)
        return self.G("oooo") + _pab(x) + _ein("mnef,ijef->mnij", self.G("oovv"), tau)

    def Wmnij_2(self, t1, t2=None, F=None):
        x = _ein("mnie,je->mnij", self.G("ooov"), t1)
        y = 0.25 * _ein("mnef,ijef->mnij", self.G("oovv"), _outer(t1, t1))
        return self.G("oooo") + _pab(x) + _pab(y)

    def Wabef(self, t1, t2, F=None):
        x = -_ein("amef,mb->abef", self.G("vovv"), t1)
        y = 0.5 * _ein("mnef,mnab->abef", self.G("oovv"), _outer(t1, t1))
        return (self.G("vvvv") + _pij(x)
                + 0.25 * _ein("mnef,mnab->abef", self.G("oovv"), t2) + _pij(y))

    def Wabef_2(self, t1, t2=None, F=None):
        x = -_ein("amef,mb->abef", self.G("vovv"), t1)
        tt = _outer(t1, t1)
        tau = tt - tt.swapaxes(2, 3)
        return self.G("vvvv") + _pij(x) + 0.25 * _ein("mnef,mnab->abef", self.G("oovv"), tau)

    def Wmbej(self, t1, t2, F=None):
        t2t1 = 0.5 * t2 + _ein("jf,nb->jnfb", t1, t1)
        return (self.G("ovvo")
                - _ein("mnej,nb->mbej", self.G("oovo"), t1)
                - _ein("mnef,jnfb->mbej", self.G("oovv"), t2t1)
                + _ein("mbef,jf->mbej", self.G("ovvv"), t1))

    # -- T2 residual (CCSD_Helper.py:268-309) ---------------------------
    def T2eq_rhs(self, t1, t2, F):
        g = self.G
        fae = self.Fae(t1, t2, F)
        fmi = self.Fmi(t1, t2, F)
        fme = self.Fme(t1, t2, F)
        tau = _outer(t1, t1) - _outer(t1, t1).swapaxes(2, 3)
        be = fae - 0.5 * _ein("me,mb->be", fme, t1)
        mj = fmi + 0.5 * _ein("me,je->mj", fme, t1)
        ring = (_ein("mbej,imae->ijab", self.Wmbej(t1, t2), t2)
                - _ein("mbej,ie,ma->ijab", g("ovvo"), t1, t1))
        return (g("oovv")
                + _pab(_ein("be,ijae->ijab", be, t2))
                + _pij(-_ein("mj,imab->ijab", mj, t2))
                + (0.5 * _ein("mnij,mnab->ijab", self.Wmnij(t1, t2), t2)
                   + 0.5 * _ein("mnij,mnab->ijab", self.Wmnij_2(t1), tau))
                + (0.5 * _ein("abef,ijef->ijab", self.Wabef(t1, t2), t2)
                   + 0.5 * _ein("abef,ijef->ijab", self.Wabef_2(t1), tau))
                + _pijab(ring)
                + _pij(_ein("abej,ie->ijab", g("vvvo"), t1))
                + _pab(-_ein("mbij,ma->ijab", g("ovoo"), t1)))

    # -- energies and Jacobi updates (CCSD_Helper.py:312-344, 650-677) ---
    def CCSD_Corr_E(self, t1, t2, F):
        g = self.G("oovv")
        return (_ein("ia,ia->", self.Fb(F, "ov"), t1)
                + 0.25 * _ein("ijab,ijab->", g, t2)
                + 0.5 * _ein("ijab,ia,jb->", g, t1, t1))

    def CCSD_pseudo_E(self, t1, t2, l1, l2, F):
        return (_ein("ia,ia->", self.Fb(F, "ov"), l1),
                0.25 * _ein("ijab,ijab->", self.G("oovv"), l2))

    def _denoms(self, F):
        eps = np.linalg.eigh(F)[0]
        eo, ev = eps[: self.o], eps[self.o:]
        d1 = eo[:, None] - ev[None, :]
        d2 = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
        return 1.0 / d1, 1.0 / d2

    def corrected_T1(self, t1, r1, F):
        return t1 + r1 * self._denoms(F)[0]

    def corrected_T2(self, t2, r2, F):
        return t2 + r2 * self._denoms(F)[1]

    corrected_lam1 = corrected_T1
    corrected_lam2 = corrected_T2

    def MP2_guess(self, F):
        """t2 = <ij||ab>/D_ijab with eigh(F) denominators (CCSD_Helper.py:102-124)."""
        return self.G("oovv") * self._denoms(F)[1]

    # -- Lambda Hbar intermediates (CCSD_Helper.py:447-550, 586-607) -----
    def LRFea(self, t1, t2, F):
        tau = 0.5 * t2 + _outer(t1, t1)
        return (self.Fb(F, "vv")
                - _ein("ma,me->ea", self.Fb(F, "ov"), t1)
                + _ein("emaf,mf->ea", self.G("vovv"), t1)
                - _ein("mnaf,mnef->ea", self.G("oovv"), tau))

    def LRFim(self, t1, t2, F):
        tau = 0.5 * t2 + _outer(t1, t1)
        return (self.Fb(F, "oo")
                + _ein("ie,me->im", self.Fb(F, "ov"), t1)
                + _ein("inmf,nf->im", self.G("ooov"), t1)
                + _ein("inef,mnef->im", self.G("oovv"), tau))

    def LSWieam(self, t1, t2, F=None):
        tau = t2 + _outer(t1, t1)
        return (self.G("ovvo")
                + _ein("eifa,mf->ieam", self.G("vovv"), t1)
                - _ein("nima,ne->ieam", self.G("ooov"), t1)
                - _ein("ijab,mjbe->ieam", self.G("oovv"), tau))

    def LSWmnij(self, t1, t2, F=None):
        tau = 0.25 * t2 + 0.5 * _outer(t1, t1)
        return (0.5 * self.G("oooo")
                + _ein("ijme,ne->ijmn", self.G("ooov"), t1)
                + _ein("ijfe,mnfe->ijmn", self.G("oovv"), tau))

    def LSWabef(self, t1, t2, F=None):
        tau = 0.25 * t2 + 0.5 * _outer(t1, t1)
        return (0.5 * self.G("vvvv")
                - _ein("emab,mf->efab", self.G("vovv"), t1)
                + _ein("nmab,nmef->efab", self.G("oovv"), tau))

    def LRWefam(self, t1, t2, F):
        g = self.G
        fme = self.Fme(t1, t2, F)
        jfam = -g("ovvo") + _ein("jnab,nmfb->jfam", g("oovv"), t2)
        tau = 0.25 * t2 + 0.5 * _outer(t1, t1)
        return 0.5 * g("vvvo") + (
            0.5 * _ein("na,mnef->efam", fme, t2)
            + _ein("efab,mb->efam", self.LSWabef(t1, t2), t1)
            + _ein("jfam,je->efam", jfam, t1)
            + _ein("jnam,jnef->efam", g("oovo"), tau)
            - _ein("jfab,jmeb->efam", g("ovvv"), t2))

    def LRWibjm(self, t1, t2, F):
        g = self.G
        fme = self.Fme(t1, t2, F)
        ibem = -g("ovvo") - _ein("inef,nmfb->ibem", g("oovv"), t2)
        tau = 0.25 * t2 + 0.5 * _outer(t1, t1)
        return -0.5 * g("ovoo") + (
            0.5 * _ein("ie,jmbe->ibjm", fme, t2)
            + _ein("injm,nb->ibjm", self.LSWmnij(t1, t2), t1)
            + _ein("ibem,je->ibjm", ibem, t1)
            - _ein("ibef,jmef->ibjm", g("ovvv"), tau)
            + _ein("inem,jneb->ibjm", g("oovo"), t2))

    def Gfe(self, t2, l2):
        return -0.5 * _ein("mnfb,mneb->fe", l2, t2)

    def Gmn(self, t2, l2):
        return 0.5 * _ein("njed,mjed->nm", l2, t2)

    def LWfiea(self, t1):
        return self.G("vovv") - _ein("jiea,jf->fiea", self.G("oovv"), t1)

    def LWmina(self, t1):
        return self.G("ooov") + _ein("mifa,nf->mina", self.G("oovv"), t1)

    # -- Lambda residuals (CCSD_Helper.py:555-581, 610-648) --------------
    def lam_1eq_rhs(self, t1, t2, l1, l2, F):
        gfe = self.Gfe(t2, l2)
        gmn = self.Gmn(t2, l2)
        return (self.Fme(t1, t2, F)
                + (_ein("ea,ie->ia", self.LRFea(t1, t2, F), l1)
                   - _ein("im,ma->ia", self.LRFim(t1, t2, F), l1)
                   + _ein("ieam,me->ia", self.LSWieam(t1, t2), l1))
                + _ein("efam,imef->ia", self.LRWefam(t1, t2, F), l2)
                + _ein("ibjm,jmab->ia", self.LRWibjm(t1, t2, F), l2)
                - _ein("fe,fiea->ia", gfe, self.LWfiea(t1))
                - _ein("nm,mina->ia", gmn, self.LWmina(t1)))

    def lam2eq_rhs(self, t1, t2, l1, l2, F):
        g = self.G
        gbe = self.Gfe(t2, l2)
        gmj = self.Gmn(t2, l2)
        fme = self.Fme(t1, t2, F)
        ring = (_ein("jebm,imae->ijab", self.LSWieam(t1, t2), l2)
                + _ein("jb,ia->ijab", fme, l1))
        return (g("oovv")
                + _pab(_ein("eb,ijae->ijab", self.LRFea(t1, t2, F), l2))
                + _pij(-_ein("jm,imab->ijab", self.LRFim(t1, t2, F), l2))
                + _ein("ijmn,mnab->ijab", self.LSWmnij(t1, t2), l2)
                + (_ein("efab,ijef->ijab", self.LSWabef(t1, t2), l2)
                   + _pij(_ein("ejab,ie->ijab", self.LWfiea(t1), l1)))
                + _pab(-_ein("ijmb,ma->ijab", self.LWmina(t1), l1))
                + _pijab(ring)
                + _pab(_ein("ijfb,af->ijab", g("oovv"), gbe))
                + _pij(-_ein("mjab,im->ijab", g("oovv"), gmj)))

    # -- CC2 residuals (CC2_Helper.py:12-175) ----------------------------
    def T2eq_rhs_CC2(self, t1, t2, F):
        g = self.G
        tau = _outer(t1, t1) - _outer(t1, t1).swapaxes(2, 3)
        return (g("oovv")
                + _pab(_ein("be,ijae->ijab", self.Fb(F, "vv"), t2))
                + _pij(-_ein("mj,imab->ijab", self.Fb(F, "oo"), t2))
                + 0.5 * _ein("mnij,mnab->ijab", self.Wmnij_2(t1), tau)
                + 0.5 * _ein("abef,ijef->ijab", self.Wabef_2(t1), tau)
                + _pijab(-_ein("mbej,ie,ma->ijab", g("ovvo"), t1, t1))
                + _pij(_ein("abej,ie->ijab", g("vvvo"), t1))
                + _pab(-_ein("mbij,ma->ijab", g("ovoo"), t1)))

    def L1eq_rhs_CC2(self, t1, t2, l1, l2, F):
        g = self.G
        r = (self.Fme(t1, t2, F)
             + _ein("ea,ie->ia", self.LRFea(t1, t2, F), l1)
             - _ein("im,ma->ia", self.LRFim(t1, t2, F), l1))
        tt = _outer(t1, t1)
        # Wmbej with t1 only (CC2_Helper.py:73-77)
        wmbej = (g("ovvo") + _ein("mbef,jf->mbej", g("ovvv"), t1)
                 - _ein("mnej,nb->mbej", g("oovo"), t1)
                 - _ein("mnef,jnfb->mbej", g("oovv"), tt))
        gbj = -_ein("me,mjbe->bj", l1, t2)
        r = r + _ein("ijab,bj->ia", g("oovv"), gbj)
        r = r + _ein("ieam,me->ia", wmbej, l1)
        # Wmnij, Wmbij (CC2_Helper.py:89-104)
        tau = tt - tt.swapaxes(2, 3)
        wmnij = (g("oooo") + _ein("mnie,je->mnij", g("ooov"), t1)
                 - _ein("mnje,ie->mnij", g("ooov"), t1)
                 - 0.5 * _ein("ijef,mnfe->ijmn", g("oovv"), tau))
        wmbij = (g("ovoo") - _ein("nb,mnij->mbij", t1, wmnij)
                 + 0.5 * _ein("mbef,ijef->mbij", g("ovvv"), tau))
        z = _ein("mbei,je->mbij", g("ovvo"), t1) - _ein("mbej,ie->mbij", g("ovvo"), t1)
        wmbij = wmbij - z
        r = r - 0.5 * _ein("iemn,mnae->ia", wmbij, l2)
        # Wabei (CC2_Helper.py:107-122)
        zmbej = (g("ovvo") + _ein("mbef,jf->mbej", g("ovvv"), t1)
                 - 0.5 * _ein("mnej,nb->mbej", g("oovo"), t1)
                 - 0.5 * _ein("mnef,jnfb->mbej", g("oovv"), tt))
        wabei = (g("vvvo") + _ein("abef,if->abei", g("vvvv"), t1)
                 + _ein("maei,mb->abei", zmbej, t1)
                 - _ein("mbei,ma->abei", zmbej, t1))
        return r + 0.5 * _ein("efam,imef->ia", wabei, l2)

    def L2eq_rhs_CC2(self, t1, t2, l1, l2, F):
        g = self.G
        fvv = self.Fb(F, "vv")
        foo = self.Fb(F, "oo")
        wmina = self.LWmina(t1)
        weifa = self.LWfiea(t1)
        fme = self.Fme(t1, t2, F)
        r = g("oovv") + _ein("ijab,eb->ijab", l2, fvv) - _ein("ijab,eb->ijba", l2, fvv)
        r = r - _ein("imab,jm->ijab", l2, foo) + _ein("imab,jm->jiab", l2, foo)
        r = r - _ein("ijmb,ma->ijab", wmina, l1) + _ein("ijmb,ma->ijba", wmina, l1)
        r = r + _ein("ejab,ie->ijab", weifa, l1) - _ein("ejab,ie->jiab", weifa, l1)
        x = _ein("ia,jb->ijab", l1, fme)
        return r + _pijab(x)

    # -- density and dipole (CCSD_Helper.py:984-1006, 1066-1092) ---------
    def Dij(self, t1, t2, l1, l2):
        return -(_ein("je,ie->ij", l1, t1) + 0.5 * _ein("jmea,imea->ij", l2, t2))

    def Dab(self, t1, t2, l1, l2):
        return _ein("nb,na->ab", l1, t1) + 0.5 * _ein("mneb,mnea->ab", l2, t2)

    def Dai(self, t1, t2, l1, l2):
        return (t1.T
                + _ein("me,miea->ai", l1, t2)
                - _ein("me,ma,ie->ai", l1, t1, t1)
                - 0.5 * _ein("mnef,mnaf,ie->ai", l2, t2, t1)
                - 0.5 * _ein("mnef,inef,ma->ai", l2, t2, t1))

    def density(self, t1, t2, l1, l2):
        """Correlated 1-RDM [[Dij, l1], [Dai, Dab]] (CCSD_Helper.py:1075-1077)."""
        top = np.concatenate([self.Dij(t1, t2, l1, l2), l1], axis=1)
        bot = np.concatenate([self.Dai(t1, t2, l1, l2), self.Dab(t1, t2, l1, l2)], axis=1)
        return np.concatenate([top, bot], axis=0)

    def dipole_moment(self, t1, t2, l1, l2, F=None):
        """[sum_pq mu^x_pq rho_pq, ...] over the dipole components given
        (CCSD_Helper.py:1066-1092; the discarded HF density is not built)."""
        rho = self.density(t1, t2, l1, l2)
        return [_ein("ij,ij->", m, rho) for m in self.mu]

    # -- block-frozen RK4 (CCSD_Helper.py:1158-1187, CC2_Helper.py:412-433)
    def _rk4(self, f, y, t, dt, Vt):
        k1 = f(y, Vt(t))
        k2 = f(y + dt / 2.0 * k1, Vt(t + dt / 2.0))
        k3 = f(y + dt / 2.0 * k2, Vt(t + dt / 2.0))
        k4 = f(y + dt * k3, Vt(t + dt))
        return dt / 6.0 * (k1 + 2.0 * k2 + 2.0 * k3 + k4)

    def ft1(self, t, dt, t1, t2, F, Vt):
        return self._rk4(lambda y, V: self.T1eq_rhs(y, t2, F + V), t1, t, dt, Vt)

    def ft2(self, t, dt, t1, t2, F, Vt):
        return self._rk4(lambda y, V: self.T2eq_rhs(t1, y, F + V), t2, t, dt, Vt)

    def fL1(self, t, dt, t1, t2, l1, l2, F, Vt):
        return self._rk4(lambda y, V: self.lam_1eq_rhs(t1, t2, y, l2, F + V), l1, t, dt, Vt)

    def fL2(self, t, dt, t1, t2, l1, l2, F, Vt):
        return self._rk4(lambda y, V: self.lam2eq_rhs(t1, t2, l1, y, F + V), l2, t, dt, Vt)

    def ft2_CC2(self, t, dt, t1, t2, F, Vt):
        return self._rk4(lambda y, V: self.T2eq_rhs_CC2(t1, y, F + V), t2, t, dt, Vt)

    def fL1_CC2(self, t, dt, t1, t2, l1, l2, F, Vt):
        return self._rk4(lambda y, V: self.L1eq_rhs_CC2(t1, t2, y, l2, F + V), l1, t, dt, Vt)

    def fL2_CC2(self, t, dt, t1, t2, l1, l2, F, Vt):
        return self._rk4(lambda y, V: self.L2eq_rhs_CC2(t1, t2, l1, y, F + V), l2, t, dt, Vt)

    def rk4_step(self, method, t, dt, state, F, Vt, precs):
        """One step of the propagation loop body (CCSD_Helper.py:1207-1233;
        CC2_Helper.py:453-472).  ``t`` is the already advanced time (the
        reference does ``t += dt`` before the stages).  Returns the new state
        ``round(old, precs) + delta`` with delta from the unrounded state."""
        t1, t2, l1, l2 = state
        r = [np.around(x, decimals=precs) for x in (t1, t2, l1, l2)]
        d1 = -1j * self.ft1(t, dt, t1, t2, F, Vt)
        if method == "CCSD":
            d2 = -1j * self.ft2(t, dt, t1, t2, F, Vt)
            e1 = 1j * self.fL1(t, dt, t1, t2, l1, l2, F, Vt)
            e2 = 1j * self.fL2(t, dt, t1, t2, l1, l2, F, Vt)
        elif method == "CC2":
            d2 = -1j * self.ft2_CC2(t, dt, t1, t2, F, Vt)
            e1 = 1j * self.fL1_CC2(t, dt, t1, t2, l1, l2, F, Vt)
            e2 = 1j * self.fL2_CC2(t, dt, t1, t2, l1, l2, F, Vt)
        else:
            raise ValueError(method)
        return (r[0] + d1, r[1] + d2, r[2] + e1, r[3] + e2)

    def propagate(self, method, F, state, t0, dt, nsteps, Vt, precs=15):
        """Runs ``nsteps`` of the reference loop (CCSD_Helper.py:1206-1240)
        and returns (times, mu_z list including the initial point, state)."""
        t = t0
        mus = [self.dipole_moment(*state)[-1]]
        times = [t]
        for _ in range(nsteps):
            t += dt
            state = self.rk4_step(method, t, dt, state, F, Vt, precs)
            mus.append(self.dipole_moment(*state)[-1])
            times.append(t)
        return np.array(times), np.array(mus), state

    # -- ground state DIIS (CCSD_Helper.py:347-416, 702-776;
    #    CC2_Helper.py:179-248, 324-400) ---------------------------------
    def _diis(self, update, energy, x1, x2, maxsize, maxiter, e_min, early_l1_store=False):
        """Shared DIIS driver with the reference's storage pattern.

        ``update(x1, x2) -> (x1', x2')`` is one Jacobi sweep; ``energy``
        returns the scalar monitored for the stop test.  ``early_l1_store``
        reproduces the CC2 Lambda quirk (CC2_Helper.py:382): the first block
        is appended to its store *before* the sweep."""
        x1, x2 = update(x1, x2)
        s1, s2 = [x1.copy()], [x2.copy()]
        e1, e2 = [], []
        for k in range(1, maxsize + 1):
            x1, x2 = update(x1, x2)
            s1.append(x1.copy())
            s2.append(x2.copy())
            e1.append(s1[k] - s1[k - 1])
            e2.append(s2[k] - s2[k - 1])
        B = -np.ones((maxsize + 1, maxsize + 1))
        B[-1, -1] = 0.0
        E = None
        niter = 0
        for _z in range(1, maxiter):
            e_old = energy(x1, x2)
            for a in range(maxsize):
                for b in range(maxsize):
                    B[a, b] = (_ein("ia,ia->", e1[b], e1[a]) + _ein("ijab,ijab->", e2[b], e2[a])).real
            rhs = np.zeros(maxsize + 1)
            rhs[-1] = -1.0
            c = np.linalg.solve(B, rhs)
            x1 = 0.0 * x1
            x2 = 0.0 * x2
            for a in range(maxsize):
                x1 = x1 + c[a] * s1[a + 1]
                x2 = x2 + c[a] * s2[a + 1]
            old1, old2 = x1.copy(), x2.copy()
            E = energy(x1, x2)
            niter += 1
            if abs(E - e_old) < e_min:
                break
            if early_l1_store:
                s1.append(x1.copy())
                x1, x2 = update(x1, x2)
                s2.append(x2.copy())
            else:
                x1, x2 = update(x1, x2)
                s1.append(x1.copy())
                s2.append(x2.copy())
            e1.append(x1 - old1)
            e2.append(x2 - old2)
            del s1[0], s2[0], e1[0], e2[0]
        return E, x1, x2, niter

    def DIIS_solver(self, t1, t2, F, maxsize=7, maxiter=40, E_min=1e-15, method="CCSD"):
        r2 = self.T2eq_rhs if method == "CCSD" else self.T2eq_rhs_CC2

        def upd(a, b):
            return (self.corrected_T1(a, self.T1eq_rhs(a, b, F), F),
                    self.corrected_T2(b, r2(a, b, F), F))

        E, t1, t2, _ = self._diis(upd, lambda a, b: self.CCSD_Corr_E(a, b, F), t1, t2,
                                  maxsize, maxiter, E_min)
        return E, t1, t2

    def DIIS_solver_Lam(self, t1, t2, l1, l2, F, maxsize=7, maxiter=30, E_min=1e-15, method="CCSD"):
        if method == "CCSD":
            r1, r2 = self.lam_1eq_rhs, self.lam2eq_rhs
        else:
            r1, r2 = self.L1eq_rhs_CC2, self.L2eq_rhs_CC2

        def upd(a, b):
            return (self.corrected_lam1(a, r1(t1, t2, a, b, F), F),
                    self.corrected_lam2(b, r2(t1, t2, a, b, F), F))

        def pseudo(a, b):
            e1, e2 = self.CCSD_pseudo_E(t1, t2, a, b, F)
            return e1 + e2

        E, l1, l2, _ = self._diis(upd, pseudo, l1, l2, maxsize, maxiter, E_min,
                                  early_l1_store=(method == "CC2"))
        return E, l1, l2


# -- fields ------------------------------------------------------------------

def reference_field(A, w0, mu_z):
    """Vt(t) = -A mu_z exp(i 2 pi w0 t) (CCSD_Helper.py:1197-1200)."""
    return lambda t: -A * mu_z * complex(math.cos(w0 * 2 * math.pi * t), math.sin(w0 * 2 * math.pi * t))


def sin_field(A, w0, mu_z):
    """V(t) = -E(t) mu_z with E(t) = A sin(w0 t) along z."""
    return lambda t: -(A * math.sin(w0 * t)) * mu_z


def time_steps(oracle, method, F, state, t0, dt, nsteps, Vt, precs=15):
    """Wall time of ``nsteps`` oracle RK4 steps (+ dipole), seconds/step."""
    t = t0
    s = state
    t_start = time.perf_counter()
    for _ in range(nsteps):
        t += dt
        s = oracle.rk4_step(method, t, dt, s, F, Vt, precs)
        oracle.dipole_moment(*s)
    return (time.perf_counter() - t_start) / nsteps
