"""``CC_Calculator``: the reference's driver surface on the GPU engine.

Mirrors ``CC_Calculator.py`` (class at :28-267) and the propagation loop
``Runge_Kutta_solver`` / ``Runge_Kutta_solver_CC2`` (CCSD_Helper.py:1191-1256,
CC2_Helper.py:430-500):

* ``CC_Calculator(psi, w0=, A=, t0=, dt=, precs=)`` -- a missing keyword is
  ignored, as the reference's bare ``except`` does; ``tf`` is 10.1.
* ``TDCC(timeout, 'CCSD'|'CC2')`` -- MP2 guess, ground-state T by DIIS
  (7 vectors, 40 iterations, 1e-15), Lambda by DIIS starting from T
  (7, 30, 1e-15), then the propagation; any other method string prints the
  reference's usage message.
* ``TDCC_restart(timeout)`` -- reads ``Parameters.csv`` and the restart files,
  continues for 50 time units after the saved time (``t0 + dt`` is the new
  start), appending to ``H2O.csv`` / ``timing.csv``.
* ``test_MP2()`` -- the MP2 total energy.

The propagation runs on the device in chunks: ``n - 1`` steps through the
captured step graph, then the chunk's last step through ``tdcc_rk4_step`` so
that the state before it (the state the reference saves when it stops) is
still at hand.  The stop tests of the reference are applied per step: the
time limit (``elapsed > 0.9 * timeout * 60`` s, checked after each chunk) and
``|Re mu_z| > 100`` (the first such step inside a chunk is found in the
chunk's trajectory and the chunk is re-run up to the step before it).  On a
stop the rounded previous state, the trajectory and the parameters (time of
the last completed step) are written; reaching ``tf`` writes nothing, as in
the reference.

``timing.csv`` rows: ``total`` is the wall time of one step (chunk wall time
over its steps), and, as in the reference, the sum of the ``t1 t2 l1 l2``
columns.  The four blocks of a step run concurrently inside one graph and
have no separate wall times, so each step's time is split between the
columns in proportion to the blocks' own device times, measured once per
propagation by one serial step timed per kernel (``CCEngine.block_times``;
the reference times ft1/ft2/fL1/fL2 one after another,
CCSD_Helper.py:1215-1228).

Systems come from psi4 when a psi4 module is passed (``system_from_psi4``),
or from a ``System`` (e.g. ``synthetic_system``) or a workload name.
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from . import restart_io
from ._lib import make_field
from .engine import CCEngine
from .system import WORKLOADS, System, mp2_guess, synthetic_system, system_from_psi4

USAGE = ("Error in specifying whether it is a CCSD or CC2 calculation\n"
         "Correct format is:\nmol.TDCC(stop_time, CCSD)\nwhere CCSD='CCSD' or 'CC2'")


class CC_Calculator:
    """Drop-in for ``CC_Calculator.CC_Calculator`` (CC_Calculator.py:28-46)."""

    def __init__(self, psi=None, system=None, outdir=".", precision="fp64", slices=5, chunk=100,
                 verbose=True, **kwargs):
        if system is None and psi is not None and hasattr(psi, "core"):
            system = system_from_psi4(psi)
        if isinstance(system, str):
            system = synthetic_system(**WORKLOADS[system])
        if not isinstance(system, System):
            raise ValueError("CC_Calculator needs a psi4 module, a System or a workload name")
        self.psi = psi
        self.system = system
        self.outdir = outdir
        self.precision = precision
        self.slices = int(slices)
        self.chunk = max(int(chunk), 2)
        self.verbose = verbose
        self.ndocc = system.o // 2
        self._engines = {}
        self.tf = 10.1
        try:
            self.w0 = kwargs["w0"]
            self.A = kwargs["A"]
            self.t0 = kwargs["t0"]
            self.dt = kwargs["dt"]
            self.precs = kwargs["precs"]
        except KeyError:
            pass

    # -- helpers ---------------------------------------------------------
    def _log(self, *args):
        if self.verbose:
            print(*args)

    def _path(self, name):
        return os.path.join(self.outdir, name)

    def engine(self, F=None) -> CCEngine:
        """The device system for Fock matrix ``F`` (the system's own by
        default); one engine per distinct F is kept."""
        F = self.system.fock if F is None else np.asarray(np.real(F), dtype=np.float64)
        key = hash(F.tobytes())
        eng = self._engines.get(key)
        if eng is None:
            eng = CCEngine(self.system.tei(), F, self.system.mu, self.system.o)
            eng.set_precision(self.precision, self.slices)
            self._engines[key] = eng
        return eng

    def MP2_E(self):
        """(E_scf, E_scf + E_mp2, t2) as CCSD_Helper.MP2_E (CCSD_Helper.py:102-124)."""
        s = self.system
        eps = np.linalg.eigh(s.fock)[0]
        tei = s.tei()
        t2 = mp2_guess(tei, eps, s.o)
        e2 = 0.25 * float(np.sum(tei[: s.o, : s.o, s.o:, s.o:] * t2))
        return s.scf_energy, s.scf_energy + e2, t2

    def test_MP2(self):
        return self.MP2_E()[1]

    # -- drivers ---------------------------------------------------------
    def TDCC(self, timeout, CCSD_or_CC2):
        if CCSD_or_CC2 not in ("CCSD", "CC2"):
            print(USAGE)
            return None
        return self._tdcc(timeout, CCSD_or_CC2)

    def ground_state(self, method):
        """MP2 guess, then T and Lambda by DIIS (CC_Calculator.py:152-200,
        215-253).  Returns (E_corr, pseudo_E, t1, t2, l1, l2) as device tensors."""
        s = self.system
        eng = self.engine()
        scf, mp2, t2 = self.MP2_E()
        t1 = np.zeros((s.o, s.v))
        self._log("Escf=", scf)
        self._log("Emp2=", mp2 - scf)
        self._log("Etot=", mp2)
        E, t1, t2 = eng.DIIS_solver(t1, t2, maxsize=7, maxiter=40, E_min=1e-15, method=method)
        self._log(f"E_{method.lower()}_plugin=", E + scf)
        if self.psi is not None and hasattr(self.psi, "energy"):
            psienergy = self.psi.energy(method)
            self._log("difference between psi4 and plugin=", psienergy.real - (E + scf))
            self.psi.driver.p4util.compare_values(psienergy, E + scf, 10, "CCSD Energy")
        pseudo, l1, l2 = eng.DIIS_solver_Lam(t1, t2, t1, t2, maxsize=7, maxiter=30, E_min=1e-15,
                                             method=method)
        self._log("E_pseudo_plugin=", pseudo)
        return E, pseudo, t1, t2, l1, l2

    def _tdcc(self, timeout, method):
        E, pseudo, t1, t2, l1, l2 = self.ground_state(method)
        return self.Runge_Kutta_solver(self.system.fock, t1, t2, l1, l2, self.w0, self.A, self.t0, self.tf,
                                       self.dt, timeout, self.precs, method=method)

    def TDCC_restart(self, timeout):
        """CC_Calculator.TDCC_restart (CC_Calculator.py:70-147)."""
        p = restart_io.read_parameters(self._path("Parameters.csv"))
        w0, A, t0, dt = p["w0"], p["A"], p["t0"], p["dt"]
        tf = 50.0 + t0
        t0 = t0 + dt
        F, t1, t2, l1, l2 = restart_io.load_restart(self.outdir, p["i"], p["a"])
        return self.Runge_Kutta_solver(F, t1, t2, l1, l2, w0, A, t0, tf, dt, timeout, p["precs"],
                                       restart="restart", method=p["CCSD_or_CC2"])

    def Runge_Kutta_solver(self, F, t1, t2, lam1, lam2, w0, A, t0, tf, dt, timeout, precs, restart=None,
                           method="CCSD"):
        """The propagation loop (CCSD_Helper.py:1191-1256); returns a dict with
        the recorded times, mu_z values, steps taken and whether it stopped."""
        eng = self.engine(F)
        field = make_field("reference", A, w0)
        state = tuple(x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, dtype=np.complex128))
                      for x in (t1, t2, lam1, lam2))
        mua = eng.dipole_moment(*state).cpu().numpy()
        self._log("time \t\t mu_z_real \t\t mu_z_real")
        self._log(round(t0, 4), "\t", mua[-1].real, "\t", mua[-1].imag)
        limit = None if timeout is None else 0.9 * float(timeout) * 60.0
        bt = eng.block_times(method, state, t0, dt, field, precs)
        shares = [x / sum(bt) for x in bt] if sum(bt) > 0 else [0.25] * 4
        data, timing = [], []
        start = time.time()
        t = t0
        stopped = False
        while t < tf and not stopped:
            # times of this chunk, accumulated exactly as the reference loop does
            times = []
            tt = t
            while tt < tf and len(times) < self.chunk:
                tt += dt
                times.append(tt)
            n = len(times)
            c0 = time.time()
            if n > 1:
                prev, traj = eng.propagate(method, state, t, dt, n - 1, field, precs)
            else:
                prev, traj = state, None
            new, mu = eng.rk4_step(method, prev, times[-2] if n > 1 else t, dt, field, precs)
            mus = mu[-1:] if traj is None else torch.cat([traj, mu[-1:]])
            mus = mus.cpu().numpy()
            per_step = (time.time() - c0) / n
            hot = np.nonzero(np.abs(mus.real) > 100)[0]
            over = limit is not None and abs(time.time() - start) > limit
            if len(hot):
                k = int(hot[0])           # step k of the chunk is the stopping step
                if k == n - 1:
                    pass
                elif k == 0:
                    prev = state
                else:
                    prev, _ = eng.propagate(method, state, t, dt, k, field, precs)
                n, stopped = k + 1, True
            elif over:
                stopped = True
            for j in range(n):
                data.append((round(times[j], 4), float(mus[j].real), float(mus[j].imag)))
                timing.append((per_step, *(per_step * f for f in shares)))
                self._log(round(times[j], 4), "\t", mus[j].real, "\t", mus[j].imag)
            t = times[n - 1]
            if stopped:
                rounded = [np.around(x.cpu().numpy(), decimals=precs) for x in prev]
                restart_io.save_data(self.outdir, np.asarray(F), *rounded, data, timing, precs, restart)
                restart_io.write_parameters(self._path("Parameters.csv"), w0, A, t - dt, dt, precs,
                                            rounded[0].shape[0], rounded[0].shape[1], method)
            else:
                state = new
        total = time.time() - start
        steps = len(data)
        self._log("total time non-adapative step:", total)
        self._log("total steps:", steps)
        if steps:
            self._log("step-time:", total / steps)
        return {"times": np.array([d[0] for d in data]), "mu": np.array([d[1] + 1j * d[2] for d in data]),
                "steps": steps, "stopped": stopped, "state": state if not stopped else prev}


__all__ = ["CC_Calculator", "USAGE"]
