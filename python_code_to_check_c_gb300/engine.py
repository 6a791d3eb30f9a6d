"""GPU engine: a tdcc_system on one CUDA device, driven through the C ABI.

``CCEngine`` owns the device copies of the integrals and the native handle.
Its methods carry the reference's names (``CCSD_Helper`` / ``CC2_Helper``)
so code written against the reference reads the same:

===========================  =================================================
reference (file:line)        here
===========================  =================================================
T1eq_rhs  CCSD_Helper.py:177 ``T1eq_rhs(t1, t2, F)``
T2eq_rhs  CCSD_Helper.py:268 ``T2eq_rhs(t1, t2, F)``
lam_1eq_rhs  :555            ``lam_1eq_rhs(t1, t2, l1, l2, F)``
lam2eq_rhs   :610            ``lam2eq_rhs(t1, t2, l1, l2, F)``
T2eq_rhs_CC2 CC2_Helper.py:12 ``T2eq_rhs_CC2(t1, t2, F)``
L1eq_rhs_CC2 CC2_Helper.py:50 ``L1eq_rhs_CC2(t1, t2, l1, l2, F)``
L2eq_rhs_CC2 CC2_Helper.py:128 ``L2eq_rhs_CC2(t1, t2, l1, l2, F)``
dipole_moment CCSD_Helper.py:1066 ``dipole_moment(t1, t2, l1, l2)``
loop body CCSD_Helper.py:1206 ``rk4_step(method, state, t_prev, dt, field, precs)``
===========================  =================================================

Arrays may be numpy or torch; results are torch complex128 CUDA tensors.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import TDCC_CC2, TDCC_CCSD, TDCC_L1, TDCC_L2, TDCC_T1, TDCC_T2, check


def _dev():
    if not torch.cuda.is_available():
        raise _lib.TdccError("no CUDA device: the TD-CC engine runs on the GPU only")
    return torch.device("cuda", torch.cuda.current_device())


def to_dev(x, dtype=torch.complex128):
    dev = _dev()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=dev).contiguous()


def tei_from_df_device(B) -> torch.Tensor:
    """<pq||rs> = sum_Q B[Q,p,r] B[Q,q,s] - B[Q,p,s] B[Q,q,r] on the device
    (``tdcc_tei_from_df``) from the (Q, n, n) density-fitting factors; the
    integral provider of the synthetic systems (the reference reads psi4's
    ``mo_spin_eri``, ``CCSD_Helper.py:57-93``)."""
    lib = _lib.load()
    Bd = to_dev(B, torch.float64)
    nq, n, n2 = (int(x) for x in Bd.shape)
    if n != n2:
        raise ValueError("B must be (Q, n, n)")
    tei = torch.empty((n, n, n, n), dtype=torch.float64, device=Bd.device)
    check(lib.tdcc_tei_from_df(_ptr(Bd), n, nq, _ptr(tei), _stream()), "tdcc_tei_from_df")
    return tei


def _ptr(x):
    return ctypes.c_void_p(x.data_ptr()) if x is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class CCEngine:
    """One synthetic (or psi4-provided) system resident on the GPU.

    ``nb > 1`` advances nb trajectories over the same integrals together:
    every per-trajectory array then carries a leading trajectory axis
    (t1: (nb, o, v), t2: (nb, o, o, v, v), F: (nb, n, n)), dipoles are
    (nb, n_mu) and propagated trajectories (nsteps, nb)."""

    def __init__(self, tei, fock, mu, o: int, nb: int = 1):
        self.lib = _lib.load()
        self.tei = to_dev(tei, torch.float64)
        self.fock = to_dev(fock, torch.float64)
        mus = [m for m in mu] if isinstance(mu, (list, tuple)) else [mu]
        self.mu = torch.stack([to_dev(m, torch.float64) for m in mus]).contiguous()
        self.n = int(self.fock.shape[0])
        self.o = int(o)
        self.v = self.n - self.o
        if tuple(self.tei.shape) != (self.n,) * 4:
            raise ValueError("tei must be (n,n,n,n)")
        self.nb = int(nb)
        self.n_mu = int(self.mu.shape[0])
        h = ctypes.c_void_p()
        check(self.lib.tdcc_system_create_batched(self.o, self.v, _ptr(self.tei), _ptr(self.fock),
                                                  _ptr(self.mu), self.n_mu, self.nb, ctypes.byref(h)),
              "tdcc_system_create_batched")
        self.handle = h
        self.precision = "fp64"

    @classmethod
    def from_system(cls, sysm, nb: int = 1, device_integrals: bool = True):
        """Density-fitted systems build <pq||rs> on the device
        (``tei_from_df_device``) unless ``device_integrals`` is False; the
        others (explicit integrals) upload them."""
        if device_integrals and getattr(sysm, "B", None) is not None:
            tei = tei_from_df_device(sysm.B)
        else:
            tei = sysm.tei()
        return cls(tei, sysm.fock, sysm.mu, sysm.o, nb=nb)

    def set_fields(self, fields, pol=None):
        """Per-trajectory fields (a list of nb ``make_field`` results) and the
        dipole component each couples to (default: the last); None clears."""
        if fields is None:
            check(self.lib.tdcc_set_fields(self.handle, None, None), "tdcc_set_fields")
            return
        if len(fields) != self.nb:
            raise ValueError(f"need {self.nb} fields")
        arr = (_lib.TdccField * self.nb)(*fields)
        parr = None
        if pol is not None:
            if len(pol) != self.nb:
                raise ValueError(f"need {self.nb} polarisations")
            parr = (ctypes.c_int * self.nb)(*[int(p) for p in pol])
        check(self.lib.tdcc_set_fields(self.handle, arr, parr), "tdcc_set_fields")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.tdcc_system_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- configuration ----
    def set_precision(self, mode: str = "fp64", slices: int = 5):
        m = {"fp64": _lib.TDCC_PREC_FP64, "mixed": _lib.TDCC_PREC_MIXED}[mode]
        check(self.lib.tdcc_set_precision(self.handle, m, int(slices)), "tdcc_set_precision")
        self.precision = mode

    def set_tc_policy(self, min_macs: int = 1 << 18, min_k: int = 32, min_mn: int = 1):
        """Which contractions the mixed mode sends to the tensor cores."""
        check(self.lib.tdcc_set_tc_policy(self.handle, int(min_macs), int(min_k), int(min_mn)),
              "tdcc_set_tc_policy")

    def set_simt_policy(self, max_k: int = 64, min_macs: int = 1 << 14):
        """Mixed mode: contractions left out by the tensor cores with K <= max_k
        run as slice products on the FP32 pipe (max_k = 0: FP64)."""
        check(self.lib.tdcc_set_simt_policy(self.handle, int(max_k), int(min_macs)), "tdcc_set_simt_policy")

    def set_memory_sharing(self, min_bytes: int = -1):
        """Workspace buffer sharing above min_bytes per program (-1: default
        1 GiB, 0: always)."""
        check(self.lib.tdcc_set_memory_sharing(self.handle, int(min_bytes)), "tdcc_set_memory_sharing")

    def set_adjoint_store(self, mode: int = -1):
        """Reverse mode keeps the forward intermediates (1), recomputes them
        (0), or keeps them when they fit in half the free memory (-1)."""
        check(self.lib.tdcc_set_adjoint_store(self.handle, int(mode)), "tdcc_set_adjoint_store")

    def autotune(self, method: str, state, reps: int = 3):
        """Picks the launch shape of every contraction by timing candidates
        on this system (``tdcc_autotune``); returns (ops changed, summed
        contraction ms before, after)."""
        st = [to_dev(x) for x in state]
        n = ctypes.c_int(0)
        b = ctypes.c_double(0.0)
        a = ctypes.c_double(0.0)
        check(self.lib.tdcc_autotune(self.handle, _lib.METHODS[method], *(_ptr(x) for x in st), int(reps),
                                     ctypes.byref(n), ctypes.byref(b), ctypes.byref(a), _stream()),
              "tdcc_autotune")
        return n.value, b.value, a.value

    def check_errors(self):
        """Synchronises and raises if a kernel recorded an error (an expired
        bounded wait in a tensor-core kernel)."""
        check(self.lib.tdcc_check_errors(self.handle), "tdcc_check_errors")

    def workspace_bytes(self) -> int:
        return int(self.lib.tdcc_workspace_bytes(self.handle))

    # ---- residuals ----
    def rhs(self, method: str, block: int, t1, t2, l1=None, l2=None, F=None):
        m = _lib.METHODS[method]
        t1 = to_dev(t1)
        t2 = to_dev(t2)
        l1 = to_dev(l1) if l1 is not None else None
        l2 = to_dev(l2) if l2 is not None else None
        if F is None:
            F = self.fock if self.nb == 1 else self.fock.expand(self.nb, self.n, self.n)
        F = to_dev(F)
        out = torch.empty_like(t1 if block in (TDCC_T1, TDCC_L1) else t2)
        check(self.lib.tdcc_rhs(self.handle, m, block, _ptr(t1), _ptr(t2), _ptr(l1), _ptr(l2),
                                _ptr(F), _ptr(out), _stream()), "tdcc_rhs")
        return out

    def T1eq_rhs(self, t1, t2, F):
        return self.rhs("CCSD", TDCC_T1, t1, t2, F=F)

    def T2eq_rhs(self, t1, t2, F):
        return self.rhs("CCSD", TDCC_T2, t1, t2, F=F)

    def lam_1eq_rhs(self, t1, t2, l1, l2, F):
        return self.rhs("CCSD", TDCC_L1, t1, t2, l1, l2, F)

    def lam2eq_rhs(self, t1, t2, l1, l2, F):
        return self.rhs("CCSD", TDCC_L2, t1, t2, l1, l2, F)

    def T2eq_rhs_CC2(self, t1, t2, F):
        return self.rhs("CC2", TDCC_T2, t1, t2, F=F)

    def L1eq_rhs_CC2(self, t1, t2, l1, l2, F):
        return self.rhs("CC2", TDCC_L1, t1, t2, l1, l2, F)

    def L2eq_rhs_CC2(self, t1, t2, l1, l2, F):
        return self.rhs("CC2", TDCC_L2, t1, t2, l1, l2, F)

    # ---- ground state (DIIS on the device) ----
    def _eps(self, F=None):
        F = self.fock.detach().cpu().numpy() if F is None else np.asarray(F)
        return np.ascontiguousarray(np.linalg.eigh(np.real(F))[0], dtype=np.float64)

    def ground_state(self, method: str, mode: int, t1, t2, l1=None, l2=None, maxsize=7, maxiter=40,
                     E_min=1e-15, r_tol=0.0, F=None):
        """Jacobi + DIIS on the device; returns (energy, niter, x1, x2) with
        (x1, x2) = (t1, t2) for mode 0 and (l1, l2) for mode 1."""
        t1 = to_dev(t1).clone()
        t2 = to_dev(t2).clone()
        l1 = to_dev(l1).clone() if l1 is not None else None
        l2 = to_dev(l2).clone() if l2 is not None else None
        eps = self._eps(F)
        e = ctypes.c_double(0.0)
        it = ctypes.c_int(0)
        check(self.lib.tdcc_ground_state(self.handle, _lib.METHODS[method], int(mode), _ptr(t1), _ptr(t2),
                                         _ptr(l1), _ptr(l2), eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                         int(maxsize), int(maxiter), float(E_min), float(r_tol),
                                         ctypes.byref(e), ctypes.byref(it), _stream()),
              "tdcc_ground_state")
        return (e.value, it.value) + ((t1, t2) if mode == 0 else (l1, l2))

    def DIIS_solver(self, t1, t2, F=None, maxsize=7, maxiter=40, E_min=1e-15, method="CCSD"):
        """CCSD_Helper.DIIS_solver (CCSD_Helper.py:347) / DIIS_solver_CC2: returns (E, t1, t2)."""
        E, _, t1, t2 = self.ground_state(method, 0, t1, t2, maxsize=maxsize, maxiter=maxiter, E_min=E_min, F=F)
        return E, t1, t2

    def DIIS_solver_Lam(self, t1, t2, l1, l2, F=None, maxsize=7, maxiter=30, E_min=1e-15, method="CCSD"):
        """CCSD_Helper.DIIS_solver_Lam (CCSD_Helper.py:702) / DIIS_solver_Lam_CC2: (E, l1, l2)."""
        E, _, l1, l2 = self.ground_state(method, 1, t1, t2, l1, l2, maxsize=maxsize, maxiter=maxiter,
                                         E_min=E_min, F=F)
        return E, l1, l2

    # ---- density / dipole ----
    def dipole_moment(self, t1, t2, l1, l2, F=None):
        t1, t2, l1, l2 = (to_dev(x) for x in (t1, t2, l1, l2))
        out = torch.empty(self.nb * self.n_mu, dtype=torch.complex128, device=t1.device)
        check(self.lib.tdcc_dipole(self.handle, _ptr(t1), _ptr(t2), _ptr(l1), _ptr(l2), _ptr(out),
                                   _stream()), "tdcc_dipole")
        return out if self.nb == 1 else out.view(self.nb, self.n_mu)

    # ---- propagation ----
    def rk4_step(self, method: str, state, t_prev: float, dt: float, field, precs: int = 15,
                 with_mu: bool = True):
        """One reference loop-body step; returns (new_state, mu or None)."""
        t1, t2, l1, l2 = (to_dev(x) for x in state)
        outs = [torch.empty_like(x) for x in (t1, t2, l1, l2)]
        mu = torch.empty(self.nb * self.n_mu, dtype=torch.complex128, device=t1.device) if with_mu else None
        check(self.lib.tdcc_rk4_step(self.handle, _lib.METHODS[method], _ptr(t1), _ptr(t2), _ptr(l1),
                                     _ptr(l2), *(_ptr(x) for x in outs), float(t_prev), float(dt),
                                     int(precs), ctypes.byref(field) if field is not None else None,
                                     _ptr(mu), _stream()),
              "tdcc_rk4_step")
        if mu is not None and self.nb > 1:
            mu = mu.view(self.nb, self.n_mu)
        return tuple(outs), mu

    def propagate(self, method: str, state, t0: float, dt: float, nsteps: int, field, precs: int = 15):
        """nsteps device-resident steps (captured CUDA graph); returns
        (final_state, mu_z trajectory as a complex128 CUDA tensor: (nsteps,),
        or (nsteps, nb) for a batched engine).  field None: the fields of
        ``set_fields``."""
        st = [to_dev(x).clone() for x in state]
        # a stable trajectory buffer: the captured step graphs record its address
        need = max(int(nsteps), 1) * self.nb
        buf = getattr(self, "_traj_buf", None)
        if buf is None or buf.numel() < need or buf.device != st[0].device:
            buf = torch.empty(max(need, 1024 * self.nb), dtype=torch.complex128, device=st[0].device)
            self._traj_buf = buf
        traj = buf
        check(self.lib.tdcc_propagate(self.handle, _lib.METHODS[method], *(_ptr(x) for x in st),
                                      float(t0), float(dt), int(nsteps), int(precs),
                                      ctypes.byref(field) if field is not None else None, _ptr(traj),
                                      _stream()),
              "tdcc_propagate")
        traj = traj[: int(nsteps) * self.nb].clone()
        return tuple(st), (traj if self.nb == 1 else traj.view(int(nsteps), self.nb))

    def block_times(self, method: str, state, t_prev: float, dt: float, field, precs: int = 15):
        """Device milliseconds of the four RK4 blocks (T1, T2, L1, L2: the
        reference's ft1/ft2/fL1/fL2) in one step from ``state``, each block
        run alone (one serial, eager step timed per kernel by CUDA events;
        the state is not advanced)."""
        ms = [0.0] * 4
        for r in profile_step(self, method, state, t_prev, dt, field, precs):
            if 0 <= r["block"] < 4:
                ms[r["block"]] += r["ms"]
        return ms


def adjoint(eng: "CCEngine", method: str, state, t0: float, dt: float, nsteps: int, weights, field=None,
            precs: int = -1, checkpoint: int = 50, want_state_grad: bool = False):
    """Reverse mode through ``nsteps`` propagation steps (``tdcc_adjoint``).

    J_b = sum_n weights[n] Re mu_b(t_n).  Returns (J: (nb,), gE: complex
    (nsteps, 4, nb) -- dJ/dE at the four RK4 stage times of each step --,
    dJ/d(initial state) conjugated, or None)."""
    st = [to_dev(x).contiguous() for x in state]
    w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64))
    if w.shape != (int(nsteps),):
        raise ValueError("weights must have one entry per step")
    J = np.zeros(eng.nb)
    gE = np.zeros((int(nsteps), 4, eng.nb), dtype=np.complex128)
    ast = [torch.empty_like(x) for x in st] if want_state_grad else [None] * 4
    dp = ctypes.POINTER(ctypes.c_double)
    check(eng.lib.tdcc_adjoint(eng.handle, _lib.METHODS[method], *(_ptr(x) for x in st), float(t0), float(dt),
                               int(nsteps), int(precs), ctypes.byref(field) if field is not None else None,
                               w.ctypes.data_as(dp), int(checkpoint), J.ctypes.data_as(dp),
                               gE.ctypes.data_as(dp), *(_ptr(x) for x in ast), _stream()),
          "tdcc_adjoint")
    return J, gE, (tuple(ast) if want_state_grad else None)


def profile_step(eng: "CCEngine", method: str, state, t_prev: float, dt: float, field, precs: int = 15):
    """Per-kernel CUDA-event timings of one serial, eager RK4 step.  Returns a
    list of dicts (tag, kind, block, stage, backend, flops, bytes, ms)."""
    t1, t2, l1, l2 = (to_dev(x) for x in state)
    cap = 8192
    recs = (_lib.TdccOpRecord * cap)()
    n = ctypes.c_int(0)
    torch.cuda.synchronize()
    check(eng.lib.tdcc_profile_step(eng.handle, _lib.METHODS[method], _ptr(t1), _ptr(t2), _ptr(l1),
                                    _ptr(l2), float(t_prev), float(dt), int(precs), ctypes.byref(field),
                                    recs, cap, ctypes.byref(n)), "tdcc_profile_step")
    out = []
    for k in range(min(n.value, cap)):
        r = recs[k]
        out.append(dict(tag=r.tag.decode(), kind=r.kind, block=r.block, stage=r.stage,
                        backend=r.backend, flops=r.flops, bytes=r.bytes, ms=r.ms))
    return out


def launch_count() -> int:
    return int(_lib.load().tdcc_launch_count())


__all__ = ["CCEngine", "adjoint", "launch_count", "TDCC_CCSD", "TDCC_CC2", "TDCC_T1", "TDCC_T2", "TDCC_L1", "TDCC_L2"]
