"""Pulse-shaped fields and gradients of dipole-response objectives.

A pulse is E(t) = A sin(w0 t) sum_k c_k phi_k(t) with Gaussian bumps
phi_k(t) = exp(-((t - t_k) / sigma)^2 / 2), t_k = t_first + k * spacing (the
device's ``TDCC_FIELD_ENVELOPE``).  The objective is
J = sum_n w_n Re mu(t_n) over the recorded dipole after every step; with
w_n = dt cos(omega t_n) it is the rectangle rule for the integral of
mu(t) cos(omega t).  ``pulse_gradient`` gets dJ/dE at every right-hand-side
evaluation from the device's reverse mode (``tdcc_adjoint``) and applies the
chain rule through E(t; A, w0, c) on the host.  ``PulseResponse`` wraps it as
a ``torch.autograd.Function``.

The reference propagates under a fixed field (``Vt``, CCSD_Helper.py:1197)
and has no gradients; this module has no counterpart there.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from ._lib import make_field
from .engine import adjoint


@dataclass
class Pulse:
    A: float
    w0: float
    c: np.ndarray = field(default_factory=lambda: np.ones(1))
    t_first: float = 0.0
    spacing: float = 1.0
    sigma: float = 1.0

    def field(self):
        return make_field("envelope", self.A, self.w0, env_c=list(np.asarray(self.c, dtype=np.float64)),
                          env_t0=self.t_first, env_dt=self.spacing, env_sigma=self.sigma)

    def bumps(self, tau):
        """phi_k(tau) for every k: shape tau.shape + (K,)."""
        k = np.arange(len(self.c))
        tk = self.t_first + k * self.spacing
        d = (tau[..., None] - tk) / self.sigma
        return np.exp(-0.5 * d * d)

    def value_and_partials(self, tau):
        """E(tau) and dE/dA, dE/dw0, dE/dc_k (the last with a trailing K axis)."""
        phi = self.bumps(tau)
        env = phi @ np.asarray(self.c, dtype=np.float64)
        s, co = np.sin(self.w0 * tau), np.cos(self.w0 * tau)
        E = self.A * s * env
        return E, s * env, self.A * tau * co * env, (self.A * s)[..., None] * phi


def step_times(t0: float, dt: float, nsteps: int) -> np.ndarray:
    """t_(n+1) after each step, accumulated as the device does (t += dt)."""
    out = np.empty(int(nsteps))
    t = float(t0)
    for n in range(int(nsteps)):
        t += dt
        out[n] = t
    return out


def stage_times(t0: float, dt: float, nsteps: int) -> np.ndarray:
    """(nsteps, 4): the times of the four RK4 stages of every step."""
    t = step_times(t0, dt, nsteps)
    h = dt / 2.0
    return np.stack([t, t + h, t + h, t + dt], axis=1)


def cosine_weights(t0: float, dt: float, nsteps: int, omega: float = 0.8) -> np.ndarray:
    """w_n = dt cos(omega t_n): J = sum w_n Re mu(t_n) ~ integral of mu cos(omega t)."""
    return dt * np.cos(omega * step_times(t0, dt, nsteps))


def pulse_gradient(eng, method, state, pulse: Pulse, t0, dt, nsteps, weights, checkpoint=50, precs=-1):
    """(J, dJ/dA, dJ/dw0, dJ/dc) for a single-trajectory engine."""
    if eng.nb != 1:
        raise ValueError("pulse_gradient drives one trajectory")
    J, gE, _ = adjoint(eng, method, state, t0, dt, nsteps, weights, field=pulse.field(), precs=precs,
                       checkpoint=checkpoint)
    tau = stage_times(t0, dt, nsteps)
    _, dA, dw, dc = pulse.value_and_partials(tau)
    g = gE[..., 0]
    return (float(J[0]), float(np.real(np.sum(g * dA))), float(np.real(np.sum(g * dw))),
            np.real(np.einsum("ns,nsk->k", g, dc)))


class PulseResponse(torch.autograd.Function):
    """J(A, w0, c) with its gradient from the device's reverse mode.

    ``PulseResponse.apply(A, w0, c, spec)`` with 0-d tensors A, w0, a 1-d
    tensor c and ``spec`` a dict: engine, method, state, t0, dt, nsteps,
    weights, t_first, spacing, sigma, checkpoint (optional)."""

    @staticmethod
    def forward(ctx, A, w0, c, spec):
        p = Pulse(float(A), float(w0), c.detach().cpu().numpy().astype(np.float64), spec["t_first"],
                  spec["spacing"], spec["sigma"])
        J, gA, gw, gc = pulse_gradient(spec["engine"], spec["method"], spec["state"], p, spec["t0"], spec["dt"],
                                       spec["nsteps"], spec["weights"], spec.get("checkpoint", 50))
        ctx.save_for_backward(torch.tensor(gA, dtype=torch.float64), torch.tensor(gw, dtype=torch.float64),
                              torch.as_tensor(gc, dtype=torch.float64))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gA, gw, gc = ctx.saved_tensors
        return gJ * gA, gJ * gw, gJ * gc, None


__all__ = ["Pulse", "PulseResponse", "cosine_weights", "pulse_gradient", "stage_times", "step_times"]
