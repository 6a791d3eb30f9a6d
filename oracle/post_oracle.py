"""CPU oracle for the post-processing around the propagation (TEST
INFRASTRUCTURE ONLY: imported by ``tests/`` alone, never by the product).

* ``spectrum``: the reference's dipole spectrum, ``Plots.py:20-25``:
  ``np.fft.fft`` of Re mu and of Im mu, each ``np.fft.fftshift``-ed, and the
  axis ``x / (N dt) * 2 pi * 27.211`` eV over ``range(-N/2, N/2)``.  The
  reference computes it with these same numpy calls (Plots.py also plots,
  which is left out), so the restatement is the reference's arithmetic.
  ``range(-N/2, N/2)`` is Python 2 integer division; for odd N it does not
  line up with fftshift, and the axis here follows fftshift
  (``-(N//2) ... (N-1)//2``), identical to the reference's for even N.
* ``tei_from_df``: ``<pq||rs> = (pr|qs) - (ps|qr)`` with
  ``(pr|qs) = sum_Q B[Q,p,r] B[Q,q,s]``, the synthetic integral model that
  stands in for psi4's ``mo_spin_eri`` (``CCSD_Helper.py:57-93``), written
  as an explicit loop over Q.
"""
from __future__ import annotations

import numpy as np


def spectrum(time, mu):
    """(energy_eV, Yr, Yi) of a trajectory: Plots.py:20-25."""
    time = np.asarray(time, dtype=np.float64)
    mu = np.asarray(mu, dtype=np.complex128)
    N = len(time)
    dt = time[1] - time[0]
    Yr = np.fft.fftshift(np.fft.fft(mu.real))
    Yi = np.fft.fftshift(np.fft.fft(mu.imag))
    k = np.arange(N) - N // 2
    return k * 1.0 / (N * dt) * (2 * np.pi) * 27.211, Yr, Yi


def dft_shifted(y):
    """The definition, for pinning: Y[j] = sum_n y[n] exp(-2 pi i k n / N),
    k = (j + N - N//2) mod N (fftshift order)."""
    y = np.asarray(y, dtype=np.complex128)
    N = len(y)
    n = np.arange(N)
    out = np.empty(N, dtype=np.complex128)
    for j in range(N):
        k = (j + N - N // 2) % N
        out[j] = np.sum(y * np.exp(-2j * np.pi * ((k * n) % N) / N))
    return out


def tei_from_df(B):
    B = np.asarray(B, dtype=np.float64)
    nq, n, _ = B.shape
    J = np.zeros((n, n, n, n))
    for q in range(nq):
        J += np.einsum("pr,qs->pqrs", B[q], B[q])
    return J - J.transpose(0, 1, 3, 2)
