"""Dipole spectrum of a propagated trajectory (the reference's post-processing,
``Plots.py:20-25``): the discrete Fourier transforms of Re mu(t) and Im mu(t),
each fftshift-ed, on the energy axis (k / (N dt)) 2 pi 27.211 eV for the
shifted frequency indices k = -N/2 ... (``Plots.py`` builds that axis with
``range(-N/2, N/2)``, which matches fftshift for even N; for odd N the axis
here follows fftshift, k = -(N-1)/2 ... (N-1)/2).  The transforms run on the
device (``tdcc_spectrum``); plotting is left out."""
from __future__ import annotations

import csv
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check
from .engine import _ptr, _stream, to_dev


def spectrum(mu, dt: float):
    """mu: the dipole trajectory, complex, one entry per step (a device
    tensor, possibly strided, or anything numpy accepts).  Returns
    (energy_eV, Yr, Yi) as numpy arrays: the shifted transforms of Re mu and
    Im mu."""
    lib = _lib.load()
    if not torch.is_tensor(mu) or mu.device.type != "cuda" or mu.dtype != torch.complex128:
        mu = to_dev(mu)
    if mu.dim() != 1:
        raise ValueError("mu must be one-dimensional (one entry per step)")
    n = int(mu.shape[0])
    Yr = torch.empty(n, dtype=torch.complex128, device=mu.device)
    Yi = torch.empty_like(Yr)
    e = np.zeros(n)
    check(lib.tdcc_spectrum(_ptr(mu), n, int(mu.stride(0)), float(dt), _ptr(Yr), _ptr(Yi),
                            e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _stream()), "tdcc_spectrum")
    return e, Yr.cpu().numpy(), Yi.cpu().numpy()


def read_trajectory(path: str = "H2O.csv"):
    """(time, mu) from the trajectory table the propagation writes
    (columns time, mu_real, mu_imag after the index column)."""
    t, mr, mi = [], [], []
    with open(path, newline="") as f:
        rows = csv.reader(f)
        head = next(rows)
        c = {name: k for k, name in enumerate(head)}
        for r in rows:
            t.append(float(r[c["time"]]))
            mr.append(float(r[c["mu_real"]]))
            mi.append(float(r[c["mu_imag"]]))
    return np.array(t), np.array(mr) + 1j * np.array(mi)


def spectrum_from_csv(path: str = "H2O.csv"):
    """The spectrum of a trajectory table: dt = time[1] - time[0], as the
    reference takes it."""
    t, mu = read_trajectory(path)
    if len(t) < 2:
        raise ValueError("need at least two time points")
    return spectrum(mu, float(t[1] - t[0]))
