"""Restart and output files in the reference's formats (no pandas).

* ``write_2data`` / ``write_4data`` (CCSD_Helper.py:1107-1122): one line per
  element, tab separated, ``i<TAB>a<TAB>value`` / ``i<TAB>j<TAB>a<TAB>b<TAB>value``,
  the value rounded with ``np.around(x, precs)`` and printed as numpy prints
  a float.
* ``read_2data`` / ``read_4data``: the readers of TDCC_restart
  (``convert_2data`` / ``convert_4data``, CC_Calculator.py:85-113).
* ``Parameters.csv`` (CCSD_Helper.py:1102-1105): header
  ``,w0,A,t0,dt,precs,i,a,CCSD_or_CC2``, one row with index 1.  The
  reference's row is a mixed-type (object) row, which pandas writes with
  ``str`` rather than its ``float_format``; floats are written here as their
  shortest round-trip text, so a restart resumes at exactly the saved time.
  The reader accepts either form.  ``t0`` holds the time of the last
  completed step.
* ``H2O.csv`` / ``timing.csv`` (CCSD_Helper.py:1124-1135): pandas-style CSV
  with an index column; a restarted run appends rows without a header.
"""
from __future__ import annotations

import csv
import os

import numpy as np


def _fmt(x) -> str:
    return str(np.float64(x))


def write_2data(F, filename, precs):
    F = np.asarray(F, dtype=np.float64)
    Fr = np.around(F, decimals=precs)
    ii, aa = np.indices(F.shape)
    with open(filename, "w") as f:
        for i, a, x in zip(ii.ravel(), aa.ravel(), Fr.ravel()):
            f.write(f"{i}\t{a}\t{_fmt(x)}\n")


def write_4data(F, filename, precs):
    F = np.asarray(F, dtype=np.float64)
    Fr = np.around(F, decimals=precs)
    idx = np.indices(F.shape).reshape(4, -1)
    with open(filename, "w") as f:
        for (i, j, a, b), x in zip(idx.T, Fr.ravel()):
            f.write(f"{i}\t{j}\t{a}\t{b}\t{_fmt(x)}\n")


def read_2data(filename, n0, n1):
    out = np.zeros((n0, n1))
    data = np.loadtxt(filename, delimiter="\t", ndmin=2)
    for row in data:
        out[int(np.around(row[0])), int(np.around(row[1]))] = row[2]
    return out


def read_4data(filename, i, a):
    out = np.zeros((i, i, a, a))
    data = np.loadtxt(filename, delimiter="\t", ndmin=2)
    idx = np.around(data[:, :4]).astype(int)
    out[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]] = data[:, 4]
    return out


PARAM_COLUMNS = ("w0", "A", "t0", "dt", "precs", "i", "a", "CCSD_or_CC2")


def write_parameters(path, w0, A, t, dt, precs, i, a, method):
    vals = [repr(float(w0)), repr(float(A)), repr(float(t)), repr(float(dt)),
            str(int(precs)), str(int(i)), str(int(a)), str(method)]
    with open(path, "w", newline="") as f:
        w = csv.writer(f, lineterminator="\n")
        w.writerow([""] + list(PARAM_COLUMNS))
        w.writerow(["1"] + vals)


def read_parameters(path):
    with open(path, newline="") as f:
        rows = list(csv.reader(f))
    head, row = rows[0], rows[1]
    d = dict(zip(head[1:], row[1:]))
    return {"w0": float(d["w0"]), "A": float(d["A"]), "t0": float(d["t0"]), "dt": float(d["dt"]),
            "precs": int(float(d["precs"])), "i": int(float(d["i"])), "a": int(float(d["a"])),
            "CCSD_or_CC2": d["CCSD_or_CC2"]}


def write_table(path, columns, rows, first_index, append):
    """pandas-style CSV: index column then the named columns."""
    mode = "a" if append else "w"
    with open(path, mode, newline="") as f:
        w = csv.writer(f, lineterminator="\n")
        if not append:
            w.writerow([""] + list(columns))
        for k, r in enumerate(rows):
            w.writerow([str(first_index + k)] + [repr(float(x)) for x in r])


def save_data(outdir, F, t1, t2, l1, l2, data_rows, timing_rows, precs, restart):
    """Save_data (CCSD_Helper.py:1124-1145): the trajectory tables and the ten
    restart files (real and imaginary parts of F, t1, t2, lam1, lam2)."""
    p = lambda name: os.path.join(outdir, name)  # noqa: E731
    append = restart is not None
    write_table(p("H2O.csv"), ("time", "mu_real", "mu_imag"), data_rows, 1, append)
    write_table(p("timing.csv"), ("total", "t1", "t2", "l1", "l2"), timing_rows, 1, append)
    F = np.asarray(F)
    for name, arr, writer in (("F", F, write_2data), ("t1", t1, write_2data), ("t2", t2, write_4data),
                              ("lam1", l1, write_2data), ("lam2", l2, write_4data)):
        arr = np.asarray(arr)
        writer(np.real(arr), p(f"{name}_real.dat"), precs)
        writer(np.imag(arr) if np.iscomplexobj(arr) else np.zeros_like(arr, dtype=np.float64),
               p(f"{name}_imag.dat"), precs)


def load_restart(outdir, i, a):
    """The amplitudes and Fock matrix TDCC_restart reads (CC_Calculator.py:115-135);
    like the reference, the imaginary part of F is dropped."""
    p = lambda name: os.path.join(outdir, name)  # noqa: E731
    t1 = read_2data(p("t1_real.dat"), i, a) + 1j * read_2data(p("t1_imag.dat"), i, a)
    l1 = read_2data(p("lam1_real.dat"), i, a) + 1j * read_2data(p("lam1_imag.dat"), i, a)
    t2 = read_4data(p("t2_real.dat"), i, a) + 1j * read_4data(p("t2_imag.dat"), i, a)
    l2 = read_4data(p("lam2_real.dat"), i, a) + 1j * read_4data(p("lam2_imag.dat"), i, a)
    F = read_2data(p("F_real.dat"), i + a, i + a)
    return F, t1, t2, l1, l2
