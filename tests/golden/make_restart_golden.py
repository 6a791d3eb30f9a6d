"""Writes the restart-file fixture by running the reference's own writers.

    python tests/golden/make_restart_golden.py /path/to/reference

Imports ``CCSD_Helper`` from the reference checkout (psi4 and pandas replaced
by empty stub modules: the writers use neither) and calls its ``write_2data``
and ``write_4data`` (CCSD_Helper.py:1107-1122) on the real and imaginary
parts of a seeded complex128 state -- F (n x n), t1 and lam1 (o x v), t2 and
lam2 (o x o x v x v) -- as ``Save_data`` (CCSD_Helper.py:1136-1145) does, for
two rounding precisions.  A fresh run of the reference propagates in numpy's
extended type (clongdouble on x86), so the same files are also written from
a longdouble copy of the state.  Output: ``restart_ref.npz`` with the inputs
and every file's text.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

NAMES = ("F", "t1", "t2", "lam1", "lam2")


def state(o=2, v=3, seed=2024):
    rng = np.random.default_rng(seed)

    def c(*shape):
        return rng.standard_normal(shape) / 3.0 + 1j * rng.standard_normal(shape) / 7.0

    F = np.diag(np.linspace(-1.2, 2.1, o + v)) + 0.01 * c(o + v, o + v)
    return {"F": F, "t1": c(o, v), "t2": 0.1 * c(o, o, v, v), "lam1": c(o, v), "lam2": 0.1 * c(o, o, v, v)}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_restart_golden.py <path of the reference checkout>")
    stub_dir = tempfile.mkdtemp(prefix="refstubs_")
    for name in ("psi4", "pandas"):
        with open(os.path.join(stub_dir, name + ".py"), "w") as f:
            f.write("# empty stub: the writers use neither module\n")
    sys.path.insert(0, stub_dir)
    sys.path.insert(1, sys.argv[1])
    sys.dont_write_bytecode = True
    import CCSD_Helper  # noqa: E402

    h = CCSD_Helper.CCSD_Helper.__new__(CCSD_Helper.CCSD_Helper)
    st = state()
    out = {f"in_{k}": v for k, v in st.items()}
    work = tempfile.mkdtemp(prefix="restart_ref_")
    cwd = os.getcwd()
    os.chdir(work)
    try:
        for kind, cast in (("f64", np.complex128), ("ld", np.clongdouble)):
            for precs in (15, 8):
                for name in NAMES:
                    x = st[name].astype(cast)
                    writer = h.write_2data if x.ndim == 2 else h.write_4data
                    for part, arr in (("real", x.real), ("imag", x.imag)):
                        fn = f"{name}_{part}.dat"
                        writer(arr, fn, precs)
                        with open(fn) as f:
                            out[f"{kind}_p{precs}_{name}_{part}"] = np.array(f.read())
    finally:
        os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, "restart_ref.npz"), **out)
    print("wrote", os.path.join(HERE, "restart_ref.npz"), len(out), "entries")


if __name__ == "__main__":
    main()
