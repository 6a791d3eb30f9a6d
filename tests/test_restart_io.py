"""Restart / output files in the reference's formats (CCSD_Helper.py:1102-1145,
CC_Calculator.py:70-135).  CPU only."""
import os

import numpy as np
import pytest

from python_code_to_check_c_gb300 import restart_io


def test_write_2data_lines(tmp_path):
    """One tab-separated line per element, value rounded to precs and printed
    as numpy prints a float (what csv.writer does with np.around's result)."""
    F = np.array([[0.5, -1.0 / 3.0], [2.0, 1e-20]])
    p = tmp_path / "x.dat"
    restart_io.write_2data(F, p, 15)
    lines = p.read_text().splitlines()
    assert lines == ["0\t0\t0.5", "0\t1\t-0.333333333333333", "1\t0\t2.0", "1\t1\t0.0"]


def test_write_4data_order_and_round_trip(tmp_path):
    rng = np.random.default_rng(7)
    X = rng.standard_normal((3, 3, 4, 4))
    p = tmp_path / "t2.dat"
    restart_io.write_4data(X, p, 15)
    lines = p.read_text().splitlines()
    assert len(lines) == X.size
    assert lines[0].split("\t")[:4] == ["0", "0", "0", "0"]
    assert lines[5].split("\t")[:4] == ["0", "0", "1", "1"]
    Y = restart_io.read_4data(p, 3, 4)
    assert np.array_equal(Y, np.around(X, 15))


def test_read_2data_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((5, 7))
    p = tmp_path / "t1.dat"
    restart_io.write_2data(X, p, 10)
    assert np.array_equal(restart_io.read_2data(p, 5, 7), np.around(X, 10))


def test_parameters_round_trip(tmp_path):
    p = tmp_path / "Parameters.csv"
    t = 0.1 + 0.2   # not representable in ten decimals
    restart_io.write_parameters(p, 0.923, 0.002, t, 0.005, 15, 10, 38, "CCSD")
    head = p.read_text().splitlines()[0]
    assert head == ",w0,A,t0,dt,precs,i,a,CCSD_or_CC2"
    d = restart_io.read_parameters(p)
    assert d == {"w0": 0.923, "A": 0.002, "t0": t, "dt": 0.005, "precs": 15, "i": 10, "a": 38,
                 "CCSD_or_CC2": "CCSD"}


def test_parameters_reader_accepts_fixed_point(tmp_path):
    p = tmp_path / "Parameters.csv"
    p.write_text(",w0,A,t0,dt,precs,i,a,CCSD_or_CC2\n1,0.9230000000,0.0020000000,0.3000000000,"
                 "0.0050000000,15,4,8,CC2\n")
    d = restart_io.read_parameters(p)
    assert d["t0"] == 0.3 and d["precs"] == 15 and d["CCSD_or_CC2"] == "CC2"


def test_tables_append_without_header(tmp_path):
    p = tmp_path / "H2O.csv"
    restart_io.write_table(p, ("time", "mu_real", "mu_imag"), [(0.01, 1.5, -2.0), (0.02, 1.25, 0.0)], 1, False)
    restart_io.write_table(p, ("time", "mu_real", "mu_imag"), [(0.03, 1.0, 0.5)], 1, True)
    assert p.read_text().splitlines() == [",time,mu_real,mu_imag", "1,0.01,1.5,-2.0", "2,0.02,1.25,0.0",
                                          "1,0.03,1.0,0.5"]


def test_save_and_load_restart(tmp_path):
    rng = np.random.default_rng(11)
    o, v = 2, 3
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    F = rng.standard_normal((o + v, o + v)) + 0.5j
    t1, t2, l1, l2 = c(o, v), c(o, o, v, v), c(o, v), c(o, o, v, v)
    restart_io.save_data(tmp_path, F, t1, t2, l1, l2, [(0.01, 1.0, 2.0)], [(0.1, 0.0, 0.0, 0.0, 0.0)], 15, None)
    names = sorted(x.name for x in tmp_path.iterdir())
    assert names == sorted(["H2O.csv", "timing.csv"] + [f"{n}_{p}.dat" for n in ("F", "t1", "t2", "lam1", "lam2")
                                                        for p in ("real", "imag")])
    F2, a1, a2, b1, b2 = restart_io.load_restart(tmp_path, o, v)
    assert np.array_equal(F2, np.around(F.real, 15))        # the imaginary part of F is dropped
    for x, y in ((a1, t1), (a2, t2), (b1, l1), (b2, l2)):
        assert np.array_equal(x, np.around(y.real, 15) + 1j * np.around(y.imag, 15))


# ---- pinned to the reference's own writers (fixture: tests/golden/make_restart_golden.py) ----
REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "restart_ref.npz")
NAMES = ("F", "t1", "t2", "lam1", "lam2")


@pytest.fixture(scope="module")
def ref():
    return dict(np.load(REF))


@pytest.mark.parametrize("precs", [15, 8])
def test_save_data_files_byte_identical_to_reference(tmp_path, ref, precs):
    """save_data writes the ten restart files exactly as the reference's
    write_2data / write_4data (CCSD_Helper.py:1107-1122) write a complex128
    state (the engine's precision)."""
    st = {n: ref[f"in_{n}"] for n in NAMES}
    restart_io.save_data(tmp_path, st["F"], st["t1"], st["t2"], st["lam1"], st["lam2"], [], [], precs, None)
    for n in NAMES:
        for part in ("real", "imag"):
            got = (tmp_path / f"{n}_{part}.dat").read_text()
            assert got == str(ref[f"f64_p{precs}_{n}_{part}"]), (n, part)


@pytest.mark.parametrize("kind", ["f64", "ld"])
@pytest.mark.parametrize("precs", [15, 8])
def test_readers_parse_reference_files(tmp_path, ref, kind, precs):
    """The readers give back the arrays the reference wrote: each value as the
    nearest float64 to its text (what the reference's convert_2data /
    convert_4data, CC_Calculator.py:85-113, read back), including files a
    fresh reference run writes from its extended-precision (longdouble)
    state; for a complex128 state that is np.around(x, precs) exactly."""
    o, v = ref["in_t1"].shape
    for n in NAMES:
        x = ref[f"in_{n}"]
        for part, arr in (("real", x.real), ("imag", x.imag)):
            p = tmp_path / f"{n}_{part}.dat"
            text = str(ref[f"{kind}_p{precs}_{n}_{part}"])
            p.write_text(text)
            got = restart_io.read_2data(p, *x.shape) if x.ndim == 2 else restart_io.read_4data(p, o, v)
            want = np.array([float(line.split("\t")[-1]) for line in text.splitlines()]).reshape(x.shape)
            assert np.array_equal(got, want), (n, part)
            if kind == "f64":
                assert np.array_equal(got, np.around(arr, precs)), (n, part)
            else:
                assert np.abs(got - np.around(arr, precs)).max() <= 10.0 ** -precs
