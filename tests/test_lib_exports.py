"""The C-ABI library loads (no GPU needed) and exports every symbol that
include/tdcc.h declares, with the signatures the ctypes binding expects."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tdcc.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tdcc_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from python_code_to_check_c_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from python_code_to_check_c_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("tdcc_rhs", "tdcc_rk4_step", "tdcc_propagate", "tdcc_dipole", "tdcc_system_create"):
        assert s in syms


def test_every_declared_symbol_is_exported(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from python_code_to_check_c_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_version_and_error_path(lib):
    from python_code_to_check_c_gb300 import _lib
    assert lib.tdcc_version() >= 1
    h = ctypes.c_void_p()
    rc = lib.tdcc_system_create(0, 5, None, None, None, 1, ctypes.byref(h))
    assert rc == -1
    assert "o and v" in _lib.last_error()
    rc = lib.tdcc_rhs(None, 0, 0, None, None, None, None, None, None, None)
    assert rc == -1


def test_argument_checks_without_a_gpu(lib):
    """Bad arguments fail with TDCC_ERR_ARG and a message before any CUDA
    call: the policy setters, reverse-mode storage, integral build, spectrum."""
    from python_code_to_check_c_gb300 import _lib
    assert lib.tdcc_set_tc_policy(None, 0, 1, 1) == -1
    assert lib.tdcc_set_simt_policy(None, 64, 0) == -1
    assert lib.tdcc_set_adjoint_store(None, 1) == -1
    assert lib.tdcc_set_memory_sharing(None, 0) == -1
    assert lib.tdcc_tei_from_df(None, 4, 8, None, None) == -1
    assert "NULL" in _lib.last_error()
    dummy = ctypes.c_void_p(16)
    assert lib.tdcc_tei_from_df(dummy, 0, 8, dummy, None) == -1
    assert "sizes" in _lib.last_error()
    assert lib.tdcc_spectrum(None, 8, 1, 0.1, None, None, None, None) == -1
    assert lib.tdcc_spectrum(dummy, 0, 1, 0.1, dummy, dummy, None, None) == -1
    assert lib.tdcc_spectrum(dummy, 8, 1, 0.0, dummy, dummy, None, None) == -1
    assert "dt" in _lib.last_error()
