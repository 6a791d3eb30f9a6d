"""ctypes binding of libtdcc.so (the C ABI declared in include/tdcc.h).

The library is built in-tree by ``python -m python_code_to_check_c_gb300.build``
(or ``__graft_entry__.build()``).  There is no fallback: if the library is
missing every GPU entry point raises ``TdccError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtdcc.so")

TDCC_CCSD, TDCC_CC2 = 0, 1
TDCC_T1, TDCC_T2, TDCC_L1, TDCC_L2 = 0, 1, 2, 3
TDCC_PREC_FP64, TDCC_PREC_MIXED = 0, 1
TDCC_FIELD_NONE, TDCC_FIELD_SIN, TDCC_FIELD_REFERENCE, TDCC_FIELD_ENVELOPE = 0, 1, 2, 3
TDCC_MAX_ENVELOPE = 64

METHODS = {"CCSD": TDCC_CCSD, "CC2": TDCC_CC2}

# every symbol include/tdcc.h declares, with (restype, argtypes)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_ll = ctypes.c_longlong


class TdccField(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("A", ctypes.c_double),
        ("w0", ctypes.c_double),
        ("n_env", ctypes.c_int),
        ("env_t0", ctypes.c_double),
        ("env_dt", ctypes.c_double),
        ("env_sigma", ctypes.c_double),
        ("env_c", ctypes.c_double * TDCC_MAX_ENVELOPE),
    ]


class TdccOpRecord(ctypes.Structure):
    _fields_ = [
        ("tag", ctypes.c_char * 96),
        ("kind", ctypes.c_int),
        ("block", ctypes.c_int),
        ("stage", ctypes.c_int),
        ("backend", ctypes.c_int),
        ("flops", ctypes.c_double),
        ("bytes", ctypes.c_double),
        ("ms", ctypes.c_double),
    ]


SIGNATURES = {
    "tdcc_version": (_i, []),
    "tdcc_last_error": (_i, [ctypes.c_char_p, ctypes.c_size_t]),
    "tdcc_launch_count": (_ll, []),
    "tdcc_system_create": (_i, [_i, _i, _vp, _vp, _vp, _i, ctypes.POINTER(_vp)]),
    "tdcc_system_destroy": (_i, [_vp]),
    "tdcc_system_create_batched": (_i, [_i, _i, _vp, _vp, _vp, _i, _i, ctypes.POINTER(_vp)]),
    "tdcc_system_batch": (_i, [_vp]),
    "tdcc_set_fields": (_i, [_vp, ctypes.POINTER(TdccField), ctypes.POINTER(_i)]),
    "tdcc_set_precision": (_i, [_vp, _i, _i]),
    "tdcc_workspace_bytes": (_ll, [_vp]),
    "tdcc_check_errors": (_i, [_vp]),
    "tdcc_set_tc_policy": (_i, [_vp, _ll, _i, _i]),
    "tdcc_set_simt_policy": (_i, [_vp, _i, _ll]),
    "tdcc_set_memory_sharing": (_i, [_vp, _ll]),
    "tdcc_set_adjoint_store": (_i, [_vp, _i]),
    "tdcc_tei_from_df": (_i, [_vp, _i, _i, _vp, _vp]),
    "tdcc_spectrum": (_i, [_vp, _ll, _ll, _d, _vp, _vp, _vp, _vp]),
    "tdcc_ground_state": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp, ctypes.POINTER(_d), _i, _i, _d, _d,
                               ctypes.POINTER(_d), ctypes.POINTER(_i), _vp]),
    "tdcc_rhs": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "tdcc_dipole": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "tdcc_rk4_step": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _i,
                           ctypes.POINTER(TdccField), _vp, _vp]),
    "tdcc_propagate": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _d, _i, _i,
                            ctypes.POINTER(TdccField), _vp, _vp]),
    "tdcc_autotune": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _i, ctypes.POINTER(_i), ctypes.POINTER(_d),
                           ctypes.POINTER(_d), _vp]),
    "tdcc_adjoint": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _d, _i, _i, ctypes.POINTER(TdccField),
                          ctypes.POINTER(_d), _i, ctypes.POINTER(_d), ctypes.POINTER(_d), _vp, _vp, _vp, _vp, _vp]),
    "tdcc_dipole_noalloc": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "tdcc_program_json": (_ll, [_i, _i, _i, _i, _i, _i, ctypes.c_char_p, ctypes.c_size_t]),
    "tdcc_adjoint_program_json": (_ll, [_i, _i, _i, _i, _i, _i, ctypes.c_char_p, ctypes.c_size_t]),
    "tdcc_profile_step": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _d, _i, ctypes.POINTER(TdccField),
                               ctypes.POINTER(TdccOpRecord), _i, ctypes.POINTER(_i)]),
}


class TdccError(RuntimeError):
    pass


_lock = threading.Lock()
_lib = None


def load(path: str = LIB_PATH):
    """Loads libtdcc.so once and declares its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise TdccError(f"{path} is not built; run `python -m python_code_to_check_c_gb300.build`")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(4096)
    load().tdcc_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise TdccError(f"{what} failed with code {rc}: {last_error()}")


def program_json(o: int, v: int, method: str, block: int, n_mu: int = 3, nb: int = 1) -> dict:
    """The op list libtdcc runs for (method, block) at sizes (o, v) and nb
    trajectories, as a dict (block 4 = density / dipole).  Works without a GPU."""
    import json
    lib = load()
    cap = 1 << 20
    while True:
        buf = ctypes.create_string_buffer(cap)
        n = lib.tdcc_program_json(o, v, METHODS[method], block, n_mu, nb, buf, cap)
        if n >= 0:
            return json.loads(buf.value.decode())
        if n != -6:
            raise TdccError(f"tdcc_program_json failed: {last_error()}")
        cap *= 4


def adjoint_program_json(o: int, v: int, method: str, block: int, n_mu: int = 3, nb: int = 1) -> dict:
    """The reverse-mode op list of (method, block): forward slots [0, nfwd),
    adjoint slots after them (adj_of[s] for forward slot s).  No GPU needed."""
    import json
    lib = load()
    cap = 1 << 21
    while True:
        buf = ctypes.create_string_buffer(cap)
        n = lib.tdcc_adjoint_program_json(o, v, METHODS[method], block, n_mu, nb, buf, cap)
        if n >= 0:
            return json.loads(buf.value.decode())
        if n != -6:
            raise TdccError(f"tdcc_adjoint_program_json failed: {last_error()}")
        cap *= 4


def make_field(kind: str = "sin", A: float = 0.0, w0: float = 0.0, env_c=(), env_t0: float = 0.0,
               env_dt: float = 1.0, env_sigma: float = 1.0) -> TdccField:
    kinds = {"none": TDCC_FIELD_NONE, "sin": TDCC_FIELD_SIN, "reference": TDCC_FIELD_REFERENCE,
             "envelope": TDCC_FIELD_ENVELOPE}
    f = TdccField()
    f.kind = kinds[kind]
    f.A = float(A)
    f.w0 = float(w0)
    env_c = list(env_c)
    if len(env_c) > TDCC_MAX_ENVELOPE:
        raise ValueError("too many envelope coefficients")
    f.n_env = len(env_c)
    f.env_t0, f.env_dt, f.env_sigma = float(env_t0), float(env_dt), float(env_sigma)
    for k, c in enumerate(env_c):
        f.env_c[k] = float(c)
    return f
