"""tdcc_dipole_noalloc: the dipole without device allocation.

Some callers cannot call cudaMalloc (code running inside another library's
stream capture, plugins whose host framework owns all device memory).  For
them the library computes the dipole with its intermediates in a static
device array.  This checks, through the C ABI, that it returns what the
allocating entry point tdcc_dipole returns, on two calls in a row (the second
sees the first call's leftovers in the shared array), and that sizes above
the array's limit are refused.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from golden_util import load

pytestmark = pytest.mark.gpu

TOL = 1e-14  # absolute, a.u.; the tolerance of the other dipole parity tests


def _call(lib, o, v, st, mu, n_mu, out, stream):
    return lib.tdcc_dipole_noalloc(o, v, *(ctypes.c_void_p(x.data_ptr()) for x in st),
                                   ctypes.c_void_p(mu.data_ptr()), n_mu,
                                   ctypes.c_void_p(out.data_ptr()), stream)


@pytest.mark.parametrize("name", ["golden_o6_v10.npz", "golden_o4_v8.npz"])
def test_noalloc_dipole_matches_allocating_entry(name):
    import torch

    from python_code_to_check_c_gb300 import _lib
    from python_code_to_check_c_gb300.engine import CCEngine

    d, sysm = load(name)
    o, v = sysm.o, sysm.v
    lib = _lib.load()
    eng = CCEngine.from_system(sysm)
    dev = torch.device("cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)
    states = [(d["t1"], d["t2"], d["l1"], d["l2"]),
              tuple(x * (1.0 + 0.3j) + 0.01 * rng.standard_normal(x.shape) for x in
                    (d["t1"], d["t2"], d["l1"], d["l2"]))]
    try:
        for st in states:  # two calls in a row
            dst = [torch.as_tensor(np.ascontiguousarray(x), dtype=torch.complex128, device=dev) for x in st]
            ref = eng.dipole_moment(*dst).cpu().numpy()
            out = torch.full((3,), float("nan"), dtype=torch.complex128, device=dev)
            rc = _call(lib, o, v, dst, eng.mu, 3, out, stream)
            assert rc == 0, _lib.last_error()
            got = out.cpu().numpy()
            assert np.abs(got - ref).max() < TOL
    finally:
        eng.close()


def test_noalloc_rejects_sizes_beyond_its_array():
    import torch

    from python_code_to_check_c_gb300 import _lib

    lib = _lib.load()
    x = torch.zeros(4, dtype=torch.complex128, device="cuda")
    mu = torch.zeros(4, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = _call(lib, 65, 10, [x, x, x, x], mu, 1, x, stream)
    assert rc == -6
    assert "o <= 64" in _lib.last_error()
    rc = _call(lib, 10, 257, [x, x, x, x], mu, 1, x, stream)
    assert rc == -6
