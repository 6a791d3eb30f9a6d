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


def _system_without_integrals(lib, o, v, mu, n_mu):
    """A tdcc_system for the dipole alone: the density program reads the
    amplitudes and the dipole integrals only, never <pq||rs> or F, so a
    one-element stand-in is passed for those (sizes where the n^4 integrals
    would not fit in memory)."""
    import torch
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    h = ctypes.c_void_p()
    rc = lib.tdcc_system_create_batched(o, v, ctypes.c_void_p(dummy.data_ptr()), ctypes.c_void_p(dummy.data_ptr()),
                                        ctypes.c_void_p(mu.data_ptr()), n_mu, 1, ctypes.byref(h))
    assert rc == 0
    return h, dummy


@pytest.mark.parametrize("o,v,n_mu", [(64, 8, 3), (4, 256, 3), (64, 256, 1), (5, 7, 1)])
def test_noalloc_dipole_at_its_size_limits(o, v, n_mu):
    """The largest systems the static array is sized for (o = 64, v = 256,
    and both at once: the density program's scratch 2o^2 + 3v^2 + ov at its
    maximum), and one dipole component (n_mu = 1), against tdcc_dipole."""
    import torch

    from python_code_to_check_c_gb300 import _lib

    lib = _lib.load()
    n = o + v
    g = torch.Generator(device="cuda").manual_seed(1000 * o + v)

    def amp(*shape):
        re = torch.randn(*shape, generator=g, device="cuda", dtype=torch.float64)
        im = torch.randn(*shape, generator=g, device="cuda", dtype=torch.float64)
        return (0.01 * torch.complex(re, im)).contiguous()

    st = [amp(o, v), amp(o, o, v, v), amp(o, v), amp(o, o, v, v)]
    mu = torch.randn(n_mu, n, n, generator=g, device="cuda", dtype=torch.float64)
    mu = (0.5 * (mu + mu.transpose(1, 2))).contiguous()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    h, dummy = _system_without_integrals(lib, o, v, mu, n_mu)
    try:
        ref = torch.full((n_mu,), float("nan"), dtype=torch.complex128, device="cuda")
        rc = lib.tdcc_dipole(h, *(ctypes.c_void_p(x.data_ptr()) for x in st), ctypes.c_void_p(ref.data_ptr()),
                             stream)
        assert rc == 0, _lib.last_error()
        for _ in range(2):  # two calls in a row
            out = torch.full((n_mu,), float("nan"), dtype=torch.complex128, device="cuda")
            rc = _call(lib, o, v, st, mu, n_mu, out, stream)
            assert rc == 0, _lib.last_error()
            r, got = ref.cpu().numpy(), out.cpu().numpy()
            assert np.isfinite(got).all()
            assert np.abs(got - r).max() <= TOL * max(1.0, np.abs(r).max()), (got, r)
    finally:
        lib.tdcc_system_destroy(h)


def test_noalloc_dipole_inside_a_captured_graph():
    """The use it exists for: called while the stream is being captured into
    a CUDA graph (where cudaMalloc is not allowed).  The first call, outside
    the capture, sets the device's array address up; the captured call is
    then replayed on new amplitudes and compared with tdcc_dipole."""
    import torch

    from python_code_to_check_c_gb300 import _lib
    from python_code_to_check_c_gb300.engine import CCEngine

    d, sysm = load("golden_o6_v10.npz")
    o, v = sysm.o, sysm.v
    lib = _lib.load()
    eng = CCEngine.from_system(sysm)
    dev = torch.device("cuda")
    st = [torch.as_tensor(np.ascontiguousarray(x), dtype=torch.complex128, device=dev)
          for x in (d["t1"], d["t2"], d["l1"], d["l2"])]
    out = torch.zeros(3, dtype=torch.complex128, device=dev)
    try:
        rc = _call(lib, o, v, st, eng.mu, 3, out, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            cap = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            rc = _call(lib, o, v, st, eng.mu, 3, out, cap)
        assert rc == 0, _lib.last_error()
        for scale in (1.0, 0.7 - 0.2j):
            for x, x0 in zip(st, (d["t1"], d["t2"], d["l1"], d["l2"])):
                x.copy_(torch.as_tensor(np.ascontiguousarray(x0 * scale), dtype=torch.complex128))
            out.fill_(float("nan"))
            graph.replay()
            torch.cuda.synchronize()
            ref = eng.dipole_moment(*st).cpu().numpy()
            assert np.abs(out.cpu().numpy() - ref).max() < TOL
    finally:
        eng.close()
