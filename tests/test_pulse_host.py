"""Host side of the pulse gradients (no GPU): the envelope field's partial
derivatives against central differences, and the step / stage times the
chain rule evaluates them at (accumulated t += dt, as the device does)."""
import numpy as np
import pytest

from python_code_to_check_c_gb300.pulse import Pulse, cosine_weights, stage_times, step_times


def test_partials_match_central_differences():
    rng = np.random.default_rng(5)
    p = Pulse(A=0.003, w0=0.923, c=rng.uniform(0.5, 1.5, 6), t_first=0.1, spacing=0.4, sigma=0.35)
    tau = np.linspace(0.0, 2.5, 41)
    E, dA, dw, dc = p.value_and_partials(tau)
    h = 1e-6

    def E_of(**kw):
        q = Pulse(**{**dict(A=p.A, w0=p.w0, c=p.c.copy(), t_first=p.t_first, spacing=p.spacing,
                            sigma=p.sigma), **kw})
        return q.value_and_partials(tau)[0]

    np.testing.assert_allclose(dA, (E_of(A=p.A + h) - E_of(A=p.A - h)) / (2 * h), rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(dw, (E_of(w0=p.w0 + h) - E_of(w0=p.w0 - h)) / (2 * h), rtol=1e-6, atol=1e-12)
    for k in range(len(p.c)):
        cp, cm = p.c.copy(), p.c.copy()
        cp[k] += h
        cm[k] -= h
        fd = (E_of(c=cp) - E_of(c=cm)) / (2 * h)
        np.testing.assert_allclose(dc[:, k], fd, rtol=1e-7, atol=1e-12)
    # E = A sin(w0 t) sum_k c_k phi_k(t)
    np.testing.assert_allclose(E, p.A * np.sin(p.w0 * tau) * (p.bumps(tau) @ p.c), rtol=1e-15, atol=0)


def test_times_accumulate_like_the_device():
    t = step_times(0.3, 0.01, 1000)
    ref = 0.3
    for n in range(1000):
        ref += 0.01
        assert t[n] == ref  # the same sequence of roundings, not 0.3 + (n + 1) * 0.01
    st = stage_times(0.3, 0.01, 5)
    assert st.shape == (5, 4)
    np.testing.assert_array_equal(st[:, 0], t[:5])
    np.testing.assert_array_equal(st[:, 1], st[:, 2])
    np.testing.assert_array_equal(st[:, 3], t[:5] + 0.01)
    w = cosine_weights(0.3, 0.01, 5, omega=0.8)
    np.testing.assert_array_equal(w, 0.01 * np.cos(0.8 * t[:5]))
