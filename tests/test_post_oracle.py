"""Post-processing oracle, pinned on the CPU: the spectrum against the DFT
definition and the reference's energy axis (Plots.py:20-25); the
density-fitted integrals against the host provider and the antisymmetry of
<pq||rs>."""
import numpy as np
import pytest

from oracle.post_oracle import dft_shifted, spectrum, tei_from_df


@pytest.mark.parametrize("N", [2, 7, 8, 64, 125])
def test_spectrum_matches_definition(N):
    rng = np.random.default_rng(N)
    mu = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    dt = 0.05
    t = np.arange(N) * dt + 0.3
    e, Yr, Yi = spectrum(t, mu)
    np.testing.assert_allclose(Yr, dft_shifted(mu.real), rtol=0, atol=1e-12 * max(1, N))
    np.testing.assert_allclose(Yi, dft_shifted(mu.imag), rtol=0, atol=1e-12 * max(1, N))
    if N % 2 == 0:  # the reference's axis: range(-N/2, N/2) (integer N/2), dt = time[1] - time[0]
        h = t[1] - t[0]
        ref = np.array([x * 1.0 / (N * h) * (2 * np.pi) * 27.211 for x in range(-N // 2, N // 2)])
        np.testing.assert_array_equal(e, ref)


def test_tei_from_df_matches_host_provider():
    from python_code_to_check_c_gb300.system import synthetic_system, tei_from_df as host
    s = synthetic_system(3, 5, 11, 7)
    g = tei_from_df(s.B)
    h = host(s.B)
    assert np.abs(g - h).max() <= 1e-15 * np.abs(h).max()
    # <pq||rs> = -<pq||sr> = -<qp||rs>
    assert np.abs(g + g.transpose(0, 1, 3, 2)).max() == 0.0
    assert np.abs(g + g.transpose(1, 0, 2, 3)).max() <= 1e-15 * np.abs(g).max()


def test_trajectory_table_round_trip(tmp_path):
    """The spectrum reads the propagation's H2O.csv (index, time, mu_real,
    mu_imag) as the table writer produces it, values exactly."""
    from python_code_to_check_c_gb300 import restart_io
    from python_code_to_check_c_gb300.spectrum import read_trajectory
    rng = np.random.default_rng(3)
    t = np.arange(1, 11) * 0.005
    mu = rng.standard_normal(10) + 1j * rng.standard_normal(10)
    path = str(tmp_path / "H2O.csv")
    restart_io.write_table(path, ("time", "mu_real", "mu_imag"), [(a, b.real, b.imag) for a, b in zip(t, mu)], 0,
                           False)
    t2, mu2 = read_trajectory(path)
    np.testing.assert_array_equal(t2, t)
    np.testing.assert_array_equal(mu2, mu)
