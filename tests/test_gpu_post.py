"""Device integral provider and spectrum against the oracle:
tdcc_tei_from_df (FP64 GEMM + antisymmetrisation) and tdcc_spectrum
(shifted DFTs of Re mu and Im mu, Plots.py:20-25)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("o,v,nq", [(3, 5, 11), (4, 8, 16), (10, 38, 144)])
def test_tei_from_df_device(o, v, nq):
    from oracle.post_oracle import tei_from_df
    from python_code_to_check_c_gb300.engine import tei_from_df_device
    from python_code_to_check_c_gb300.system import synthetic_system
    s = synthetic_system(o, v, nq, 5)
    g = tei_from_df_device(s.B).cpu().numpy()
    ref = tei_from_df(s.B) if o < 10 else s.tei()
    assert np.abs(g - ref).max() <= 1e-14 * np.abs(ref).max()
    assert np.abs(g + g.transpose(0, 1, 3, 2)).max() == 0.0


@pytest.mark.parametrize("N", [2, 7, 64, 2001])
def test_spectrum_device(N):
    import torch

    from oracle.post_oracle import spectrum as ref_spectrum
    from python_code_to_check_c_gb300.spectrum import spectrum
    rng = np.random.default_rng(N)
    mu = rng.standard_normal(N) * 1e-3 + 1j * rng.standard_normal(N) * 1e-5
    dt = 0.005
    t = np.arange(N) * dt
    e, Yr, Yi = spectrum(mu, dt)
    e0, Yr0, Yi0 = ref_spectrum(t, mu)
    np.testing.assert_allclose(e, e0, rtol=1e-15, atol=0)
    assert np.abs(Yr - Yr0).max() <= 1e-12 * np.abs(Yr0).max()
    assert np.abs(Yi - Yi0).max() <= 1e-12 * np.abs(Yi0).max()
    # a strided column of a (steps, trajectories) table
    tab = torch.as_tensor(np.stack([mu * (1 + z) for z in range(3)], axis=1), device="cuda")
    _, Yr2, Yi2 = spectrum(tab[:, 2], dt)
    assert np.abs(Yr2 - 3 * Yr0).max() <= 3e-12 * np.abs(Yr0).max()
    assert np.abs(Yi2 - 3 * Yi0).max() <= 3e-12 * np.abs(Yi0).max()


def test_spectrum_of_propagated_trajectory(tmp_path):
    """Through the calculator's trajectory table (H2O.csv) as the reference's
    post-processing reads it."""
    from golden_util import load
    from oracle.post_oracle import spectrum as ref_spectrum
    from python_code_to_check_c_gb300 import restart_io
    from python_code_to_check_c_gb300._lib import make_field
    from python_code_to_check_c_gb300.engine import CCEngine
    from python_code_to_check_c_gb300.spectrum import read_trajectory, spectrum_from_csv
    d, sysm = load("golden_o4_v8.npz")
    st = [d["gs_" + k] + 0j for k in ("t1", "t2", "l1", "l2")]
    eng = CCEngine.from_system(sysm)
    try:
        dt = 0.01
        _, traj = eng.propagate("CCSD", st, 0.0, dt, 300, make_field("sin", 0.01, 0.923))
        mu = traj.detach().cpu().numpy()
    finally:
        eng.close()
    rows = [(dt * (k + 1), m.real, m.imag) for k, m in enumerate(mu)]
    path = str(tmp_path / "H2O.csv")
    restart_io.write_table(path, ("time", "mu_real", "mu_imag"), rows, 0, False)
    t, m = read_trajectory(path)
    e, Yr, Yi = spectrum_from_csv(path)
    e0, Yr0, Yi0 = ref_spectrum(t, m)
    np.testing.assert_allclose(e, e0, rtol=1e-12, atol=0)
    assert np.abs(Yr - Yr0).max() <= 1e-12 * np.abs(Yr0).max()
    assert np.abs(Yi - Yi0).max() <= 1e-12 * np.abs(Yi0).max()
