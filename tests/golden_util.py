"""Loads the golden fixtures and rebuilds their systems (shared by tests)."""
import os

import numpy as np

from python_code_to_check_c_gb300.system import synthetic_system

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["golden_o4_v8.npz", "golden_o6_v10.npz", "golden_o3_v5.npz"]


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, name)))
    sysm = synthetic_system(int(d["o"]), int(d["v"]), int(d["nq"]), int(d["seed"]))
    return d, sysm


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)
