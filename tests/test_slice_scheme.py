"""The exact slice-product scheme of the mixed mode, modelled on the CPU with
the kernels' arithmetic (the kernels themselves are checked on the GPU):

* digits: x 2^-e is cut into S balanced digits from the bits of x
  (f = floor(|x| 2^(7S - e)), recoded from the least significant 7 bits up:
  a digit >= 64 becomes d - 128 with a carry), |q_1| <= 128, |q_s| <= 64;
* level sums: products q_s r_t with s + t = L summed in FP32 over a K chunk
  are exact integers when every partial sum stays within 2^24: 512-wide
  chunks (tensor cores, real levels) and K <= 64 (FP32 pipe, complex levels)
  always do, 1024-wide chunks did not in the worst case;
* recombination: sum_L V_L 2^(u - 7L) in int64, scaled by 2^(ea + eb - u),
  equals the product of the truncated operands up to the final rounding.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

S = 5


def row_exp(xs):
    m = max(abs(x) for x in xs)
    return math.frexp(m)[1] if m != 0 else 0  # m = f 2^e, f in [0.5, 1): |x| < 2^e


def digits(x, e, S=S):
    f = math.floor(abs(Fraction(x)) * Fraction(2) ** (7 * S - e))
    assert f < 2 ** (7 * S)
    q = [0] * S
    g = f
    for i in range(S - 1, 0, -1):  # least significant first, as the kernels do
        d = g & 127
        g >>= 7
        if d >= 64:
            d -= 128
            g += 1
        q[i] = d
    q[0] = g
    assert sum(v << (7 * (S - 1 - s)) for s, v in enumerate(q)) == f
    return [-v for v in q] if x < 0 else q


def truncated(x, e, S=S):
    return sum(Fraction(q) * Fraction(2) ** (e - 7 * (s + 1)) for s, q in enumerate(digits(x, e, S)))


def test_digit_ranges_and_truncation():
    rng = np.random.default_rng(1)
    for _ in range(200):
        row = rng.standard_normal(16) * 10.0 ** rng.integers(-8, 8)
        e = row_exp(row)
        for x in row:
            q = digits(x, e)
            assert abs(q[0]) <= 128 and all(abs(v) <= 64 for v in q[1:])
            err = abs(Fraction(x) - truncated(x, e))
            assert err < Fraction(2) ** (e - 7 * S)  # truncation below the last digit


def level_bound_per_k(S, complex_pair, qmax=None):
    """Largest |sum over pairs of level L| at one K index for digit bounds
    qmax (default: the balanced digits, |q_1| <= 128, |q_s| <= 64)."""
    qmax = qmax or [128] + [64] * (S - 1)
    best = 0
    for L in range(2, S + 2):
        tot = sum(qmax[s - 1] * qmax[L - s - 1] for s in range(1, L) if s <= S and L - s <= S)
        best = max(best, tot * (2 if complex_pair else 1))
    return best


def test_level_sums_stay_exact():
    # tensor cores: real level sums over a 512-wide chunk
    assert level_bound_per_k(5, False) * 512 <= 2 ** 24
    assert level_bound_per_k(6, False) * 512 <= 2 ** 24
    # the 1024-wide chunk used before could exceed 2^24, and so could plain
    # 7-bit digit magnitudes (up to 127) even over 512
    assert level_bound_per_k(5, False) * 1024 > 2 ** 24
    assert level_bound_per_k(5, False, [127] * 5) * 512 > 2 ** 24
    # FP32 pipe: complex level sums (two products per pair) up to K = 64
    assert level_bound_per_k(6, True) * 64 <= 2 ** 22


def test_fp32_accumulation_worst_case():
    """Same-sign maximal digits: FP32 running sums of one level are exact over
    512 products of the largest level and inexact beyond 2^24."""
    v = np.float32(28672.0)  # 2^14 + 2^13 + 2^12, the largest level-6 term (S = 5)
    acc = np.float32(0.0)
    for _ in range(512):
        acc = np.float32(acc + v)
    assert int(acc) == 28672 * 512
    odd = np.float32(28673.0)
    acc = np.float32(0.0)
    for _ in range(1024):
        acc = np.float32(acc + odd)
    assert int(acc) != 28673 * 1024  # past 2^24 the odd units round away


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_recombination_reproduces_truncated_product(seed):
    """A row of A and a column of B (K = 37): level sums, int64 recombination
    with u = 7 (min(S, 5) + 1) and the exponent scale give the exact dot
    product of the truncated operands (then one rounding to double)."""
    rng = np.random.default_rng(seed)
    K = 37
    a = rng.standard_normal(K) * 3.1
    b = rng.standard_normal(K) * 0.07
    ea, eb = row_exp(a), row_exp(b)
    da = [digits(x, ea) for x in a]
    db = [digits(x, eb) for x in b]
    levels = [0] * S
    for k in range(K):
        for s in range(S):
            for t in range(S - s):  # 0-based: level s + t, s + t <= S - 1
                levels[s + t] += da[k][s] * db[k][t]
    u = 7 * (min(S, 5) + 1)
    X = sum(v << (u - 7 * (L + 2)) for L, v in enumerate(levels))
    got = Fraction(X) * Fraction(2) ** (ea + eb - u)
    # the pairs dropped (s + t > S + 1) are below the truncation: compare to
    # the exact dot product of the truncated operands within that bound
    exact = sum(truncated(x, ea) * truncated(y, eb) for x, y in zip(a, b))
    dropped_bound = K * sum(128 * 128 * Fraction(2) ** (ea + eb - 7 * (s + t + 2))
                            for s in range(S) for t in range(S) if s + t > S - 1)
    assert abs(got - exact) <= dropped_bound
    # and the whole scheme within 2^-30 of the FP64 product's magnitude scale
    ref = float(np.dot(a, b))
    scale = float(np.dot(np.abs(a), np.abs(b)))
    assert abs(float(got) - ref) <= 2.0 ** -30 * scale
