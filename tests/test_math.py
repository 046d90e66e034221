"""include/rc_math.h: the portable exp/log/pow of the FP64 path (no GPU).

The FP64 kernels and the oracle both evaluate exp/log/pow with these
functions, so their results are bit-identical; here they are pinned against
the host libm (numpy): within 1 ulp for exp and log and 4 ulp for pow over the
argument ranges of the solver (temperatures 200-60000 K, concentrations,
Arrhenius exponents), and against exact values (Python's decimal module):
exp within 0.51 ulp, log within 0.8 ulp.  The tables and reduction constants
of the header are regenerated here in exact arithmetic and compared entry by
entry.
"""
import os
import re
from decimal import Decimal, getcontext

import numpy as np

import oracle

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "rc_math.h")


def _ln2():
    getcontext().prec = 60
    return Decimal(2).ln()


def _round_to(d, bits):
    """d rounded to the nearest multiple of 2^-bits (exact, in Decimal)."""
    q = Decimal(2) ** bits
    return (d * q).to_integral_value() / q


def exp_table():
    """2^(j/128) for j = 0..127 as (lead, trail) pairs: lead = RN(2^(j/128)),
    trail = RN(2^(j/128) - lead) (Tang, ACM TOMS 15(2), 1989)."""
    ln2 = _ln2()
    out = []
    for j in range(128):
        v = (ln2 * j / 128).exp()
        hi = float(v)
        out += [hi, float(v - Decimal(hi))]
    return out


def log_table():
    """Per interval j of the reduced argument z (centre c = 1 + j/128, c = 1
    for j = 0): invc = RN(1/c), and -log(invc) as lead (a multiple of 2^-42,
    so that e ln2_lead + lead is exact) + trail, padded to 4 doubles."""
    getcontext().prec = 60
    out = []
    for j in range(128):
        invc = 1.0 if j == 0 else float(Decimal(1) / (1 + Decimal(j) / 128))
        lv = -Decimal(invc).ln()
        hi = _round_to(lv, 42)
        out += [invc, float(hi), float(lv - hi), 0.0]
    return out


def split_constants():
    """The reduction constants: 128/ln2, ln2/128 as lead + trail, ln2 as a
    42-bit lead + trail."""
    ln2 = _ln2()
    a = ln2 / 128
    a_hi = float(a)
    l_hi = _round_to(ln2, 42)
    return {"INV_LN2_128": float(128 / ln2), "LN2_128_HI": a_hi, "LN2_128_LO": float(a - Decimal(a_hi)),
            "LN2_HI42": float(l_hi), "LN2_LO42": float(ln2 - l_hi)}


def _header_array(name):
    src = open(HEADER).read()
    m = re.search(r"#define " + name + r"\s*\\?\s*\{([^}]*)\}", src)
    assert m, name
    return [float.fromhex(t) for t in re.findall(r"-?0x[0-9a-fp.+-]+", m.group(1))]


def _header_const(name):
    src = open(HEADER).read()
    m = re.search(r"constexpr double " + name + r" = (-?0x[0-9a-fp.+-]+);", src)
    assert m, name
    return float.fromhex(m.group(1))


def ulps(a, ref):
    a = np.asarray(a)
    ref = np.asarray(ref)
    sp = np.spacing(np.abs(ref))
    return np.where(a == ref, 0.0, np.abs(a - ref) / sp)


def test_exp_within_one_ulp():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-50, 12, 200000), rng.uniform(-700, 700, 20000), [0.0, -1e-300, 1e-10]])
    assert ulps(oracle.math("exp", x), np.exp(x)).max() <= 1.0


def test_log_within_one_ulp():
    rng = np.random.default_rng(1)
    x = np.concatenate([np.exp(rng.uniform(-40, 40, 200000)), rng.uniform(200, 60000, 50000),
                        [1.0, 2.0, 0.5, np.sqrt(2.0), 1e-310]])
    assert ulps(oracle.math("log", x), np.log(x)).max() <= 1.0


def test_pow_within_four_ulp():
    rng = np.random.default_rng(2)
    x = np.exp(rng.uniform(-12, 8, 200000))
    y = rng.uniform(-3, 3, 200000)
    assert ulps(oracle.math("pow", x, y), np.power(x, y)).max() <= 4.0
    # the exponents of the reference: omega_D, the global rate orders, Wilke
    for e in (-0.15610, 0.2, 1.3, 0.25):
        assert ulps(oracle.math("pow", x, np.full_like(x, e)), np.power(x, e)).max() <= 2.0


def test_special_values():
    assert oracle.math("exp", np.array([800.0]))[0] == np.inf
    assert oracle.math("exp", np.array([-800.0]))[0] == 0.0
    assert oracle.math("log", np.array([0.0]))[0] == -np.inf
    assert np.isnan(oracle.math("log", np.array([-1.0]))[0])
    assert oracle.math("pow", np.array([0.0]), np.array([0.2]))[0] == 0.0


def test_tables_and_constants_match_exact_arithmetic():
    assert _header_array("RCM_EXP_TAB_VALUES") == exp_table()
    assert _header_array("RCM_LOG_TAB_VALUES") == log_table()
    for name, v in split_constants().items():
        assert _header_const(name) == v, name


def _exact_ulps(got, x, f):
    import math
    getcontext().prec = 50
    out = []
    for g, xi in zip(got, x):
        ex = f(Decimal(float(xi)))
        out.append(float(abs(Decimal(float(g)) - ex)) / math.ulp(float(ex)))
    return np.array(out)


def test_errors_against_exact_values():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-700, 700, 3000), rng.uniform(-0.01, 0.01, 1000)])
    assert _exact_ulps(oracle.math("exp", x), x, lambda d: d.exp()).max() <= 0.51
    # log near 1 (results down to 2^-9 and below) and over the whole range
    x = np.concatenate([np.exp(rng.uniform(-700, 700, 2000)), 1 + rng.uniform(-0.01, 0.01, 2000)])
    assert _exact_ulps(oracle.math("log", x), x, lambda d: d.ln()).max() <= 0.8


def test_exp_overflow_and_underflow_thresholds():
    big = 709.782712893384  # the largest x with a finite exp(x)
    got = oracle.math("exp", np.array([big, np.nextafter(big, 800.0), -745.1332191019411, -745.1332191019412,
                                       -708.4, -740.0]))
    ref = np.array([np.exp(big), np.inf, 5e-324, 0.0, np.exp(-708.4), np.exp(-740.0)])
    assert np.array_equal(got, ref)
