"""include/rc_math.h: the portable exp/log/pow of the FP64 path (no GPU).

The FP64 kernels and the oracle both evaluate exp/log/pow with these
functions, so their results are bit-identical; here they are pinned against
the host libm (numpy): within 1 ulp for exp and log and 4 ulp for pow over the
argument ranges of the solver (temperatures 200-60000 K, concentrations,
Arrhenius exponents).
"""
import numpy as np

import oracle


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
