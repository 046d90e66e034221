"""Batched form: several independent nozzle cases in one context (needs a GB300).

Each case of a batch runs the recurrences it runs alone (the LU-SGS levels of
the shared numbering never mix cases), so its state and its norms are
expected to be bit-identical to a single-case context, in every precision and
chemistry mode.
"""
import os

import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from rocketcombustor_gb300 import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_dirs(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("batch"))
    return cases.make_batch(d, n=5, seed=9, ne_min=300, ne_max=3000)


@pytest.mark.parametrize("precision,chem", [(rc.RC_PREC_FP64, rc.RC_CHEM_EXPLICIT),
                                            (rc.RC_PREC_FP64, rc.RC_CHEM_INTEGRATED),
                                            (rc.RC_PREC_MIXED, rc.RC_CHEM_EXPLICIT)])
def test_batch_equals_cases_alone(batch_dirs, precision, chem):
    cs = [rc.Case(d) for d in batch_dirs]
    b = rc.BatchSolver(cs, precision=precision)
    b.set_chemistry(chem)
    b.run(25)
    PA, WA = b.get_state()
    rb, mb = b.residual()
    for k, c in enumerate(cs):
        s = rc.Solver(c, precision=precision)
        s.set_chemistry(chem)
        s.run(25)
        pa, wa = s.get_state()
        sl = b.case_slice(k)
        assert np.array_equal(PA[sl], pa), k
        assert np.array_equal(WA[sl], wa), k
        r, m = s.residual()
        assert np.array_equal(rb[k], r) and mb[k] == m, k
        s.close()


def test_batch_case_matches_oracle(batch_dirs):
    cs = [rc.Case(d) for d in batch_dirs]
    b = rc.BatchSolver(cs)
    b.run(10)
    PA, _ = b.get_state()
    k = len(cs) - 1
    o = oracle.Oracle(batch_dirs[k], threads=4)
    o.run(10)
    assert np.array_equal(PA[b.case_slice(k)], o.array("PA"))


def test_batch_uneven_sizes_and_conditions(batch_dirs):
    ne = [rc.Case(d).NE for d in batch_dirs]
    assert max(ne) > 2 * min(ne)
    cfgs = cases.batch_configs(n=5, seed=9, ne_min=300, ne_max=3000)
    assert len({round(c.p0) for c in cfgs}) == 5 and len({c.h_exit for c in cfgs}) == 5


def test_autotune_keeps_the_bits(batch_dirs):
    cs = [rc.Case(d) for d in batch_dirs]
    a = rc.BatchSolver(cs)
    b = rc.BatchSolver(cs)
    rep = b.autotune(2)
    assert "chosen" in rep
    a.run(15)
    b.run(15)
    assert np.array_equal(a.get_state()[0], b.get_state()[0])
