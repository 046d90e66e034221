"""The FP64 GPU path against the committed golden vectors (needs a GB300).

tests/golden/ holds three 288-cell cases in the reference's file formats and
the CPU oracle's state after 50 steady iterations (t1 inviscid perfect gas,
t2 reacting viscous) or 3 physical BDF2 steps (t2u).  The GPU must give the
same bits through the subroutine-level Solver, the C++ steady driver and the
unsteady driver, without the oracle being built or run.  The residual norms
come from identical states and differ from the oracle's serial sums only by
the order of the GPU's reduction.
"""
import os
import sys

import numpy as np
import pytest

import rocketcombustor_gb300 as rc

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as mg  # noqa: E402

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12  # same states, another summation order of the norms

STEADY = [n for n, (kind, _) in mg.CASES.items() if kind == "steady"]


def _check_norms(res, romax, row):
    np.testing.assert_allclose(res, row[:-1], rtol=NORM_RTOL, atol=0.0)
    assert romax == pytest.approx(row[-1], rel=NORM_RTOL)


@pytest.mark.parametrize("name", STEADY)
def test_solver_iterations_equal_the_golden_vectors(name, tmp_path):
    gold = mg.load(name)
    c = rc.Case(mg.working_copy(name, str(tmp_path)))
    s = rc.Solver(c, device=0)
    for it in range(1, mg.CASES[name][1] + 1):
        s.lu_sgs_stage(it)
        _check_norms(*s.residual(), gold["history"][it - 1])
    PA, WA = s.get_state()
    assert np.array_equal(PA, gold["PA"])
    assert np.array_equal(WA, gold["WA"])
    assert np.array_equal(s.get_array("hWA"), gold["hWA"])
    s.close()


@pytest.mark.parametrize("name", STEADY)
def test_steady_driver_equals_the_golden_vectors(name, tmp_path):
    gold = mg.load(name)
    c = rc.Case(mg.working_copy(name, str(tmp_path)))
    hist = c.run_steady(mg.CASES[name][1], every=1)
    for row, ref in zip(hist, gold["history"]):
        _check_norms(row[:-1], row[-1], ref)
    assert np.array_equal(c.array("PA"), gold["PA"])
    assert np.array_equal(c.array("WA"), gold["WA"])


def test_unsteady_steps_equal_the_golden_vectors(tmp_path):
    gold = mg.load("t2u")
    c = rc.Case(mg.working_copy("t2u", str(tmp_path)))
    _, inner = c.run_unsteady(mg.CASES["t2u"][1])
    assert list(inner) == list(gold["inner"])
    assert np.array_equal(c.array("PA"), gold["PA"])
    assert np.array_equal(c.array("WA"), gold["WA"])
