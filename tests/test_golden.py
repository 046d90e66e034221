"""The committed golden vectors (tests/golden/) against the CPU oracle.

The vectors were made by tests/golden/make_golden.py from the oracle on three
committed 288-cell cases; these tests check that the committed inputs are the
ones the vectors were made from, that the oracle still reproduces them bit for
bit, and that the case generator still writes the committed inputs.  The GPU
side of the same vectors is tests/test_gpu_golden.py.
"""
import filecmp
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as mg  # noqa: E402


@pytest.mark.parametrize("name", list(mg.CASES))
def test_committed_inputs_match_their_digest(name):
    assert mg.digest(mg.case_dir(name)) == str(mg.load(name)["digest"])


@pytest.mark.parametrize("name", list(mg.CASES))
def test_oracle_reproduces_the_golden_vectors(name, tmp_path):
    gold = mg.load(name)
    out = mg.oracle_outputs(name, mg.working_copy(name, str(tmp_path)))
    for k, v in out.items():
        assert np.array_equal(v, gold[k]), k


@pytest.mark.parametrize("name", list(mg.CASES))
def test_case_generator_writes_the_committed_inputs(name, tmp_path):
    from rocketcombustor_gb300 import cases

    d = os.path.join(str(tmp_path), name)
    cases.make_case(d, name)
    cmp = filecmp.dircmp(d, mg.case_dir(name))
    stack = [cmp]
    while stack:
        c = stack.pop()
        assert not (c.left_only or c.right_only or c.diff_files or c.funny_files), (c.left, c.diff_files)
        stack.extend(c.subdirs.values())
    assert mg.digest(d) == mg.digest(mg.case_dir(name))


def test_golden_histories_are_physical():
    """Positive, finite norms; the residual falls over the first iterations
    from the uniform/isentropic start, and the unsteady steps converge their
    inner loops within the shipped limit of 10."""
    for name, (kind, n) in mg.CASES.items():
        g = mg.load(name)
        assert np.isfinite(g["PA"]).all() and (g["PA"][:, 0] > 0).all() and (g["PA"][:, 3] > 0).all()
        if kind == "steady":
            h = g["history"]
            assert h.shape[0] == n and (h > 0).all() and np.isfinite(h).all()
            assert (h[-1, :-1] < h[0, :-1]).all()
        else:
            assert len(g["inner"]) == n and (1 <= g["inner"]).all() and (g["inner"] <= 10).all()
