"""rc_set_state / rc_get_state with page-locked host buffers (converted in
place by the device over the CPU-GPU link) give the same bits as with
pageable buffers (one copy through the staging buffer).  Needs a GB300."""
import numpy as np
import pytest

import rocketcombustor_gb300 as rc
from conftest import make_case

pytestmark = pytest.mark.gpu


def test_page_locked_and_pageable_state_transfers_agree(case_root):
    torch = pytest.importorskip("torch")
    d = make_case(case_root, "t2")
    c = rc.Case(d)
    s = rc.Solver(c)
    s.run(3)
    PA, WA = s.get_state()  # pageable
    PA_p = torch.zeros((c.NE, c.NVar), dtype=torch.float64, pin_memory=True).numpy()
    WA_p = torch.zeros((c.NE, c.NVar), dtype=torch.float64, pin_memory=True).numpy()
    s.get_state(PA_p, WA_p)  # page-locked, written in place by the device
    assert np.array_equal(PA, PA_p) and np.array_equal(WA, WA_p)
    # round trip through page-locked input, then one iteration from either path
    rng = np.random.default_rng(5)
    PA_p *= 1 + 1e-6 * rng.standard_normal(PA_p.shape)
    WA_p *= 1 + 1e-6 * rng.standard_normal(WA_p.shape)
    s.set_state(PA_p, WA_p)
    s.sync()
    a = s.get_state()
    assert np.array_equal(a[0], PA_p) and np.array_equal(a[1], WA_p)
    s.lu_sgs_stage(1)
    x = s.get_state()
    s.set_state(PA_p.copy(), WA_p.copy())  # pageable copies of the same values
    s.lu_sgs_stage(1)
    y = s.get_state()
    assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
