"""GPU chemistry integrator against the CPU oracle (needs a GB300).

The device integrator (csrc/rc_chem.cuh) keeps the oracle's operation order
with FMA contraction off and the shared exp/log/pow, so states and substep
counts are expected to be bit-identical.
"""
import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from conftest import make_case
from test_chem import states

pytestmark = pytest.mark.gpu


def test_batch_integration_bit_identical(case_root):
    import torch
    d = make_case(case_root, "t2")
    o = oracle.Oracle(d, threads=4)
    s = rc.Solver(rc.Case(d))
    P = states(o, 4096, 21)
    dt = 10 ** np.random.default_rng(22).uniform(-9, -5, len(P))
    ref, nref = o.chem_integrate(P, dt)
    Pd = torch.tensor(P.T.copy(), dtype=torch.float64, device="cuda")
    out, nsub = s.chem_integrate(Pd, torch.tensor(dt, device="cuda"))
    out = out.cpu().numpy().T
    assert np.array_equal(nsub.cpu().numpy(), nref)
    assert np.array_equal(out, ref)
    assert nref.max() > 10  # the sample spans uneven work


@pytest.mark.parametrize("name,over", [("t2", {}), ("c2", {"nx": 60, "ny": 10})])
def test_integrated_source_stage_bit_identical(case_root, name, over):
    d = make_case(case_root, name, **over)
    o = oracle.Oracle(d, threads=4)
    o.set_chemistry(1)
    s = rc.Solver(rc.Case(d))
    s.set_chemistry(rc.RC_CHEM_INTEGRATED)
    s.run(20)
    o.run(20)
    PA, WA = s.get_state()
    assert np.array_equal(s.chem_substeps(), o.chem_nsub())
    assert np.array_equal(PA, o.array("PA"))
    assert np.array_equal(WA, o.array("WA"))


def test_integrated_source_subroutine_calls_equal_stage(case_t2):
    c = rc.Case(case_t2)
    a, b = rc.Solver(c), rc.Solver(c)
    for s in (a, b):
        s.set_chemistry(rc.RC_CHEM_INTEGRATED)
    for it in range(1, 4):
        a.lu_sgs_stage(it)
        b.timestep(); b.reconstruction(); b.flux_sourceterm(); b.lu_sgs_steady()
    pa, _ = a.get_state()
    pb, _ = b.get_state()
    assert np.array_equal(pa, pb)


def test_integrated_source_mixed_precision(case_root):
    d = make_case(case_root, "c2", nx=60, ny=10)
    c = rc.Case(d)
    ref = rc.Solver(c)
    mix = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    for s in (ref, mix):
        s.set_chemistry(rc.RC_CHEM_INTEGRATED)
        s.run(20)
    pr, _ = ref.get_state()
    pm, _ = mix.get_state()
    err = np.abs(pm - pr).max(axis=0) / np.abs(pr).max(axis=0)
    assert np.all(np.isfinite(pm)) and err.max() <= 1e-3, err
