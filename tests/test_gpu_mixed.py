"""Mixed-precision form (needs a GB300).

RC_PREC_MIXED runs reconstruction, limiter, face fluxes and the LU-SGS
off-diagonal terms in FP32 (compensated FP32 gather into an FP64 residual) and
keeps the step, diagonal division, chemistry, Newton update and norms in FP64.
RC_PREC_MIXED_DC (defect correction) drives the FP32 sweeps with the FP64
residual, so its fixed point is the FP64 one.  The error against the FP64
path is measured and bounded here: after 20 iterations the measured
differences are at most 2.3e-6 (t1) and 1.0e-6 (t2) relative L-infinity per
field, bounded at 1e-5 (a margin of 4-10 for other boxes and builds).  That
defect correction lands on the FP64 fixed point is tested at the converged
steady state (tests/test_gpu_steady.py).
"""
import numpy as np
import pytest

import rocketcombustor_gb300 as rc
from conftest import make_case

pytestmark = pytest.mark.gpu


def rel_linf(a, b):
    den = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return np.abs(a - b).max(axis=0) / den


@pytest.mark.parametrize("name", ["t1", "t2"])
def test_mixed_tracks_fp64(case_root, name):
    d = make_case(case_root, name)
    c = rc.Case(d)
    ref = rc.Solver(c, precision=rc.RC_PREC_FP64)
    mix = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    ref.run(20)
    mix.run(20)
    pr, _ = ref.get_state()
    pm, _ = mix.get_state()
    e = rel_linf(pm, pr)
    assert np.isfinite(pm).all()
    assert e.max() < 1e-5, e


def test_defect_correction_uses_fp64_residual(case_t2):
    """From one state, an FP64 step and a defect-correction step see the same
    residual; their updates differ only by the FP32 sweeps."""
    c = rc.Case(case_t2)
    a = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    b = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    a.set_precision(rc.RC_PREC_FP64)
    b.set_precision(rc.RC_PREC_MIXED_DC)
    for s in (a, b):
        s.timestep(); s.reconstruction(); s.flux_sourceterm()
    ra, rb = a.get_array("hWA"), b.get_array("hWA")
    # same FP64 reconstruction and flux; only the spectral radius is FP32 in DC
    assert rel_linf(rb, ra).max() < 1e-12
    a.lu_sgs_steady(); b.lu_sgs_steady()
    da, db = a.get_array("hWA"), b.get_array("hWA")
    assert rel_linf(db, da).max() < 1e-4


def test_mixed_stage_graph_equals_subroutines(case_t2):
    c = rc.Case(case_t2)
    a = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    b = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    for it in range(1, 4):
        a.lu_sgs_stage(it)
        b.timestep(); b.reconstruction(); b.flux_sourceterm(); b.lu_sgs_steady()
    assert np.array_equal(a.get_state()[0], b.get_state()[0])


def test_mode_switching_keeps_graphs_apart(case_t1):
    c = rc.Case(case_t1)
    s = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    s.run(3)
    s.set_precision(rc.RC_PREC_MIXED_DC)
    s.run(3)
    s.set_precision(rc.RC_PREC_FP64)
    s.run(3)
    s.set_precision(rc.RC_PREC_MIXED)
    s.run(3)
    assert np.isfinite(s.get_state()[0]).all()
    plain = rc.Solver(c)
    with pytest.raises(rc.RcError):
        plain.set_precision(rc.RC_PREC_MIXED)


def test_steady_driver_fp64_equals_solver_run(case_root):
    """rc_run_steady (the host driver of fvm2d.f90's steady loop) runs the
    same graph as Solver.run: identical states."""
    d = make_case(case_root, "t2")
    a = rc.Case(d)
    hist = a.run_steady(40, every=10)
    b = rc.Solver(rc.Case(d))
    b.run(40)
    assert hist.shape == (4, a.NVar + 1)
    assert np.array_equal(a.array("PA"), b.get_state()[0])


def test_defect_correction_switch(case_root):
    """Mixed precision switches to the FP64 residual once the FP32 residual
    stalls; afterwards the iteration continues from the mixed state."""
    d = make_case(case_root, "c1", nx=60, ny=12)
    c = rc.Case(d)
    hist, sw = c.run_steady_dc(600, every=10, window=3)
    assert 0 < sw <= 600, sw
    assert np.all(np.isfinite(c.array("PA")))
    assert np.all(np.isfinite(hist))
