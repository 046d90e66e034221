"""GPU parity of the unsteady dual-time BDF2 and backward Euler stages with the CPU oracle (needs a GB300).

BDF2_LU_SGS (Time_BDF2.f90:71-337) keeps the reference's operation order on
the device, including the per-cell dgesvx steps (equilibration, LU with
partial pivoting, the triangular solves and dgerfs's refinement), with FMA
contraction off; the results are expected to be bit-identical to the
oracle's.  The inner-iteration stop compares norms whose GPU reduction order
differs from the oracle's serial sum (rounding only), so the inner counts are
compared too.
"""
import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from conftest import make_case

pytestmark = pytest.mark.gpu

T1U = {"unsteady": True, "inner_loop": 4, "rel_tol": 1e-3, "totaltime": 1e-3, "nstep": 100000}


def _assemble(s, o):
    s.timestep(); s.reconstruction(); s.flux_sourceterm()
    o.call("timestep"); o.call("reconstruction"); o.call("flux_sourceterm")


@pytest.mark.parametrize("name,over", [("t2u", {}), ("t1", T1U), ("t2u", {"order": "random"})])
def test_bdf2_lusgs_bit_identical_to_oracle(case_root, name, over):
    d = make_case(case_root, name, **over)
    c = rc.Case(d)
    s = rc.Solver(c)
    o = oracle.Oracle(d, threads=4)
    dt = o.unsteady()["dt"]
    rng = np.random.default_rng(7)
    WA = o.array("WA").copy()
    WP = WA * (1 + 1e-3 * rng.standard_normal(WA.shape))
    WP2 = WA * (1 + 2e-3 * rng.standard_normal(WA.shape))
    o.array("WP")[:] = WP
    o.array("WP2")[:] = WP2
    s.set_array("WP", WP)
    s.set_array("WP2", WP2)
    for inner in (1, 2):
        _assemble(s, o)
        assert np.array_equal(s.get_array("hWA"), o.array("hWA"))
        assert o.bdf2_lusgs(inner, 0.5) == 0
        s.bdf2_lusgs(inner, 0.5, dt)
        s.sync()
        assert np.array_equal(s.get_array("hWA"), o.array("hWA")), inner
        PA, WA = s.get_state()
        assert np.array_equal(PA, o.array("PA")), inner
        assert np.array_equal(WA, o.array("WA")), inner


@pytest.mark.parametrize("name,over", [("t2u", {}), ("t1", T1U), ("t2u", {"order": "colored"}),
                                       ("t2u", {"a_p": 0.05, "f_p": 2.0e6}), ("t2u", {"time_method": 3}),
                                       ("t1", {**T1U, "time_method": 3})])
def test_unsteady_steps_bit_identical_to_oracle(case_root, name, over):
    """Ten physical steps of the driver (time advance, compute_p_out,
    BDF2_stage) against the oracle's; the last case has a moving exit
    pressure."""
    d = make_case(case_root, name, **over)
    c = rc.Case(d)
    _, inner_gpu = c.run_unsteady(10)
    o = oracle.Oracle(d, threads=4)
    inner_cpu = [o.unsteady_step(i)[0] for i in range(1, 11)]
    assert list(inner_gpu) == inner_cpu
    assert np.array_equal(c.array("PA"), o.array("PA"))
    assert np.array_equal(c.array("WA"), o.array("WA"))
    assert c.unsteady["ttime"] == o.unsteady()["ttime"]


@pytest.mark.parametrize("name,over", [("t2u", {}), ("t2u", {"nx": 300, "ny": 20}), ("t1", T1U),
                                       ("t2u", {"order": "random"})])
def test_bdf2_dataflow_sweeps_equal_level_sweeps(case_root, name, over, monkeypatch):
    """Both BDF2 sweeps as one cooperative dataflow launch (passes of up to 8
    positions of one level, per-pass flags between the SMs) against one
    launch per level: the same inner counts and bits after five physical
    steps; BDF2_LU_SGS is then three launches (set-up, sweeps, update)."""
    d = make_case(case_root, name, **over)
    got = {}
    for sched in ("levels", "dataflow"):
        monkeypatch.setenv("RC_BDF2_SCHEDULE", sched)
        c = rc.Case(d)
        _, inner = c.run_unsteady(5)
        got[sched] = (list(inner), c.array("PA").copy(), c.array("WA").copy())
        c.close()
    assert got["levels"][0] == got["dataflow"][0]
    assert np.array_equal(got["levels"][1], got["dataflow"][1])
    assert np.array_equal(got["levels"][2], got["dataflow"][2])
    c = rc.Case(d)
    s = rc.Solver(c)
    dt = oracle.Oracle(d).unsteady()["dt"]
    s.timestep(); s.reconstruction(); s.flux_sourceterm()
    n0 = s.stats()["kernel_launches"]
    s.bdf2_lusgs(2, 0.5, dt)
    s.sync()
    assert s.stats()["kernel_launches"] - n0 == 3
    s.close()


def test_bdf2_dataflow_wait_timeout_is_reported(case_root, monkeypatch):
    """A poll limit of 1 makes the BDF2 dataflow sweeps give up on a pass of
    another block: RC_ERR_SYNC, every block still finishes the launch, and
    after the error is cleared and the state set again the next call (a new
    epoch of the pass flags) gives the oracle's bits."""
    monkeypatch.setenv("RC_BDF2_SCHEDULE", "dataflow")
    d = make_case(case_root, "t2u")
    c = rc.Case(d)
    s = rc.Solver(c)
    o = oracle.Oracle(d, threads=4)
    dt = o.unsteady()["dt"]
    PA0, WA0 = c.array("PA").copy(), c.array("WA").copy()
    s.set_array("WP", WA0)
    s.set_array("WP2", WA0)
    s.set_wait_limit(1)
    s.timestep(); s.reconstruction(); s.flux_sourceterm()
    s.bdf2_lusgs(1, 0.5, dt)
    with pytest.raises(rc.RcError) as e:
        s.sync()
    assert e.value.code & 64
    s.clear_error()
    s.set_wait_limit(1 << 24)
    s.set_state(PA0, WA0)
    o.array("WP")[:] = WA0
    o.array("WP2")[:] = WA0
    _assemble(s, o)
    assert o.bdf2_lusgs(1, 0.5) == 0
    s.bdf2_lusgs(1, 0.5, dt)
    s.sync()
    PA, WA = s.get_state()
    assert np.array_equal(s.get_array("hWA"), o.array("hWA"))
    assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA"))
    s.close()


def test_stage_residual_and_history_levels(case_root):
    """Solver.bdf2_stage: after the stage hWA is the residual of the final
    flux_sourceterm, as in the oracle; the time levels WP / WP2 are WA of the
    previous steps."""
    d = make_case(case_root, "t2u")
    c = rc.Case(d)
    s = rc.Solver(c)
    o = oracle.Oracle(d, threads=4)
    u = o.unsteady()
    s.set_p_out(u["p_out"])
    WA_prev = []
    for istep in (1, 2, 3):
        WA_prev.append(s.get_state()[1])
        n = s.bdf2_stage(istep, u["dt"], u["inner_loop"], u["rel_tol"])
        m, _ = o.unsteady_step(istep)
        assert n == m
    assert np.array_equal(s.get_array("hWA"), o.array("hWA"))
    assert np.array_equal(s.get_array("WP"), WA_prev[2])
    assert np.array_equal(s.get_array("WP2"), WA_prev[1])
    PA, WA = s.get_state()
    assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA"))


def test_bdf2_rejects_what_it_does_not_cover(case_root):
    d = make_case(case_root, "t2u")
    c = rc.Case(d)
    s = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    with pytest.raises(rc.RcError):
        s.bdf2_stage(1, 1e-8, 2, 1e-3)
    steady = rc.Case(make_case(case_root, "t2"))
    with pytest.raises(rc.RcError):
        steady.run_unsteady(1)


def test_euler_lusgs_bit_identical_to_oracle(case_root):
    d = make_case(case_root, "t2u", time_method=3)
    c = rc.Case(d)
    s = rc.Solver(c)
    o = oracle.Oracle(d, threads=4)
    dt = o.unsteady()["dt"]
    for inner in (1, 2):
        _assemble(s, o)
        assert o.euler_lusgs(inner) == 0
        s.euler_lusgs(inner, dt)
        s.sync()
        assert np.array_equal(s.get_array("hWA"), o.array("hWA")), inner
        PA, WA = s.get_state()
        assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA")), inner


def test_driver_shortens_the_last_step_like_the_reference(case_root):
    """fvm2d.f90:52-56: the step that would pass totaltime is shortened to end
    on it and the loop stops; the driver does the same on the GPU."""
    d = make_case(case_root, "t2u", totaltime=2.5e-8, nstep=2, inner_loop=3)
    c = rc.Case(d)
    _, inner = c.run_unsteady(10)
    o = oracle.Oracle(d, threads=4)
    ref = []
    for i in range(1, 11):
        n, stop = o.unsteady_step(i)
        ref.append(n)
        if stop:
            break
    assert len(ref) == 2 and list(inner[:2]) == ref and inner[2:].sum() == 0
    assert c.unsteady["ttime"] == o.unsteady()["ttime"] == pytest.approx(2.5e-8, rel=1e-12)
    assert np.array_equal(c.array("PA"), o.array("PA"))


def test_bdf2_step_bit_identical_at_full_size(case_root):
    """One physical step of the shipped scheme on the 120,000-cell reacting
    nozzle (301 + 301 levels, 3-4 inner iterations) against the oracle."""
    d = make_case(case_root, "c2u")
    c = rc.Case(d)
    _, inner = c.run_unsteady(1)
    o = oracle.Oracle(d, threads=oracle.Oracle.max_threads())
    n, _ = o.unsteady_step(1)
    assert int(inner[0]) == n
    assert np.array_equal(c.array("PA"), o.array("PA"))
    assert np.array_equal(c.array("WA"), o.array("WA"))
