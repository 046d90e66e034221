"""GPU parity of the plain FP64 path against the CPU oracle (needs a GB300).

The FP64 kernels keep the reference's operation order with FMA contraction
off, so +,-,*,/ and sqrt round exactly as on the CPU, and exp/log/pow come
from include/rc_math.h on both sides.  The GPU results are therefore expected
to be bit-identical to the oracle's; `test_fp64_path_bit_identical_to_oracle`
checks exactly that.  The tolerance tests keep the stated bars: 1e-12 relative
L-infinity per field for a single subroutine and 1e-9 after 100 iterations.
"""
import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from conftest import make_case

pytestmark = pytest.mark.gpu

ONE_CALL_RTOL = 1e-12
ITER_RTOL = 1e-9


def rel_linf(a, b):
    """max |a-b| / max |b| per trailing column (per field)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    a2 = a.reshape(a.shape[0], -1) if a.ndim > 1 else a[:, None]
    b2 = b.reshape(b.shape[0], -1) if b.ndim > 1 else b[:, None]
    den = np.maximum(np.abs(b2).max(axis=0), 1e-300)
    return (np.abs(a2 - b2).max(axis=0) / den)


def solver_and_oracle(d, threads=4):
    c = rc.Case(d)
    s = rc.Solver(c)
    o = oracle.Oracle(d, threads=threads)
    return c, s, o


@pytest.mark.parametrize("name", ["t1", "t2"])
def test_subroutines_match_oracle(case_root, name):
    d = make_case(case_root, name)
    c, s, o = solver_and_oracle(d)
    s.timestep(); o.call("timestep")
    r = rel_linf(s.get_array("alpaF"), o.array("alpaF")).max()
    if name == "t1":
        assert np.array_equal(s.get_array("alpaF"), o.array("alpaF"))
        assert np.array_equal(s.get_array("step"), o.array("step"))
    assert r <= ONE_CALL_RTOL
    assert rel_linf(s.get_array("step"), o.array("step")).max() <= ONE_CALL_RTOL
    s.reconstruction(); o.call("reconstruction")
    assert rel_linf(s.get_array("GPA"), o.array("GPA")).max() <= ONE_CALL_RTOL
    assert rel_linf(s.get_array("GradC"), o.array("GradC")).max() <= ONE_CALL_RTOL
    s.flux_sourceterm(); o.call("flux_sourceterm")
    assert rel_linf(s.get_array("hWA"), o.array("hWA")).max() <= 1e-11
    s.lu_sgs_steady(); o.call("lu_sgs_steady")
    assert rel_linf(s.get_array("hWA"), o.array("hWA")).max() <= 1e-10
    PA, WA = s.get_state()
    assert rel_linf(PA, o.array("PA")).max() <= ONE_CALL_RTOL
    assert rel_linf(WA, o.array("WA")).max() <= ONE_CALL_RTOL


@pytest.mark.parametrize("name,over", [("t1", {}), ("t2", {}), ("t1", {"order": "random"}),
                                       ("t2", {"order": "colored"})])
def test_100_iterations_match_oracle(case_root, name, over):
    d = make_case(case_root, name, **over)
    c, s, o = solver_and_oracle(d)
    s.run(100)
    o.run(100)
    PA, WA = s.get_state()
    err_pa = rel_linf(PA, o.array("PA"))
    err_wa = rel_linf(WA, o.array("WA"))
    assert err_pa.max() <= ITER_RTOL, err_pa
    assert err_wa.max() <= ITER_RTOL, err_wa
    r_gpu, m_gpu = s.residual()
    r_cpu, m_cpu = o.residual()
    np.testing.assert_allclose(r_gpu, r_cpu, rtol=1e-7, atol=1e-300)
    assert m_gpu == pytest.approx(m_cpu, rel=1e-9)


@pytest.mark.parametrize("name,over", [("t1", {}), ("t2", {}), ("t2", {"order": "random"}),
                                       ("c1", {"nx": 60, "ny": 12}), ("t2", {"inlet_burnt": 0.9, "nx": 12, "ny": 4})])
def test_fp64_path_bit_identical_to_oracle(case_root, name, over):
    d = make_case(case_root, name, **over)
    c, s, o = solver_and_oracle(d)
    gpu_code = cpu_code = 0
    try:
        s.run(100)
    except rc.RcError as e:
        gpu_code = e.code
    for it in range(100):  # stops at the first stop condition, as the reference does
        cpu_code = o.call("lu_sgs_stage")
        if cpu_code:
            break
    if cpu_code or gpu_code:
        # a case that stops must stop on both; the GPU keeps running after the
        # latch, so it may have collected more conditions
        assert cpu_code and gpu_code and (cpu_code & gpu_code) == cpu_code, (cpu_code, gpu_code)
        return
    PA, WA = s.get_state()
    assert np.array_equal(PA, o.array("PA")), rel_linf(PA, o.array("PA"))
    assert np.array_equal(WA, o.array("WA")), rel_linf(WA, o.array("WA"))
    assert np.array_equal(s.get_array("hWA"), o.array("hWA"))


def test_stage_graph_equals_subroutine_calls(case_t2):
    c = rc.Case(case_t2)
    a = rc.Solver(c)
    b = rc.Solver(c)
    for it in range(1, 4):
        a.lu_sgs_stage(it)
        b.timestep(); b.reconstruction(); b.flux_sourceterm(); b.lu_sgs_steady()
    pa, wa = a.get_state()
    pb, wb = b.get_state()
    assert np.array_equal(pa, pb) and np.array_equal(wa, wb)


def test_bit_reproducible_run_to_run(case_root):
    d = make_case(case_root, "c1", nx=80, ny=16)
    c = rc.Case(d)
    out = []
    for _ in range(2):
        s = rc.Solver(c)
        s.run(50)
        out.append(s.get_state()[0].tobytes())
        s.close()
    assert out[0] == out[1]


def test_full_size_c1_100_iterations(case_root):
    """The 20k-triangle inviscid nozzle at its full size, 100 iterations."""
    d = make_case(case_root, "c1")
    c, s, o = solver_and_oracle(d, threads=oracle.Oracle.max_threads())
    s.run(100)
    o.run(100)
    PA, WA = s.get_state()
    assert rel_linf(PA, o.array("PA")).max() <= ITER_RTOL
    assert rel_linf(WA, o.array("WA")).max() <= ITER_RTOL
    assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA"))


def test_full_size_c2_20_iterations(case_root):
    """The 120k-triangle reacting viscous nozzle at its full size, 20
    iterations (the autotuned schedule), bit for bit."""
    d = make_case(case_root, "c2")
    c, s, o = solver_and_oracle(d, threads=oracle.Oracle.max_threads())
    s.autotune(2)
    s.run(20)
    o.run(20)
    PA, WA = s.get_state()
    assert rel_linf(PA, o.array("PA")).max() <= ITER_RTOL
    assert rel_linf(WA, o.array("WA")).max() <= ITER_RTOL
    assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA"))


@pytest.mark.parametrize("precision", [rc.RC_PREC_FP64, rc.RC_PREC_MIXED])
def test_full_size_c4_3_iterations(case_root, precision):
    """The 2,000,000-triangle reacting viscous nozzle (the benchmark workload)
    at its full size: 3 iterations with the autotuned schedule.  FP64 is bit
    for bit the oracle's (run on all host threads); the mixed form stays
    within its stated bound of the oracle (p, T 1e-4, Y_k 1e-3 relative
    L-infinity after 3 iterations from the same state)."""
    d = make_case(case_root, "c4")
    c = rc.Case(d)
    s = rc.Solver(c, precision=precision)
    s.autotune(2)
    s.set_state(c.array("PA"), c.array("WA"))
    s.run(3)
    o = oracle.Oracle(d, threads=oracle.Oracle.max_threads())
    o.run(3)
    PA, WA = s.get_state()
    if precision == rc.RC_PREC_FP64:
        assert np.array_equal(PA, o.array("PA")), rel_linf(PA, o.array("PA"))
        assert np.array_equal(WA, o.array("WA")), rel_linf(WA, o.array("WA"))
    else:
        e = rel_linf(PA, o.array("PA"))
        assert e[0] <= 1e-4 and e[3] <= 1e-4 and e[4:].max() <= 1e-3, e
    s.close()
    o.close()


def test_device_stop_condition_is_reported(case_t1):
    """A negative pressure planted in the host state is caught by TimeStep's
    check (TimeStep.f90:66-70) and reported at the next synchronising call."""
    c = rc.Case(case_t1)
    s = rc.Solver(c)
    PA = c.array("PA").copy()
    PA[5, 0] = -PA[5, 0]
    s.set_state(PA, c.array("WA"))
    s.timestep()
    with pytest.raises(rc.RcError) as e:
        s.sync()
    assert e.value.code & 4


@pytest.mark.parametrize("precision", [rc.RC_PREC_FP64, rc.RC_PREC_MIXED])
@pytest.mark.parametrize("name,over", [("c1", {"nx": 40, "ny": 8}), ("t2", {})])
def test_persistent_and_per_level_schedules_agree(case_root, precision, name, over, monkeypatch):
    """The cooperative one-launch LU-SGS, the one-launch-per-level LU-SGS
    (4 lanes per cell with 8 or 1 cells per warp, 8 lanes per cell, or the work
    of each slot split over two or four warps) and the dataflow launches run
    the same recurrences: identical states after 30 iterations.  In mixed
    precision the dataflow launch does the FP64 Newton update inside the sweep
    launch and the other schedules in a separate k_update: the one-species
    inviscid nozzle and the four-species reacting viscous case check both
    builds of that update."""
    d = make_case(case_root, name, **over)
    c = rc.Case(d)
    states = []
    for sched in ("persistent", "levels", "levels8", "levels2w", "levels4w", "flow", "flow2", "flow3", "flowc",
                  "flowc2"):
        for cpw in ("8", "1"):
            monkeypatch.setenv("RC_LUSGS_SCHEDULE", sched)
            monkeypatch.setenv("RC_LUSGS_CPW", cpw)
            s = rc.Solver(c, precision=precision)
            s.run(30)
            states.append(s.get_state())
            s.close()
    for st in states[1:]:
        assert np.array_equal(states[0][0], st[0])
        assert np.array_equal(states[0][1], st[1])


@pytest.mark.parametrize("sched", ["flow", "flow2", "flow3", "flowc", "flowc2"])
def test_dataflow_schedule_bit_identical_to_oracle(case_root, sched, monkeypatch):
    """The dataflow LU-SGS (cells split into per-SM blocks, waits only on the
    passes of other blocks that hold a neighbour; passes of up to 8, 16 or 24
    cells over 1, 2 or 3 groups of compute warps, or compact passes of one
    or two groups of up to 16 cells and 32 active pairs) on the reacting
    viscous case and on the colored order, 20 iterations against the oracle."""
    monkeypatch.setenv("RC_LUSGS_SCHEDULE", sched)
    for name, over in (("t2", {}), ("c1", {"nx": 120, "ny": 20}), ("t2", {"order": "colored"})):
        d = make_case(case_root, name, **over)
        c = rc.Case(d)
        s = rc.Solver(c)
        s.run(20)
        PA, WA = s.get_state()
        o = oracle.Oracle(d, threads=4)
        o.run(20)
        assert np.array_equal(PA, o.array("PA")), (name, over)
        assert np.array_equal(WA, o.array("WA")), (name, over)
        s.close()


THIN = {"nx": 9000, "ny": 4}


@pytest.mark.parametrize("name,over", [("c1", THIN), ("c2", THIN)])
@pytest.mark.parametrize("sched", ["flowc", "flowc2"])
def test_compact_dataflow_wide_levels_bit_identical_to_oracle(case_root, sched, name, over, monkeypatch):
    """A long, thin nozzle (9000 x 4 columns of triangles, 72,000 cells) puts
    about 39 cells of every level in each of the 152 blocks: a compact group
    holds up to 32 active (cell, face) pairs and 128 / V cells (32 for one
    species, 18 for four), so passes fill two groups (fewer passes with two
    groups than with one).  The one-species inviscid and the four-species
    reacting viscous physics, 20 iterations against the oracle, bit for bit."""
    from test_flow_plan import _graph

    nv = 4 if name == "c1" else 7
    nface, cother = _graph(over["nx"], over["ny"], "natural")
    one = rc.flow_plan_check(nface, cother, 152, groups=1, compact=True, nvar=nv)
    two = rc.flow_plan_check(nface, cother, 152, groups=2, compact=True, nvar=nv)
    assert two["passes_fwd"] < one["passes_fwd"] and two["passes_bwd"] < one["passes_bwd"]
    monkeypatch.setenv("RC_LUSGS_SCHEDULE", sched)
    d = make_case(case_root, name, **over)
    c = rc.Case(d)
    s = rc.Solver(c)
    s.run(20)
    PA, WA = s.get_state()
    o = oracle.Oracle(d, threads=oracle.Oracle.max_threads())
    o.run(20)
    assert np.array_equal(PA, o.array("PA")), rel_linf(PA, o.array("PA"))
    assert np.array_equal(WA, o.array("WA")), rel_linf(WA, o.array("WA"))
    s.close()


@pytest.mark.parametrize("name,over", [("c1", THIN), ("c2", THIN)])
def test_compact_mixed_dataflow_equals_per_level_sweeps(case_root, name, over, monkeypatch):
    """The mixed-precision compact dataflow launch (FP32 terms of the active
    pairs only, groups of up to 16 cells, the FP64 Newton update inside the
    launch) on the long, thin nozzle whose passes fill two groups: after 20
    iterations its state is bit for bit that of the per-level FP32 sweeps
    followed by k_update, with one group and with two."""
    d = make_case(case_root, name, **over)
    c = rc.Case(d)
    states = {}
    for sched in ("levels", "flowc", "flowc2"):
        monkeypatch.setenv("RC_LUSGS_SCHEDULE", sched)
        s = rc.Solver(c, precision=rc.RC_PREC_MIXED)
        s.run(20)
        states[sched] = s.get_state()
        s.close()
    for sched in ("flowc", "flowc2"):
        assert np.array_equal(states["levels"][0], states[sched][0]), sched
        assert np.array_equal(states["levels"][1], states[sched][1]), sched


@pytest.mark.parametrize("sched", ["flow", "flow3", "flowc2"])
def test_dataflow_wait_timeout_is_reported(case_root, sched, monkeypatch):
    """A poll limit of 1 makes the dataflow LU-SGS give up on a pass of
    another block: RC_ERR_SYNC, every block still finishes the launch, and
    after the error is cleared the next launches (a new epoch) are exact."""
    monkeypatch.setenv("RC_LUSGS_SCHEDULE", sched)
    d = make_case(case_root, "c1", nx=60, ny=12)
    c = rc.Case(d)
    s = rc.Solver(c)
    s.set_wait_limit(1)
    s.lu_sgs_stage(1)
    with pytest.raises(rc.RcError) as e:
        s.sync()
    assert e.value.code & 64
    s.clear_error()
    s.set_wait_limit(1 << 24)
    s.set_state(c.array("PA"), c.array("WA"))
    s.run(5)
    o = oracle.Oracle(d, threads=4)
    o.run(5)
    PA, WA = s.get_state()
    assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA"))


@pytest.mark.parametrize("sched", ["flow", "flowc2", "persistent"])
def test_mixed_wait_timeout_is_reported(case_root, sched, monkeypatch):
    """The mixed-precision LU-SGS launches give up the same way: a poll limit
    of 1 ends the staging, hand-over and update-warp waits of the FP32 dataflow
    launches (8-position or compact passes) or the level waits of the FP32
    persistent launch with RC_ERR_SYNC;
    after the error is cleared and the state set again, five iterations give
    the bits of a clean mixed run from the same state."""
    monkeypatch.setenv("RC_LUSGS_SCHEDULE", sched)
    d = make_case(case_root, "t2")
    c = rc.Case(d)
    s = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    s.set_wait_limit(1)
    s.lu_sgs_stage(1)
    with pytest.raises(rc.RcError) as e:
        s.sync()
    assert e.value.code & 64
    s.clear_error()
    s.set_wait_limit(1 << 24)
    s.set_state(c.array("PA"), c.array("WA"))
    s.run(5)
    clean = rc.Solver(c, precision=rc.RC_PREC_MIXED)
    clean.set_state(c.array("PA"), c.array("WA"))
    clean.run(5)
    PA, WA = s.get_state()
    PA0, WA0 = clean.get_state()
    assert np.array_equal(PA, PA0) and np.array_equal(WA, WA0)
    s.close()
    clean.close()


def test_forced_level_wait_timeout_is_reported(case_root, monkeypatch):
    """A tiny poll limit makes the persistent LU-SGS give up waiting for the
    previous level: RC_ERR_SYNC is reported, the kernel returns, and the
    context stays usable after the error is cleared."""
    monkeypatch.setenv("RC_LUSGS_SCHEDULE", "persistent")
    d = make_case(case_root, "c1", nx=60, ny=12)
    c = rc.Case(d)
    s = rc.Solver(c)
    s.set_wait_limit(1)
    s.lu_sgs_stage(1)
    with pytest.raises(rc.RcError) as e:
        s.sync()
    assert e.value.code & 64
    s.clear_error()
    s.set_wait_limit(1 << 24)
    s.set_state(c.array("PA"), c.array("WA"))
    s.run(5)
    o = oracle.Oracle(d, threads=4)
    o.run(5)
    assert np.array_equal(s.get_state()[0], o.array("PA"))


def test_out_of_range_temperature_is_reported(case_t1):
    """T beyond the thermo fit in one cell stops at the next synchronising call
    (ComputeGasParameter, thermo_property.f90:97-101)."""
    c = rc.Case(case_t1)
    s = rc.Solver(c)
    PA = c.array("PA").copy()
    PA[3, 3] = 1.0e6
    s.set_state(PA, c.array("WA"))
    s.timestep()
    with pytest.raises(rc.RcError) as e:
        s.sync()
    assert e.value.code & 1
