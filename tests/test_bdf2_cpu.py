"""The unsteady dual-time BDF2 and backward Euler schemes on the CPU oracle (no GPU).

The reference solves each cell's system of its BDF2 sweeps with LAPACK's
dgesvx (advanced_linear_solve_lapack, la_math.f90:120-213).  The oracle
restates dgesvx; that restatement is pinned here against SciPy's LAPACK on
badly scaled random systems and on the BDF2 cell matrices themselves, then
the scheme is checked by its own properties: serial (reference loop order)
and level-scheduled runs agree bit for bit, a fluid at rest stays at rest,
with a tiny physical step the update is dt times the residual per volume,
the inner-iteration stop and the final shortened step behave as
Time_BDF2.f90 and fvm2d.f90 say.
"""
import numpy as np
import pytest

import oracle
from conftest import make_case


def _badly_scaled(rng, n):
    a = rng.standard_normal((n, n))
    a *= 10.0 ** rng.uniform(-6, 6, (n, 1))
    a *= 10.0 ** rng.uniform(-4, 4, (1, n))
    return a


def _check_against_lapack(a, b, rtol=1e-12):
    lapack = pytest.importorskip("scipy.linalg.lapack")
    x, info, equed, rcond = oracle.dgesvx(a, b)
    res = lapack.dgesvx(a, b[:, None], fact="E")
    x_ref, equed_ref, rcond_ref, info_ref = res[7][:, 0], res[3], res[8], res[-1]
    assert info == info_ref
    assert equed == (equed_ref.decode() if isinstance(equed_ref, bytes) else equed_ref)
    if info == 0:
        # rcond: both are Hager-Higham estimates (lower bounds of ||A^-1||),
        # so at least the true reciprocal condition number
        As = res[0]
        true = 1.0 / (np.linalg.norm(As, 1) * np.linalg.norm(np.linalg.inv(As), 1))
        assert true * (1 - 1e-6) <= rcond <= 10 * true  # (numpy's inverse is itself inexact)
        # both refine to the componentwise backward error eps; the triangular
        # solves of the two LAPACK builds round differently, so the solutions
        # agree to the condition number of the equilibrated matrix times eps
        tol = max(rtol, 50 * 2.22e-16 / true)
        assert np.max(np.abs(x - x_ref)) <= tol * np.max(np.abs(x_ref))
    return x, info, equed


def test_dgesvx_restatement_matches_lapack_on_badly_scaled_systems():
    rng = np.random.default_rng(0)
    seen = set()
    for _ in range(600):
        n = int(rng.integers(1, 9))
        a = _badly_scaled(rng, n)
        b = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3, n)
        _, _, equed = _check_against_lapack(a, b)
        seen.add(equed)
    assert seen == {"N", "R", "C", "B"}  # every equilibration branch was exercised


def test_dgesvx_singular_matrix_reports_the_zero_pivot():
    a = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [1.0, 0.0, 1.0]])
    a[:, 2] = a[:, 0] + a[:, 1]  # rank 2, exactly singular in floating point
    x, info, equed, rcond = oracle.dgesvx(a, np.ones(3))
    assert info > 0 or rcond < 1.1102230246251565e-16


def test_dgesvx_on_the_bdf2_cell_matrices(case_root):
    """The matrices the sweeps solve: dU/dP dd - vol d omega/dP."""
    d = make_case(case_root, "t2u")
    o = oracle.Oracle(d)
    rng = np.random.default_rng(3)
    PA, vol = o.array("PA"), o.array("VOL")
    for i in rng.choice(o.NE, 40, replace=False):
        dd = 10.0 ** rng.uniform(-6, -2)
        a = o.con_to_pri_jaco(PA[i]) * dd
        a[4:] -= vol[i] * o.dwdp(PA[i])
        b = rng.standard_normal(o.NVar) * np.abs(a).max(axis=1)
        x, info, _ = _check_against_lapack(a, b)
        assert info == 0


@pytest.mark.parametrize("name", ["t2u", "t1u", "t2u_euler"])
def test_serial_and_level_scheduled_bdf2_agree_bitwise(case_root, name):
    over = {"t2u": {}, "t2u_euler": {"time_method": 3},
            "t1u": {"unsteady": True, "inner_loop": 4, "rel_tol": 1e-3, "totaltime": 1e-3, "nstep": 100000}}[name]
    d = make_case(case_root, "t1" if name == "t1u" else "t2u", **over)
    out = []
    for th in (1, 4):
        o = oracle.Oracle(d, threads=th)
        inner = [o.unsteady_step(i)[0] for i in range(1, 5)]
        out.append((o.array("PA").copy(), o.array("WA").copy(), o.array("hWA").copy(), inner))
    for a, b in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(a, b)
    assert out[0][3] == out[1][3]


def test_fluid_at_rest_stays_at_rest(case_root):
    d = make_case(case_root, "t1", closed=True, unsteady=True, inner_loop=3, totaltime=1e-3, nstep=1000)
    o = oracle.Oracle(d)
    PA0 = o.array("PA").copy()
    for i in range(1, 4):
        o.unsteady_step(i)
    dev = np.abs(o.array("PA") - PA0).max(axis=0)
    assert dev[0] <= 1e-13 * PA0[:, 0].max() and dev[3] <= 1e-13 * PA0[:, 3].max()
    assert dev[1] <= 1e-9 and dev[2] <= 1e-9  # m/s, from rest


@pytest.mark.parametrize("method", [5, 3])
def test_tiny_step_moves_the_state_by_dt_times_the_residual(case_root, method):
    """The first BDF2 step (phi = 0) and every backward Euler step are implicit
    Euler in physical time: for dt much below the pseudo time steps,
    (U1 - U0) vol / dt -> R(U0), the residual of flux_sourceterm."""
    dt = 1e-12
    d = make_case(case_root, "t2u", totaltime=dt * 1e5, nstep=100000, inner_loop=6, rel_tol=1e-12,
                  time_method=method)
    o = oracle.Oracle(d)
    assert o.unsteady()["dt"] == pytest.approx(dt, rel=1e-12)
    assert o.unsteady()["method"] == method
    WA0 = o.array("WA").copy()
    o.call("timestep"); o.call("reconstruction"); o.call("flux_sourceterm")
    R0 = o.array("hWA").copy()
    o2 = oracle.Oracle(d)
    o2.unsteady_step(1)
    rate = (o2.array("WA") - WA0) * o2.array("VOL")[:, None] / dt
    scale = np.abs(R0).max(axis=0)
    assert np.max(np.abs(rate - R0) / scale) < 1e-3


def test_inner_iterations_stop_at_rel_tol(case_root):
    loose = make_case(case_root, "t2u", rel_tol=0.5, inner_loop=10)
    never = make_case(case_root, "t2u", rel_tol=0.0, inner_loop=4)
    o = oracle.Oracle(loose)
    n_loose = o.unsteady_step(1)[0]
    o = oracle.Oracle(never)
    n_never = o.unsteady_step(1)[0]
    assert 2 <= n_loose < 10
    assert n_never == 4  # RoRes < 0 never holds: the inner loop runs to InnerLoop


def test_last_step_ends_at_totaltime(case_root):
    d = make_case(case_root, "t2u", totaltime=3.0e-8, nstep=3, inner_loop=2)
    o = oracle.Oracle(d)
    stops = [o.unsteady_step(i)[1] for i in (1, 2, 3)]
    assert stops == [False, False, True]
    assert o.unsteady()["ttime"] == pytest.approx(3.0e-8, rel=1e-12)


def test_euler_differs_from_bdf2_only_after_the_first_step(case_root):
    """Step 1 of BDF2 has phi = 0 and WP = WA: the backward Euler step; from
    step 2 on the schemes differ."""
    runs = {}
    for m in (5, 3):
        o = oracle.Oracle(make_case(case_root, "t2u", time_method=m))
        o.unsteady_step(1)
        s1 = o.array("WA").copy()
        o.unsteady_step(2)
        runs[m] = (s1, o.array("WA").copy())
    assert np.array_equal(runs[5][0], runs[3][0])
    assert not np.array_equal(runs[5][1], runs[3][1])
