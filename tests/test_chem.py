"""Chemistry integrator (new; the reference has none) and the reference
Jacobians it is built on, on the CPU oracle.

Compute_Con_to_Pri_Jaco (Con_to_Pri_Jacobian.f90:1-87) and
compute_derivative_production_rate (chemical_kinetics.f90:167-265) are
checked against central differences of the functions they differentiate; the
integrator against its invariants (rho, e, element balance), a fine-tolerance
run and the explicit rate at small dt.
"""
import numpy as np
import pytest

import oracle
from conftest import make_case


@pytest.fixture(scope="module")
def orc(case_root):
    return oracle.Oracle(make_case(case_root, "t2"), threads=2)


def states(o, n, seed):
    """Seeded near-burnt H2/O2/H2O/Ar states: T 1500-3800 K, p 0.05-10 MPa."""
    rng = np.random.default_rng(seed)
    P = np.zeros((n, o.NVar))
    P[:, 0] = 10 ** rng.uniform(np.log10(5e4), 7, n)
    P[:, 1] = rng.uniform(-200, 2000, n)
    P[:, 2] = rng.uniform(-100, 100, n)
    P[:, 3] = rng.uniform(1500, 3800, n)
    P[:, 4] = rng.uniform(0, 0.05, n)
    P[:, 5] = rng.uniform(0, 0.05, n)
    P[:, 6] = 1 - P[:, 4] - P[:, 5] - rng.uniform(0, 0.02, n)
    return P


def prim_to_con(o, P):
    Y = np.append(P[4:], 1 - P[4:].sum())
    _, _, R = o.gas(Y, P[3])
    r = P[0] / (R * P[3])
    h = (Y * o.enthalpy(P[3])).sum()
    return np.array([r, r * P[1], r * P[2], r * (h + 0.5 * (P[1] ** 2 + P[2] ** 2)) - P[0], *(r * P[4:])])


def omega(o, P):
    Y = np.append(P[4:], 1 - P[4:].sum())
    _, _, R = o.gas(Y, P[3])
    return o.production(P[3], P[0] / (R * P[3]), Y)[:o.Nsp - 1]


def central(f, P, c):
    h = 1e-6 * max(abs(P[c]), 1e-3)
    e = np.zeros_like(P)
    e[c] = h
    return (f(P + e) - f(P - e)) / (2 * h)


def test_jacobians_match_central_differences(orc):
    for P in states(orc, 6, 11):
        J = orc.con_to_pri_jaco(P)
        Jfd = np.stack([central(lambda x: prim_to_con(orc, x), P, c) for c in range(orc.NVar)], axis=1)
        assert np.abs(J - Jfd).max() <= 1e-6 * np.abs(J).max()
        D = orc.dwdp(P)
        Dfd = np.stack([central(lambda x: omega(orc, x), P, c) for c in range(orc.NVar)], axis=1)
        assert np.abs(D - Dfd).max() <= 1e-5 * np.abs(D).max()


def test_integrator_invariants(orc):
    P = states(orc, 64, 12)
    dt = 10 ** np.random.default_rng(13).uniform(-9, -5, len(P))
    out, nsub = orc.chem_integrate(P, dt)
    assert nsub.min() >= 1 and nsub.max() <= 200
    for a, b in zip(P, out):
        ca, cb = prim_to_con(orc, a), prim_to_con(orc, b)
        np.testing.assert_allclose(cb[:4], ca[:4], rtol=1e-10, atol=1e-9 * abs(ca[3]))  # rho, rho u, rho v, rho E
        assert np.all(np.isfinite(b))
        dY = b[4:] - a[4:]
        # the one global reaction moves Y along its stoichiometric direction
        # (element balance), and only forward: reactants never increase
        w = omega(orc, a)
        if np.abs(w).max() > 0:
            u = w / np.linalg.norm(w)
            assert np.linalg.norm(dY - (dY @ u) * u) <= 1e-10 * max(np.linalg.norm(dY), 1e-300)
            assert dY @ u >= -1e-15


def test_integrator_converges_with_tolerance(orc):
    P = states(orc, 24, 14)
    P[:, 3] = np.linspace(2500, 3700, len(P))
    dt = np.full(len(P), 1e-6)
    ref, nref = orc.chem_integrate(P, dt, tol=1e-3, maxsub=100000)
    errs = []
    for tol in (0.2, 0.05, 0.0125):
        out, _ = orc.chem_integrate(P, dt, tol=tol, maxsub=100000)
        errs.append(np.abs(out[:, 4:] - ref[:, 4:]).max())
    assert errs[0] > errs[1] > errs[2]
    assert errs[1] <= 5e-4


def test_integrator_small_dt_is_the_explicit_rate(orc):
    for P in states(orc, 8, 15):
        Y = np.append(P[4:], 1 - P[4:].sum())
        _, _, R = orc.gas(Y, P[3])
        rho = P[0] / (R * P[3])
        dt = 1e-12
        out, nsub = orc.chem_integrate(P, dt)
        rate = rho * (out[0, 4:] - P[4:]) / dt
        w = omega(orc, P)
        assert nsub[0] == 1
        np.testing.assert_allclose(rate, w, rtol=1e-3, atol=1e-6 * np.abs(w).max() + 1e-30)


def test_integrated_source_mode_runs(case_root):
    d = make_case(case_root, "t2")
    a = oracle.Oracle(d, threads=2)
    b = oracle.Oracle(d, threads=2)
    b.set_chemistry(1)
    a.run(5)
    b.run(5)
    nsub = b.chem_nsub()
    assert nsub is not None and nsub.min() >= 1
    pa, pb = a.array("PA"), b.array("PA")
    assert np.all(np.isfinite(pb))
    # same physics, another discretisation of the source
    assert not np.array_equal(pa, pb)
    assert pb[:, 3].min() > 200 and pb[:, 3].max() < 6000


def test_batch_configs_span_the_stated_ranges():
    from rocketcombustor_gb300 import cases
    cs = cases.batch_configs()
    ne = np.array([c.n_cells for c in cs])
    assert len(cs) == 64 and ne.min() >= 1800 and ne.max() <= 62000 and ne.max() > 10 * ne.min()
    p0 = np.array([c.p0 for c in cs]); of = np.array([c.of_ratio for c in cs])
    ar = np.array([c.h_exit / 0.01 for c in cs])
    assert p0.min() >= 1e6 and p0.max() <= 1e7 and of.min() >= 4 and of.max() <= 8
    assert ar.min() >= 4 and ar.max() <= 25
