"""Why the triangle cases stall and the quadrilateral ones converge (oracle, no GPU).

The reference reconstructs with a weighted least-squares gradient over the
face neighbours (gradient.f90:4-45, reconstruction_initialization.f90:90-146)
and adds Rusanov dissipation on the reconstructed states (flux_lax.f90:17-278).
Linearised about a gas at rest, that operator has eigenvalues with positive
real part on the triangulated mesh (density/entropy modes at constant
pressure grow) and none on the quadrilaterals of the same mapped grid.  With
limit_ID = 0 the triangle case therefore blows up, and the Barth limiter
(limiter.f90:5-107) only bounds the growth, which leaves the residual in a
limit cycle.  The steady presets therefore use quadrilaterals, and there the
reference scheme, Barth limiter included, reaches max_k Res_k/Res_k(1) <= 1e-8.
"""
import numpy as np
import pytest

import oracle
from conftest import make_case

R_AIR = 287.0
CV_AIR = 2.5 * R_AIR


def semi_discrete_jacobian(o):
    """d(hWA/vol)/dW by central differences through timestep, reconstruction
    and flux_sourceterm, for the one-species perfect gas (cp = 3.5 R)."""
    PA = o.array("PA")
    NE, V = PA.shape
    vol = o.array("VOL").copy()
    P0 = PA.copy()

    def w_of_p(P):
        rho = P[:, 0] / (R_AIR * P[:, 3])
        u, v = P[:, 1], P[:, 2]
        return np.stack([rho, rho * u, rho * v, rho * (CV_AIR * P[:, 3] + 0.5 * (u * u + v * v))], 1)

    def p_of_w(W):
        rho = W[:, 0]
        u, v = W[:, 1] / rho, W[:, 2] / rho
        T = (W[:, 3] / rho - 0.5 * (u * u + v * v)) / CV_AIR
        return np.stack([rho * R_AIR * T, u, v, T], 1)

    def rhs(W):
        PA[:] = p_of_w(W)
        for sub in ("timestep", "reconstruction", "flux_sourceterm"):
            assert o.call(sub) == 0
        return o.array("hWA").copy() / vol[:, None]

    W0 = w_of_p(P0)
    scale = np.abs(W0).max(axis=0)
    scale[1:3] = W0[:, 0].max() * 100.0
    n = NE * V
    J = np.zeros((n, n))
    for col in range(n):
        i, k = divmod(col, V)
        h = 1e-7 * scale[k]
        W = W0.copy()
        W[i, k] += h
        rp = rhs(W)
        W[i, k] -= 2 * h
        rm = rhs(W)
        J[:, col] = ((rp - rm) / (2 * h)).ravel()
    PA[:] = P0
    return J


@pytest.mark.parametrize("quads", [False, True])
def test_unlimited_operator_growth_on_triangles_only(case_root, quads):
    d = make_case(case_root, "t1", nx=12, ny=4 if not quads else 8, jitter=0.0, closed=True, limit_id=0,
                  quads=quads)
    o = oracle.Oracle(d, threads=4)
    ev = np.linalg.eigvals(semi_discrete_jacobian(o))
    rel = ev.real.max() / np.abs(ev).max()
    if quads:
        assert rel < 1e-8, rel
    else:
        assert rel > 0.05, rel
    o.close()


def test_steady_preset_reaches_1e8_on_the_oracle(case_root):
    """The 720-cell reacting viscous nozzle on quadrilaterals (1500 K
    chamber, the reference's Barth limiter and explicit source)."""
    d = make_case(case_root, "s2t")
    o = oracle.Oracle(d, threads=oracle.Oracle.max_threads())
    h = o.run(8000, history=True)
    r = h[:, :-1]
    m = r[0] > 0
    lv = np.where(m, r / np.where(m, r[0], 1.0), 0.0).max(axis=1)
    hit = np.nonzero(lv <= 1e-8)[0]
    assert hit.size and hit[0] < 8000 and lv[-1] <= 1e-8, lv[::1000]
    o.close()
