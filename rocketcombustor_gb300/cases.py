"""Synthetic nozzle cases written in the reference solver's own input formats.

A case directory holds exactly the files the reference reads:

* ``grid1.in`` — cell-based mesh (src/mesh.f90:10-65): header ``NE NE_Vir NNT
  NNT_Vir NF NF_Vir``, one record per cell ``kface n1 n2 n3``, node records ``x y
  0 0``, ``NConE=0``, boundary groups ``itype ibound`` + node pairs, ``NCon=0``;
* ``combustion/{species,thermo,transport,diffusion,chemical_kinetics,oxidizer,
  fuel}.in`` — read by the ``setup_*`` routines of src/combustion_modeling;
* ``flow/flow_solver_info.in`` — solver flags (src/startup.f90:55-128);
* ``fvp1.sav`` — the restart file read by ``Read_Backup`` (src/output.f90:276-338),
  used here to carry the initial field.

Geometry (planar convergent-divergent nozzle, upper half with a symmetry axis):
chamber x in [0, 0.10] with half-height 0.04, cosine contraction to a throat of
half-height 0.01 at x = 0.15, cosine expansion to 0.03 at x = 0.25.  A mapped
nx-by-ny quad grid is split into triangles with alternating diagonals and the
interior nodes are jittered by a seeded uniform +-10 % of the local spacing.

Boundary codes follow src/update_flow_variables.f90:132-260: 2 symmetry (axis),
3 mass-flux inlet (x = 0), 5 outlet (x = 0.25), 6 slip wall or 1 no-slip wall.

Cell order — the order in ``grid1.in`` fixes the Gauss-Seidel recurrence of the
LU-SGS sweeps, for the reference and for this project alike:

* ``"natural"``: columns marching downstream, bottom to top inside a column;
* ``"colored"``: a greedy colouring of the cell adjacency graph (natural order
  inside each colour class), which gives a handful of sweep levels;
* ``"random"``: a seeded permutation.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field, asdict
from typing import Dict, List, Optional, Sequence

import numpy as np

R_UNIVERSAL = 8.31446261815324  # src/combustion/species.in:9

X_CHAMBER, X_THROAT, X_EXIT = 0.10, 0.15, 0.25
H_CHAMBER, H_THROAT, H_EXIT = 0.04, 0.01, 0.03


def half_height(x: np.ndarray, h_exit: float = H_EXIT, x_exit: float = X_EXIT) -> np.ndarray:
    """Nozzle wall y = h(x): flat chamber, cosine contraction and expansion."""
    x = np.asarray(x, dtype=np.float64)
    h = np.full_like(x, H_CHAMBER)
    c = (x > X_CHAMBER) & (x <= X_THROAT)
    t = (x[c] - X_CHAMBER) / (X_THROAT - X_CHAMBER)
    h[c] = H_THROAT + 0.5 * (H_CHAMBER - H_THROAT) * (1.0 + np.cos(np.pi * t))
    e = x > X_THROAT
    t = (x[e] - X_THROAT) / (x_exit - X_THROAT)
    h[e] = H_THROAT + 0.5 * (h_exit - H_THROAT) * (1.0 - np.cos(np.pi * t))
    return h


def area_ratio_mach(ratio, gamma: float, supersonic):
    """Mach number(s) for A/A* = ratio (isentropic), by bisection; `ratio` and
    `supersonic` may be arrays."""
    ratio = np.asarray(ratio, dtype=np.float64)
    sup = np.broadcast_to(np.asarray(supersonic, dtype=bool), ratio.shape)
    g1 = (gamma + 1.0) / (2.0 * (gamma - 1.0))
    lo = np.where(sup, 1.0, 1e-6)
    hi = np.where(sup, 50.0, 1.0)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        f = (1.0 / mid) * ((2.0 / (gamma + 1.0)) * (1.0 + 0.5 * (gamma - 1.0) * mid * mid)) ** g1 - ratio
        go_up = (f > 0) == (~sup)
        lo2 = np.where(go_up, mid, lo)
        hi2 = np.where(go_up, hi, mid)
        # once every bracket is two adjacent doubles, further steps change nothing
        done = np.array_equal(lo2, lo) and np.array_equal(hi2, hi)
        lo, hi = lo2, hi2
        if done:
            break
    m = 0.5 * (lo + hi)
    return float(m) if m.ndim == 0 else m


@dataclass
class Mesh:
    coor: np.ndarray          # (NNT, 2) float64
    cells: np.ndarray         # (NE, 3) or (NE, 4) int64, 1-based node ids, counter-clockwise
    boundaries: List[tuple]   # [(itype, (nb,2) int64 1-based node pairs)]
    nx: int
    ny: int

    @property
    def ne(self) -> int:
        return int(self.cells.shape[0])

    @property
    def nnt(self) -> int:
        return int(self.coor.shape[0])

    @property
    def nf(self) -> int:
        """Number of distinct cell edges."""
        c = self.cells.astype(np.int64)
        k = c.shape[1]
        e = np.concatenate([c[:, [q, (q + 1) % k]] for q in range(k)])
        key = np.minimum(e[:, 0], e[:, 1]) * (self.nnt + 1) + np.maximum(e[:, 0], e[:, 1])
        return int(np.unique(key).shape[0])


def _color_order(cells: np.ndarray, nnt: int) -> np.ndarray:
    """Natural order inside colour classes of a greedy edge-adjacency colouring."""
    ne = cells.shape[0]
    edges = np.concatenate([cells[:, [0, 1]], cells[:, [1, 2]], cells[:, [2, 0]]])
    owner = np.concatenate([np.arange(ne)] * 3)
    key = np.minimum(edges[:, 0], edges[:, 1]).astype(np.int64) * (nnt + 1) + np.maximum(edges[:, 0], edges[:, 1])
    order = np.argsort(key, kind="stable")
    ks, ow = key[order], owner[order]
    same = ks[1:] == ks[:-1]
    a, b = ow[:-1][same], ow[1:][same]
    adj: List[List[int]] = [[] for _ in range(ne)]
    for u, v in zip(a.tolist(), b.tolist()):
        adj[u].append(v)
        adj[v].append(u)
    color = np.full(ne, -1, dtype=np.int64)
    for c in range(ne):
        used = {color[n] for n in adj[c] if color[n] >= 0}
        k = 0
        while k in used:
            k += 1
        color[c] = k
    return np.lexsort((np.arange(ne), color))


def nozzle_mesh(nx: int, ny: int, seed: int, order: str = "natural", wall_type: int = 6,
                jitter: float = 0.10, h_exit: float = H_EXIT, x_exit: float = X_EXIT,
                quads: bool = False) -> Mesh:
    """Seeded nozzle mesh: (nx*ny*2) triangles, or with `quads` the nx*ny
    quadrilaterals of the mapped grid; ordering per `order`."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, x_exit, nx + 1)
    hx = half_height(xs, h_exit, x_exit)
    jj = np.arange(ny + 1) / ny
    X = np.repeat(xs[:, None], ny + 1, axis=1)
    Y = hx[:, None] * jj[None, :]
    dxl = x_exit / nx
    dyl = hx[:, None] / ny * np.ones((1, ny + 1))
    jx = rng.uniform(-jitter, jitter, size=X.shape) * dxl
    jy = rng.uniform(-jitter, jitter, size=X.shape) * dyl
    interior = np.zeros(X.shape, dtype=bool)
    interior[1:-1, 1:-1] = True
    X = np.where(interior, X + jx, X)
    Y = np.where(interior, Y + jy, Y)
    # node id (i, j) -> i*(ny+1) + j + 1
    nid = lambda i, j: i * (ny + 1) + j + 1  # noqa: E731
    coor = np.stack([X.ravel(), Y.ravel()], axis=1)
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    I, J = I.ravel(), J.ravel()
    a, b, c, d = nid(I, J), nid(I + 1, J), nid(I + 1, J + 1), nid(I, J + 1)
    if quads:
        cells = np.stack([a, b, c, d], 1).astype(np.int64)
    else:
        diag_ac = ((I + J) % 2) == 0
        t1 = np.where(diag_ac[:, None], np.stack([a, b, c], 1), np.stack([a, b, d], 1))
        t2 = np.where(diag_ac[:, None], np.stack([a, c, d], 1), np.stack([b, c, d], 1))
        cells = np.stack([t1, t2], axis=1).reshape(-1, 3).astype(np.int64)
    if order == "natural":
        pass
    elif order == "colored":
        cells = cells[_color_order(cells, coor.shape[0])]
    elif order == "random":
        cells = cells[np.random.default_rng(seed + 1000).permutation(cells.shape[0])]
    else:
        raise ValueError(f"unknown cell order {order!r}")
    i_all = np.arange(nx)
    j_all = np.arange(ny)
    axis = np.stack([nid(i_all, 0), nid(i_all + 1, 0)], 1)
    wall = np.stack([nid(i_all + 1, ny), nid(i_all, ny)], 1)
    inlet = np.stack([nid(0, j_all + 1), nid(0, j_all)], 1)
    outlet = np.stack([nid(nx, j_all), nid(nx, j_all + 1)], 1)
    boundaries = [(2, axis), (wall_type, wall), (3, inlet), (5, outlet)]
    return Mesh(coor=coor, cells=cells, boundaries=boundaries, nx=nx, ny=ny)


def _write_rows(f, arr, fmt) -> None:
    """The text np.savetxt(f, arr, fmt) writes (space-separated, one line per
    row, each field through `%`), formatted a chunk of rows at a time."""
    arr = np.asarray(arr)
    if arr.ndim == 1:
        arr = arr[:, None]
    ncol = arr.shape[1]
    row = (" ".join(fmt) if isinstance(fmt, (list, tuple)) else " ".join([fmt] * ncol)) + "\n"
    step = 65536
    for a in range(0, arr.shape[0], step):
        blk = arr[a:a + step]
        f.write((row * blk.shape[0]) % tuple(blk.ravel().tolist()))


def write_grid(path: str, mesh: Mesh) -> None:
    """grid1.in in the layout read by ReadMesh (src/mesh.f90:10-65)."""
    ne, nnt, nf = mesh.ne, mesh.nnt, mesh.nf
    with open(path, "w") as f:
        f.write(f"{ne} {ne} {nnt} {nnt} {nf} {nf}\n")
        cells = np.concatenate([np.full((ne, 1), mesh.cells.shape[1], dtype=np.int64), mesh.cells], axis=1)
        _write_rows(f, cells, "%d")
        cz = np.concatenate([mesh.coor, np.zeros((nnt, 2))], axis=1)
        _write_rows(f, cz, ["%.17g", "%.17g", "%d", "%d"])
        f.write("0\n")  # NConE
        nbmax = max(len(p) for _, p in mesh.boundaries)
        f.write(f"{len(mesh.boundaries)} {nbmax}\n")
        for itype, pairs in mesh.boundaries:
            f.write(f"{itype} {len(pairs)}\n")
            _write_rows(f, pairs, "%d")
        f.write("0\n")  # NCon


# ----------------------------------------------------------------- physics --
@dataclass
class Species:
    names: List[str]
    mole_weight: List[float]


def _fmt(x: float) -> str:
    return repr(float(x))


def write_species(d: str, sp: Species) -> None:
    with open(os.path.join(d, "combustion", "species.in"), "w") as f:
        f.write("# number of species\n")
        f.write(f"{len(sp.names)}\n")
        f.write("# species name, mole weight (kg/mol)\n")
        for n, m in zip(sp.names, sp.mole_weight):
            f.write(f"{n} , {_fmt(m)}\n")
        f.write("# gas constant R (J/mol/K)\n")
        f.write(f"{_fmt(R_UNIVERSAL)}\n")


def write_thermo(d: str, low: np.ndarray, high: np.ndarray, b1: Sequence[float],
                 trange=(200.0, 1000.0, 60000.0)) -> None:
    """thermo.in (thermo_property.f90:18-59); coefficient arrays are (Nsp, 7)."""
    nsp = low.shape[0]
    with open(os.path.join(d, "combustion", "thermo.in"), "w") as f:
        f.write("# reference temperature\n298.15\n# order of Cp polynomial\n7\n")
        f.write("# Cp polynomial coefficients\n")
        f.write(", ".join(_fmt(t) for t in trange) + "\n")
        for i in range(nsp):
            f.write(", ".join(_fmt(v) for v in low[i]) + "\n")
            f.write(_fmt(b1[i]) + "\n")
            f.write(", ".join(_fmt(v) for v in high[i]) + "\n")
            f.write(_fmt(b1[i]) + "\n")
        f.write("# heat of formation (J/mol) unused?\n")
        for i in range(nsp):
            f.write("0\n")


# Shipped property data of the H2/O2/H2O/Ar mixture (src/combustion/*.in).
H2O2_SPECIES = Species(["H2", "O2", "H2O", "Ar"], [2.0e-3, 32.0e-3, 18.0e-3, 40.0e-3])
H2O2_TRANSPORT = [
    [0.57388074E0, -0.98544160E2, 0.20012204E4, 0.17536015E1],
    [0.65074534E0, 0.23936771E2, -0.22020183E5, 0.11244058E1],
    [0.11770360E1, -0.17422121E3, 0.22865563E5, -0.55146852E0],
    [0.49214767E0, -0.91598343E3, 0.87265127E5, 0.48489412E1],
    [0.61936357E0, -0.44608607E2, -0.13460714E4, 0.19597562E1],
    [0.63839563E0, -0.12344438E1, -0.22885810E5, 0.18056937E1],
    [0.81595343E0, -0.34366856E2, 0.22785080E4, 0.10050999E1],
    [0.80805788E0, 0.11982181E3, -0.47335931E5, 0.95189193E0],
    [0.54330318E0, -0.18823898E3, 0.88726567E4, 0.24499362E1],
    [0.65318879E0, 0.51738759E2, -0.62834882E5, 0.15227045E1],
    [0.53726173E0, -0.49928331E3, 0.37397504E5, 0.32903619E1],
    [0.66068182E0, -0.12741845E3, -0.81580328E5, 0.21817907E1],
    [0.78387780E0, -0.38260408E3, 0.49040158E5, 0.85222785E0],
    [0.50714993E0, -0.68966913E3, 0.87454750E5, 0.30285155E1],
    [0.15541443E1, 0.66106305E2, 0.55969886E4, -0.39259598E1],
    [0.79349503E0, -0.13340063E4, 0.37864327E6, 0.23591474E1],
]
H2O2_DIFFUSION = [(3.758, 148.6), (3.467, 106.7), (3.941, 195.2), (2.641, 809.1)]
# 2 H2 + O2 -> 2 H2O; global rate constants (chemical_kinetics.in:4-9)
H2O2_STOICH = [(2.0, 0.0), (1.0, 0.0), (0.0, 2.0), (0.0, 0.0)]
H2O2_RATE = (2.12e11, 0.0, 2.025e5)
H2O_HOF_J_PER_MOL = -241826.0  # thermo.in:16,18


def write_transport(d: str, rows: List[List[float]]) -> None:
    with open(os.path.join(d, "combustion", "transport.in"), "w") as f:
        f.write("# transport_lowest_tem,transport_critical_tem,transport_highest_tem\n")
        f.write("200.0, 1000.0, 50000.0\n# low_mu_A,low_mu_B,low_mu_C,low_mu_D\n")
        for r in rows:
            f.write(", ".join(_fmt(v) for v in r) + "\n")


def write_diffusion(d: str, pairs) -> None:
    with open(os.path.join(d, "combustion", "diffusion.in"), "w") as f:
        f.write("# Boltzmann's constant k_B (m2*kg*s-2*K-1)\n1.38064852E-23\n")
        f.write("# hard-sphere collision diameter sigma (A), Lennard-Jones energy epsilon/k_B (K)\n")
        for s, e in pairs:
            f.write(f"{_fmt(s)}, {_fmt(e)}\n")


def write_kinetics(d: str, stoich, rate, model: int) -> None:
    with open(os.path.join(d, "combustion", "chemical_kinetics.in"), "w") as f:
        f.write("# number of reactions\n")
        f.write(f"1, {model}\n")
        f.write("# forwar reaction coefficient, reverse reaction coefficient\n")
        for a, b in stoich:
            f.write(f"{_fmt(a)}, {_fmt(b)}\n")
        f.write("# pre-exponential factor, temperature exponent, activation energy (J)\n")
        f.write(", ".join(_fmt(v) for v in rate) + "\n")
        f.write("# entropy change, enthalpy change unused?\n0., 0.\n# p_a\n1.0e5\n")


def write_inlet(path: str, Y: Sequence[float], T: float, p: float, mflow: float, what: str) -> None:
    with open(path, "w") as f:
        f.write(f"# {what} mass fraction\n")
        for y in Y:
            f.write(_fmt(y) + "\n")
        f.write("# temperature (K), pressure (K)\n")
        f.write(f"{_fmt(T)}, {_fmt(p)}\n# mass flow rate (kg/s)\n{_fmt(mflow)}\n")


def write_flow_info(d: str, combustion: bool, viscous: bool, cfl: float, nstep: int,
                    limit_id: int, p_out_ratio: float, unsteady: bool = False, totaltime: float = 1.0,
                    inner_loop: int = 1, rel_tol: float = 1.0e-8, a_p: float = 0.0, f_p: float = 5000.0,
                    time_method: int = 5) -> None:
    """flow/flow_solver_info.in (startup.f90:55-128).  Steady implicit LU-SGS,
    or with `unsteady` a dual-time scheme (implicit_time_method `time_method`:
    5 BDF2, 3 backward Euler;
    physical step totaltime/nstep, inner_loop inner iterations stopped at
    rel_tol, exit pressure p_static (1 + a_p sin(2 pi f_p t)))."""
    L = lambda b: ".true." if b else ".false."  # noqa: E731
    with open(os.path.join(d, "flow", "flow_solver_info.in"), "w") as f:
        f.write(f"# If_turn_on_combustion, chemical model\n{L(combustion)}\n")
        f.write("# IfRightDomain\n.false.\n# NPreviousPar\n1\n# Npar, number of processors\n1\n")
        f.write("# unit\n1.0\n")
        f.write(f"# IfSteady, IfViscous, IfReadBackup, IfExplicit\n{L(not unsteady)}, {L(viscous)}, .true., .false.\n")
        f.write("# implicit_time_method: 1-> Implicit Runge-Kutta, 2-> Trapezoidal, 3-> Euler, 4-> Midpoint, 5-> BDF2\n"
                f"{time_method}\n")
        f.write(f"# cfl,totaltime,nstep_max,save_start_time, save_end_time\n{_fmt(cfl)}, {_fmt(totaltime)}, {nstep}, 0.0, 0.5\n")
        f.write(f"# IfFixDt\n.false.\n# InLoop, InnerLoop, relTol\n1, {inner_loop}, {_fmt(rel_tol)}\n")
        f.write("# NScreenOutput,NFileOutput,NFileBackup,NWriteMonitor\n100,100000,100000,100000\n")
        f.write(f"# rc_detector\n3.0\n# n_wbap,limit_ID: 0-> no limiter, 1-> WBAP, 2-> WBAP_Char\n10, {limit_id}\n")
        f.write("# number of monitor points\n1\n# x_monitor_point, y_monitor_point\n0,0\n")
        f.write(f"# exit pressure ratio, A_p, f_p\n{_fmt(p_out_ratio)}, {_fmt(a_p)}, {_fmt(f_p)}\n")


def write_backup(path: str, mesh: Mesh, PA: np.ndarray) -> None:
    """fvp1.sav (output.f90:256-273): ttime, NE, then x y PA(1:NVar) per cell."""
    cxy = mesh.coor[mesh.cells - 1].mean(axis=1)
    with open(path, "w") as f:
        f.write("0.0\n")
        f.write(f"{mesh.ne}\n")
        _write_rows(f, np.concatenate([cxy, PA], axis=1), "%.17g")


# --------------------------------------------------------------- configs ---
@dataclass
class CaseConfig:
    """One synthetic nozzle case; `name` keys the presets below."""
    name: str
    nx: int
    ny: int
    seed: int
    order: str = "natural"
    nsp: int = 1
    viscous: bool = False
    combustion: bool = False
    p0: float = 2.0e6
    T0: float = 3000.0
    cfl: float = 5.0
    nstep: int = 2000
    limit_id: int = 1
    thermo_seed: int = 3
    perturb_seed: int = 4
    perturb: float = 0.0
    chem_model: int = 0
    of_ratio: float = 6.0
    inlet_burnt: float = 0.99  # fraction of the O2 already converted at the inlet
    closed: bool = False       # every boundary a wall, fluid initially at rest (test case)
    p_out_factor: float = 1.0  # exit pressure as a multiple of the isentropic design exit pressure
    jitter: float = 0.10       # interior node jitter, fraction of the local spacing
    init: str = "uniform"      # initial field: "uniform" inlet state or "isentropic" quasi-1D nozzle flow
    h_exit: float = H_EXIT     # exit half-height (area ratio h_exit / 0.01)
    wall: int = 0              # wall BC code: 0 = no-slip (1) when viscous, else slip (6)
    x_exit: float = X_EXIT     # exit station (divergent length x_exit - 0.15)
    # unsteady dual-time BDF2 (implicit_time_method 5) instead of steady LU-SGS:
    # nstep physical steps of totaltime/nstep, inner_loop inner iterations
    unsteady: bool = False
    totaltime: float = 1.0
    inner_loop: int = 1
    rel_tol: float = 1.0e-8
    a_p: float = 0.0           # exit-pressure oscillation amplitude (fraction of p_static)
    f_p: float = 5000.0        # and frequency (Hz)
    time_method: int = 5       # implicit_time_method: 5 BDF2, 3 backward Euler
    # subsonic nozzle: the throat Mach number of a nozzle flow that stays
    # subsonic (inlet mass flux, initial field and exit pressure from the
    # subsonic isentropic branch through the throat at this Mach number);
    # 0 = the choked design (sonic throat, supersonic divergent section)
    throat_mach: float = 0.0
    quads: bool = False        # quadrilateral cells of the mapped grid instead of its triangles

    @property
    def n_cells(self) -> int:
        return (1 if self.quads else 2) * self.nx * self.ny


PRESETS: Dict[str, CaseConfig] = {
    # small inviscid perfect-gas nozzle (about 20k triangles)
    "c1": CaseConfig("c1", nx=250, ny=40, seed=1),
    # reacting viscous nozzle (about 120k triangles)
    "c2": CaseConfig("c2", nx=600, ny=100, seed=2, nsp=4, viscous=True, combustion=True,
                     p0=5.0e6, T0=3500.0, perturb=0.02, init="isentropic"),
    # large reacting viscous nozzle (2M triangles)
    "c4": CaseConfig("c4", nx=2500, ny=400, seed=6, nsp=4, viscous=True, combustion=True,
                     p0=5.0e6, T0=3500.0, perturb=0.02, nstep=500, init="isentropic"),
    # tiny cases for tests
    "t1": CaseConfig("t1", nx=24, ny=6, seed=11),
    "t2": CaseConfig("t2", nx=24, ny=6, seed=12, nsp=4, viscous=True, combustion=True,
                     p0=5.0e6, T0=3500.0, perturb=0.02, init="isentropic"),
    # the shipped configuration's time scheme (flow_solver_info.in: BDF2, CFL 10,
    # dt = 5e-3 / 500000 = 1e-8 s, 10 inner iterations to 1e-3) on the tiny and
    # the 120k-cell reacting nozzles
    "t2u": CaseConfig("t2u", nx=24, ny=6, seed=12, nsp=4, viscous=True, combustion=True,
                      p0=5.0e6, T0=3500.0, perturb=0.02, init="isentropic", unsteady=True, cfl=10.0,
                      totaltime=5.0e-3, nstep=500000, inner_loop=10, rel_tol=1.0e-3),
    # steady-state cases: the reacting viscous nozzle on quadrilaterals with a
    # 1500 K chamber (same mechanism, 99 % burnt inlet).  On triangles the
    # reference's face-neighbour least-squares reconstruction makes entropy
    # modes grow (the Barth limiter then holds the residual in a limit cycle)
    # and the explicit rate at 3500 K with O2 nearly used up cycles at the
    # Y = 0 clip; these converge to 1e-8 and below
    "s2": CaseConfig("s2", nx=120, ny=24, seed=21, nsp=4, viscous=True, combustion=True,
                     p0=5.0e6, T0=1500.0, perturb=0.02, init="isentropic", quads=True, nstep=12000),
    "s2t": CaseConfig("s2t", nx=60, ny=12, seed=22, nsp=4, viscous=True, combustion=True,
                      p0=5.0e6, T0=1500.0, perturb=0.02, init="isentropic", quads=True, nstep=8000),
    "c2u": CaseConfig("c2u", nx=600, ny=100, seed=2, nsp=4, viscous=True, combustion=True,
                      p0=5.0e6, T0=3500.0, perturb=0.02, init="isentropic", unsteady=True, cfl=10.0,
                      totaltime=5.0e-3, nstep=500000, inner_loop=10, rel_tol=1.0e-3),
}


def synthetic_cp(nsp: int, seed: int) -> np.ndarray:
    """Seeded smooth cp/R = a3 + a4 T + a5 T^2, rising from a3 in [3.5, 3.7] at
    T -> 0 to a maximum in [4.2, 4.5] at 4000 K (coefficient slots 3..5 of the
    7-term polynomial, thermo_property.f90:84-96)."""
    rng = np.random.default_rng(seed)
    coef = np.zeros((nsp, 7))
    for i in range(nsp):
        a3 = rng.uniform(3.5, 3.7)
        top = rng.uniform(4.2, 4.5)
        a5 = (a3 - top) / 16.0e6
        coef[i, 2] = a3
        coef[i, 3] = -8000.0 * a5
        coef[i, 4] = a5
    return coef


def sonic_height(cfg: CaseConfig, gamma: float) -> float:
    """Half-height of the isentropic flow's sonic section: the throat for the
    choked design, below it (A* = A_throat / (A/A*)(M_throat)) for a subsonic
    nozzle."""
    if cfg.throat_mach <= 0.0:
        return H_THROAT
    m = cfg.throat_mach
    g1 = (gamma + 1.0) / (2.0 * (gamma - 1.0))
    ar = (1.0 / m) * ((2.0 / (gamma + 1.0)) * (1.0 + 0.5 * (gamma - 1.0) * m * m)) ** g1
    return H_THROAT / ar


def inlet_state(cfg: CaseConfig, R: float, gamma: float):
    """Static inlet state of the subsonic chamber for total (p0, T0) at the
    chamber-to-sonic area ratio: returns (p, T, u, mass flux)."""
    M = area_ratio_mach(H_CHAMBER / sonic_height(cfg, gamma), gamma, supersonic=False)
    T = cfg.T0 / (1.0 + 0.5 * (gamma - 1.0) * M * M)
    p = cfg.p0 * (T / cfg.T0) ** (gamma / (gamma - 1.0))
    rho = p / (R * T)
    u = M * math.sqrt(gamma * R * T)
    return p, T, u, rho * u


def exit_pressure_ratio(gamma: float, h_exit: float = H_EXIT) -> float:
    M = area_ratio_mach(h_exit / H_THROAT, gamma, supersonic=True)
    return (1.0 + 0.5 * (gamma - 1.0) * M * M) ** (-gamma / (gamma - 1.0))


def write_case(d: str, cfg: CaseConfig, mesh: Optional[Mesh] = None) -> Mesh:
    """Write a complete case directory for `cfg`; returns the mesh."""
    os.makedirs(os.path.join(d, "combustion"), exist_ok=True)
    os.makedirs(os.path.join(d, "flow"), exist_ok=True)
    if mesh is None:
        wall = cfg.wall or (1 if cfg.viscous else 6)
        mesh = nozzle_mesh(cfg.nx, cfg.ny, cfg.seed, cfg.order, wall_type=wall, jitter=cfg.jitter,
                           h_exit=cfg.h_exit, x_exit=cfg.x_exit, quads=cfg.quads)
    if cfg.closed:
        wall = cfg.wall or (1 if cfg.viscous else 6)
        mesh.boundaries = [(wall, pairs) for _, pairs in mesh.boundaries]
    write_grid(os.path.join(d, "grid1.in"), mesh)
    if cfg.nsp == 1:
        # single calorically perfect gas, gamma = 1.4, R = 287
        sp = Species(["AIR"], [R_UNIVERSAL / 287.0])
        low = np.zeros((1, 7)); low[0, 2] = 3.5
        write_species(d, sp)
        write_thermo(d, low, low, [0.0])
        write_transport(d, H2O2_TRANSPORT[0:4])
        write_diffusion(d, H2O2_DIFFUSION[0:1])
        write_kinetics(d, [(0.0, 0.0)], H2O2_RATE, cfg.chem_model)
        Yin = [1.0]
        Rmix = R_UNIVERSAL / sp.mole_weight[0]
        gamma = 1.4
    else:
        sp = H2O2_SPECIES
        coef = synthetic_cp(4, cfg.thermo_seed)
        # b1 in kelvin: the formula R_k (T sum a_j basis_j + b1) expects it; the
        # shipped value in J/mol is divided by R.
        b1 = [0.0, 0.0, H2O_HOF_J_PER_MOL / R_UNIVERSAL, 0.0]
        write_species(d, sp)
        write_thermo(d, coef, coef, b1)
        write_transport(d, H2O2_TRANSPORT)
        write_diffusion(d, H2O2_DIFFUSION)
        write_kinetics(d, H2O2_STOICH, H2O2_RATE, cfg.chem_model)
        # propellant O/F by mass, with a fraction of the O2 already converted
        y_h2, y_o2 = 1.0 / (1.0 + cfg.of_ratio), cfg.of_ratio / (1.0 + cfg.of_ratio)
        burnt = cfg.inlet_burnt * y_o2
        Yin = [y_h2 - burnt * (4.0 / 32.0), y_o2 - burnt, burnt * (36.0 / 32.0), 0.0]
        Rs = [R_UNIVERSAL / m for m in sp.mole_weight]
        Rmix = sum(y * r for y, r in zip(Yin, Rs))
        cpm = sum(y * r * (coef[i, 2] + coef[i, 3] * cfg.T0 + coef[i, 4] * cfg.T0 ** 2)
                  for i, (y, r) in enumerate(zip(Yin, Rs)))
        gamma = cpm / (cpm - Rmix)
    p_in, T_in, u_in, mflux = inlet_state(cfg, Rmix, gamma)
    # oxidizer inlet carries the chamber mixture; the reference divides the .in
    # mass flow by the measured inlet diameter 2*(ymax-ymin) (initialization.f90:22)
    write_inlet(os.path.join(d, "combustion", "oxidizer.in"), Yin, T_in, cfg.p0,
                mflux * 2.0 * H_CHAMBER, "oxidizer")
    write_inlet(os.path.join(d, "combustion", "fuel.in"), Yin, T_in, cfg.p0, 0.37, "fuel")
    if cfg.throat_mach > 0.0:
        m_e = area_ratio_mach(cfg.h_exit / sonic_height(cfg, gamma), gamma, supersonic=False)
        pr = (1.0 + 0.5 * (gamma - 1.0) * m_e * m_e) ** (-gamma / (gamma - 1.0)) * cfg.p_out_factor
    else:
        pr = exit_pressure_ratio(gamma, cfg.h_exit) * cfg.p_out_factor
    write_flow_info(d, cfg.combustion, cfg.viscous, cfg.cfl, cfg.nstep, cfg.limit_id, pr, cfg.unsteady,
                    cfg.totaltime, cfg.inner_loop, cfg.rel_tol, cfg.a_p, cfg.f_p, cfg.time_method)
    # initial field: uniform inlet (chamber) state, or the quasi-1D isentropic
    # nozzle flow (subsonic up to the throat, supersonic after it) with the
    # velocity tilted along y/h * dh/dx; species optionally perturbed
    nv = 4 + len(Yin) - 1
    PA = np.zeros((mesh.ne, nv))
    PA[:, 0], PA[:, 1], PA[:, 2], PA[:, 3] = p_in, (0.0 if cfg.closed else u_in), 0.0, T_in
    if cfg.init == "isentropic" and not cfg.closed:
        cxy = mesh.coor[mesh.cells - 1].mean(axis=1)
        x, y = cxy[:, 0], cxy[:, 1]
        h = half_height(x, cfg.h_exit, cfg.x_exit)
        eps = 1e-6
        dh = (half_height(x + eps, cfg.h_exit, cfg.x_exit) - half_height(x - eps, cfg.h_exit, cfg.x_exit)) / (2 * eps)
        hs = sonic_height(cfg, gamma)
        M = area_ratio_mach(np.maximum(h / hs, 1.0 + 1e-9), gamma,
                            supersonic=(x > X_THROAT) & (cfg.throat_mach <= 0.0))
        T = cfg.T0 / (1.0 + 0.5 * (gamma - 1.0) * M * M)
        p = cfg.p0 * (T / cfg.T0) ** (gamma / (gamma - 1.0))
        q = M * np.sqrt(gamma * Rmix * T)
        slope = y / h * dh
        PA[:, 0], PA[:, 3] = p, T
        PA[:, 1] = q / np.sqrt(1.0 + slope * slope)
        PA[:, 2] = PA[:, 1] * slope
    elif cfg.init != "uniform" and not cfg.closed:
        raise ValueError(f"unknown init {cfg.init!r}")
    if len(Yin) > 1:
        Y = np.tile(np.asarray(Yin), (mesh.ne, 1))
        if cfg.perturb > 0:
            rng = np.random.default_rng(cfg.perturb_seed)
            Y = Y * (1.0 + rng.uniform(-cfg.perturb, cfg.perturb, size=Y.shape))
            Y = Y / Y.sum(axis=1, keepdims=True)
        PA[:, 4:] = Y[:, :-1]
    write_backup(os.path.join(d, "fvp1.sav"), mesh, PA)
    with open(os.path.join(d, "case.json"), "w") as f:
        import json
        json.dump(asdict(cfg), f, indent=1)
    return mesh


def make_case(d: str, name: str, **over) -> CaseConfig:
    """Write preset `name` (with field overrides) into directory `d`."""
    cfg = CaseConfig(**{**asdict(PRESETS[name]), **over})
    write_case(d, cfg)
    return cfg


def _area_ratio(u: float, lo: float, hi: float) -> float:
    """A draw u from [4, 25] mapped onto [lo, hi] (u itself for the default range)."""
    if (lo, hi) == (4.0, 25.0):
        return u
    return lo + (u - 4.0) / 21.0 * (hi - lo)


def batch_configs(n: int = 64, seed: int = 5, ne_min: int = 2000, ne_max: int = 60000,
                  ar_min: float = 4.0, ar_max: float = 25.0, **over) -> List[CaseConfig]:
    """n independent reacting viscous nozzle cases of uneven size (the batched
    workload): cells log-uniform in [ne_min, ne_max] (nx = 6 ny), chamber
    pressure uniform in 1-10 MPa, O/F uniform in 4-8 and area ratio uniform in
    4-25 through the exit half-height, with the divergent section lengthened
    in proportion so that the wall keeps the base nozzle's steepest slope; the
    physics of preset c2 otherwise."""
    rng = np.random.default_rng(seed)
    base = asdict(PRESETS["c2"])
    per_quad = 1 if over.get("quads") else 2  # cells per quadrilateral of the mapped grid
    out = []
    for c in range(n):
        ne = math.exp(rng.uniform(math.log(ne_min), math.log(ne_max)))
        ny = max(4, int(round(math.sqrt(ne / (6.0 * per_quad)))))
        cfg = {**base, "name": f"b{c:02d}", "nx": 6 * ny, "ny": ny, "seed": seed * 1000 + c,
               "p0": float(rng.uniform(1.0e6, 1.0e7)), "of_ratio": float(rng.uniform(4.0, 8.0)),
               "h_exit": _area_ratio(float(rng.uniform(4.0, 25.0)), ar_min, ar_max) * H_THROAT,
               "perturb_seed": seed * 1000 + 500 + c}
        cfg["x_exit"] = X_THROAT + (X_EXIT - X_THROAT) * (cfg["h_exit"] - H_THROAT) / (H_EXIT - H_THROAT)
        cfg.update(over)
        out.append(CaseConfig(**cfg))
    return out


def steady_batch_configs(n: int = 16, seed: int = 8) -> List[CaseConfig]:
    """The batched steady-state workload: n cases of the batch_configs spread
    (1-10 MPa, O/F 4-8) with area ratios 4-12 at 500-5000 cells each, on
    quadrilaterals with the 1500 K chamber of preset s2."""
    return batch_configs(n, seed, ne_min=500, ne_max=5000, ar_min=4.0, ar_max=12.0, quads=True, T0=1500.0,
                         nstep=12000)


def make_batch(d: str, n: int = 64, seed: int = 5, **over) -> List[str]:
    """Write the batch of `batch_configs` as d/bNN case directories."""
    dirs = []
    for cfg in batch_configs(n, seed, **over):
        cd = os.path.join(d, cfg.name)
        write_case(cd, cfg)
        dirs.append(cd)
    return dirs
