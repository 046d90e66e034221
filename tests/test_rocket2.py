"""The reference's own combustor mesh (inv-nozzle-no-BL-rocket/rocket2.msh,
82,898 triangles; fixture tests/golden/rocket2_mesh.npz made by
tests/golden/make_rocket2.py) through the reader, the set-up and the solvers.

The CPU test checks the set-up against the reference's runtime invariants:
XYH below 1e-8 in every cell (reconstruction_initialization.f90:83-86),
neighbours + ghosts = faces (ghostcell.f90:163), one ghost per boundary face,
the face count of the file, and the LU-SGS level depth of the file's element
order (156 forward, 156 backward); the host set-up and the oracle agree bit
for bit.  The GPU test runs 20 FP64 iterations against the oracle.
"""
import os
import sys

import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from rocketcombustor_gb300 import cases

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_rocket2  # noqa: E402

SETUP = ["KFace", "Neighbor", "FNode", "NeighF", "Neigh", "NeighC", "Ghostcell", "Num_ghostcell", "Hostcell",
         "BCtype_Ghostcell", "COOR", "VECX", "VOL", "CELLXY", "reflen", "wdis", "AMLS", "XYH", "PA", "WA"]


@pytest.fixture(scope="module")
def rocket2_dir(tmp_path_factory):
    """The mesh with the reacting viscous physics of the nozzle cases (4
    species, model 0, the 99 % burnt inlet mixture), started from the uniform
    inlet state (the reference's zone initialiser assumes its own cell
    layout)."""
    d = str(tmp_path_factory.mktemp("rocket2") / "case")
    cfg = cases.CaseConfig("rocket2", nx=0, ny=0, seed=0, nsp=4, viscous=True, combustion=True, p0=5.0e6,
                           T0=3500.0, init="uniform")
    cases.write_case(d, cfg, mesh=make_rocket2.load_mesh())
    return d


def test_rocket2_setup_invariants(rocket2_dir):
    m = make_rocket2.load_mesh()
    nb = sum(len(p) for _, p in m.boundaries)
    assert m.cells.shape == (82898, 3) and m.coor.shape == (42194, 2)
    assert sorted(c for c, _ in m.boundaries) == [1, 2, 3, 4, 5, 6]
    o = oracle.Oracle(rocket2_dir, threads=oracle.Oracle.max_threads())
    c = rc.Case(rocket2_dir)
    assert (o.NE, o.NF, o.Nghost) == (82898, 125091, nb)
    assert (o.nlev_fwd, o.nlev_bwd) == (156, 156)
    assert np.abs(o.array("XYH")).sum(axis=1).max() < 1e-8
    assert np.array_equal(o.array("Neigh") + o.array("Num_ghostcell"), o.array("KFace"))
    for name in SETUP:
        assert np.array_equal(c.array(name), o.array(name)), name
    o.close()
    c.close()


@pytest.mark.gpu
def test_rocket2_20_iterations_bit_identical(rocket2_dir):
    c = rc.Case(rocket2_dir)
    s = rc.Solver(c)
    s.run(20)
    o = oracle.Oracle(rocket2_dir, threads=oracle.Oracle.max_threads())
    o.run(20)
    PA, WA = s.get_state()
    assert np.array_equal(PA, o.array("PA")) and np.array_equal(WA, o.array("WA"))
    s.close()
    o.close()
