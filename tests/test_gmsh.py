"""gmsh 4.1 reader (readgmsh.f90 restated for one partition): a mesh written
as gmsh and read back gives the same nodes, cells in order and boundary
groups with the solver's codes, and the case it makes runs."""
import os

import numpy as np

import oracle
import rocketcombustor_gb300 as rc
from rocketcombustor_gb300 import cases, gmsh


def test_gmsh_round_trip_and_case(tmp_path):
    m = cases.nozzle_mesh(30, 6, seed=3, wall_type=6)
    phys = {2: 5, 6: 6, 3: 2, 5: 4}  # solver code -> physical tag (inverse of the system table)
    path = str(tmp_path / "n.msh")
    gmsh.write_msh(path, m, phys)
    r = gmsh.read_msh(path)
    assert np.array_equal(r.coor, m.coor)
    assert np.array_equal(r.cells, m.cells)
    got = {code: {tuple(e) for e in pairs} for code, pairs in r.boundaries}
    want = {code: {tuple(e) for e in pairs} for code, pairs in m.boundaries}
    assert got == want
    cfg = cases.CaseConfig("g", nx=30, ny=6, seed=3)
    d = str(tmp_path / "case")
    cases.write_case(d, cfg, mesh=r)
    c = rc.Case(d)
    assert c.NE == m.cells.shape[0]
    o = oracle.Oracle(d, threads=2)
    o.run(3)
    assert np.all(np.isfinite(o.array("PA")))
