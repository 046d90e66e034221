"""Restart file and VTK written from a solver's device state (needs a GB300).

After 10 FP64 iterations on the GPU the state goes through
Solver.write_backup and Solver.write_vtk.  The restart file must have the
layout of BackupData (output.f90:256-273: ttime, NE, then per cell x, y and
PA(1:NVar)), hold the oracle's state after the same iterations exactly, and
read back through Read_Backup (the case reader) bit for bit.  Every VTK scalar
of output_vtk (output.f90:5-227) must equal the value computed from the
oracle's state to the 8 significant digits of its e20.8 edit descriptor.
"""
import os
import shutil

import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from conftest import make_case

pytestmark = pytest.mark.gpu

VTK_RTOL = 1e-7  # e20.8: 8 significant digits


def vtk_scalars(path):
    lines = open(path).read().split("\n")
    ne = int(lines[[k for k, ln in enumerate(lines) if ln.startswith("CELL_DATA")][0]].split()[1])
    out = {}
    for k, ln in enumerate(lines):
        if ln.startswith("SCALARS"):
            assert lines[k + 1].strip() == "LOOKUP_TABLE default"
            out[ln.split()[1]] = np.array([float(x) for x in lines[k + 2:k + 2 + ne]])
    return out


def expected_scalars(o):
    """output_vtk's columns from the oracle's state (output.f90:26-56): rho =
    p/(R T), Ma = |u|/sqrt(gamma R T), Y_k with the last species closing the
    sum, transported-species values below 1e-15 written as 0, and the production rates of the
    transported species (compute_production_rate at the state)."""
    PA = o.array("PA")
    ne, nv = PA.shape
    nsp = nv - 3
    out = {k: np.zeros(ne) for k in ("rho", "u", "v", "p", "T", "Ma")}
    Y = np.zeros((ne, nsp))
    prod = np.zeros((ne, nsp - 1))
    for i in range(ne):
        p, u, v, T = PA[i, :4]
        y = np.append(PA[i, 4:], 1.0 - PA[i, 4:].sum())
        _, gama, R = o.gas(y, T)
        rho = p / (R * T)
        out["rho"][i], out["u"][i], out["v"][i], out["p"][i], out["T"][i] = rho, u, v, p, T
        out["Ma"][i] = np.sqrt(u * u + v * v) / np.sqrt(gama * R * T)
        w = o.production(T, rho, y)[:nsp - 1]
        prod[i] = 0.0 if abs(w[0]) < 1e-15 else w
        Y[i] = y
        Y[i, :nsp - 1] = np.where(np.abs(y[:nsp - 1]) < 1e-15, 0.0, y[:nsp - 1])  # transported species only
    for k in range(nsp):
        out[f"Y{k + 1}"] = Y[:, k]
    for k in range(nsp - 1):
        out[f"Production_rate_{k + 1}"] = prod[:, k]
    return out


def test_backup_and_vtk_from_device_state(case_root, tmp_path):
    d = make_case(case_root, "t2")
    c = rc.Case(d)
    s = rc.Solver(c)
    s.run(10)
    o = oracle.Oracle(d, threads=4)
    o.run(10)
    assert np.array_equal(s.get_state()[0], o.array("PA"))
    bk, vt = str(tmp_path / "fvp1.sav"), str(tmp_path / "out.vtk")
    s.write_backup(bk, ttime=0.5)
    s.write_vtk(vt)
    # BackupData layout and values
    lines = open(bk).read().split("\n")
    assert float(lines[0]) == 0.5 and int(lines[1]) == c.NE
    rows = np.array([[float(x) for x in ln.split()] for ln in lines[2:2 + c.NE]])
    assert rows.shape == (c.NE, 2 + c.NVar)
    assert all(not ln.strip() for ln in lines[2 + c.NE:])
    assert np.array_equal(rows[:, :2], o.array("CELLXY"))
    assert np.array_equal(rows[:, 2:], o.array("PA"))
    # Read_Backup of that file (a copy of the case with it as fvp1.sav)
    d2 = str(tmp_path / "restart")
    shutil.copytree(d, d2)
    shutil.copy(bk, os.path.join(d2, "fvp1.sav"))
    c2 = rc.Case(d2)
    assert np.array_equal(c2.array("PA"), o.array("PA"))
    # every VTK scalar column
    got, want = vtk_scalars(vt), expected_scalars(o)
    assert list(got) == ["rho", "u", "v", "p", "T", "Ma", "Y1", "Y2", "Y3", "Y4",
                         "Production_rate_1", "Production_rate_2", "Production_rate_3"]
    for k, v in want.items():
        scale = np.abs(v).max()
        np.testing.assert_allclose(got[k], v, rtol=VTK_RTOL, atol=VTK_RTOL * 1e-8 * scale, err_msg=k)
    s.close()
    o.close()
