"""Host side of the product (no GPU): set-up arrays and the C ABI surface.

librc_gpu.so carries the host set-up (rc_host.h) next to the kernels; loading it
needs only the CUDA runtime library, not a GPU.  The set-up is checked bit for
bit against the oracle's independent restatement, and the library must export
every function declared in include/*.h.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
import rocketcombustor_gb300 as rc
from conftest import ROOT, make_case

SETUP_ARRAYS = ["KFace", "Neighbor", "FNode", "NeighF", "Neigh", "NeighC", "Ghostcell", "Num_ghostcell",
                "Hostcell", "Hostface", "BCtype_Ghostcell", "COOR", "VECX", "VOL", "CELLXY", "reflen", "wdis",
                "AMLS", "Coor_Ghostnode", "CellXY_Ghostcell", "vol_Ghostcell", "XYH", "PA", "WA"]


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(rc_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = rc.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(rc.SIGNATURES), set(names) ^ set(rc.SIGNATURES)


def test_last_error_buffer_form():
    """rc_last_error_buf copies the message a Fortran host prints before it
    stops: at most len-1 bytes, always NUL-terminated; a NULL buffer or a
    length below 1 is rejected without writing.  (No context: the message is
    the fixed "no context", so no GPU is needed.)"""
    L = rc.load()
    full = L.rc_last_error(None).decode()
    for n in (1, 2, 4, len(full), len(full) + 1, 64):
        buf = ctypes.create_string_buffer(b"\xff" * n, n)
        assert L.rc_last_error_buf(None, buf, n) == rc.RC_OK
        raw = buf.raw
        k = min(len(full), n - 1)
        assert raw[:k].decode() == full[:k] and raw[k] == 0, (n, raw)
    buf = ctypes.create_string_buffer(b"\xff" * 4, 4)
    assert L.rc_last_error_buf(None, buf, 0) == rc.RC_ERR_ARG
    assert buf.raw == b"\xff" * 4
    assert L.rc_last_error_buf(None, None, 16) == rc.RC_ERR_ARG


@pytest.mark.parametrize("name,over", [("t1", {}), ("t2", {}), ("t1", {"order": "random"}),
                                       ("c1", {"nx": 60, "ny": 12})])
def test_setup_matches_oracle_bitwise(case_root, name, over):
    d = make_case(case_root, name, **over)
    o = oracle.Oracle(d)
    c = rc.Case(d)
    assert (c.NE, c.NF, c.NVar, c.Nghost, c.MaxNei) == (o.NE, o.NF, o.NVar, o.Nghost, o.MaxNei)
    for nm in SETUP_ARRAYS:
        a, b = c.array(nm), o.array(nm)
        if nm == "NeighC":
            b = b  # (0:MaxNei, NE) in both
        assert a.shape == b.shape, nm
        assert np.array_equal(a, b), nm
    m, t, g = c.views()
    assert abs(m.total_volume - o.total_volume) == 0.0
    assert g.p_out == o.p_out and g.cfl == o.cfl
    assert t.oxidizer_mass_flow == o.oxidizer_mass_flow
    assert bool(g.IfViscous) == o.viscous and bool(g.If_turn_on_combustion) == o.combustion


def test_bad_case_reports_error(tmp_path):
    with pytest.raises(rc.RcError):
        rc.Case(str(tmp_path / "missing"))


def test_backup_round_trip(case_root, tmp_path):
    """BackupData then Read_Backup (through rc_case_open) restores the state bit for bit."""
    import shutil
    d = make_case(case_root, "t2")
    c = rc.Case(d)
    PA = c.array("PA").copy()
    rng = np.random.default_rng(0)
    PA[:, 3] *= 1 + 1e-3 * rng.standard_normal(c.NE)  # a state that is not the file's
    c.set_state(PA, c.array("WA").copy())
    d2 = str(tmp_path / "copy")
    shutil.copytree(d, d2)
    c.write_backup(d2 + "/fvp1.sav", ttime=1.25)
    c2 = rc.Case(d2)
    assert np.array_equal(c2.array("PA"), PA)


def test_vtk_writer(case_root, tmp_path):
    d = make_case(case_root, "t2")
    c = rc.Case(d)
    path = str(tmp_path / "out.vtk")
    c.write_vtk(path)
    lines = open(path).read().split("\n")
    assert lines[0] == "# vtk DataFile Version 1.0" and lines[3] == "DATASET UNSTRUCTURED_GRID"
    assert lines[4] == f"POINTS {c.NNT} double"
    i = lines.index(f"CELL_DATA {c.NE}")
    names = [ln.split()[1] for ln in lines[i:] if ln.startswith("SCALARS")]
    assert names == ["rho", "u", "v", "p", "T", "Ma", "Y1", "Y2", "Y3", "Y4",
                     "Production_rate_1", "Production_rate_2", "Production_rate_3"]
    k = lines.index("SCALARS p double")
    p = np.array([float(x) for x in lines[k + 2:k + 2 + c.NE]])
    np.testing.assert_allclose(p, c.array("PA")[:, 0], rtol=1e-7)  # e20.8: 8 significant digits
    assert lines[lines.index(f"CELLS {c.NE} {4 * c.NE}") + 1].split()[0] == "3"
