"""rc_residual_noalloc: the residual norms for callers that cannot allocate.

Hosts whose device arrays are owned by another allocator or runtime (a Fortran
host with CUDA Fortran/OpenACC device arrays, say), or solver loops that must
not call cudaMalloc after set-up, pass their own device copies of hWA, WA and
VOL; the entry point uses scratch compiled into the library.  This test hands
it device buffers made by the test and checks its output against rc_residual
on the same solver state, twice in a row on different states, so that the
second call would show anything left over in the shared scratch.
"""
import ctypes

import numpy as np
import pytest

import rocketcombustor_gb300 as rc
from conftest import make_case

pytestmark = pytest.mark.gpu

_DP = ctypes.POINTER(ctypes.c_double)


def _noalloc(L, dh, dw, dv, ne, nvar, total_volume):
    res = np.zeros(nvar)
    rm = np.zeros(1)
    st = L.rc_residual_noalloc(ctypes.c_void_p(dh), ctypes.c_void_p(dw), ctypes.c_void_p(dv), ne, nvar,
                               total_volume, None, res.ctypes.data_as(_DP), rm.ctypes.data_as(_DP))
    return st, res, float(rm[0])


@pytest.mark.parametrize("name,over", [("t2", {}), ("c1", {"nx": 40, "ny": 8})])
def test_noalloc_residual_matches_rc_residual(case_root, name, over):
    """Same bits as rc_residual: both reduce over the same 304 blocks of 256
    threads in the same order with the same build flags.  The 288-cell case
    leaves 16 of the 304 blocks without cells; the 640-cell one fills all."""
    torch = pytest.importorskip("torch")
    d = make_case(case_root, name, **over)
    case = rc.Case(d)
    assert (case.NE < 304) == (name == "t2")
    solver = rc.Solver(case, device=0)
    L = rc.load()
    total_volume = case.views()[0].total_volume
    vol = torch.from_numpy(np.ascontiguousarray(case.array("VOL"))).to("cuda:0")
    for it in (1, 2):
        solver.lu_sgs_stage(it)
        res_ref, romax_ref = solver.residual()
        hwa = torch.from_numpy(solver.get_array("hWA")).to("cuda:0")
        wa = torch.from_numpy(solver.get_state()[1]).to("cuda:0")
        torch.cuda.synchronize()
        st, res, romax = _noalloc(L, hwa.data_ptr(), wa.data_ptr(), vol.data_ptr(), case.NE, case.NVar,
                                  total_volume)
        assert st == rc.RC_OK
        assert np.array_equal(res, np.asarray(res_ref, dtype=np.float64)), (res, res_ref)
        assert romax == romax_ref
    solver.close()


def test_noalloc_rejects_nvar_beyond_scratch():
    L = rc.load()
    st, _, _ = _noalloc(L, 1, 1, 1, 10, 17, 1.0)  # checked before any device work
    assert st == 1024
