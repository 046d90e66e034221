"""GB300-native steady LU-SGS hot path of RocketCombustor (harryzhou2000/RocketCombustor).

The compute path is librc_gpu.so (hand-written CUDA for sm_103a behind the C ABI
of include/rc_gpu.h).  This module is a thin ctypes host mirroring the reference
driver: `Case` performs start-up and set-up from a case directory in the
reference's input formats (include/rc_host.h) and `Solver` exposes one method per
reference subroutine of the steady iteration:

    Solver.timestep()          TimeStep            src/TimeStep.f90:4
    Solver.reconstruction()    reconstruction      src/fvm2d.f90:183
    Solver.flux_sourceterm()   flux_sourceterm     src/fvm2d.f90:196
    Solver.lu_sgs_steady()     LU_SGS_steady       src/Time_LUSGS_steady.f90:32
    Solver.lu_sgs_stage(i)     lu_sgs_stage        src/Time_LUSGS_steady.f90:4
    Solver.residual()          Residual/step_residual  src/residual.f90:4,61

and, for the unsteady dual-time scheme (implicit_time_method 5):

    Solver.bdf2_lusgs(k, phi, dt)     BDF2_LU_SGS     src/Time_BDF2.f90:71
    Solver.bdf2_stage(i, dt, n, tol)  BDF2_stage      src/Time_BDF2.f90:4
    Solver.euler_stage(i, dt, n, tol) backwardEuler_stage  src/Time_BackwardEuler.f90:4
    Case.run_unsteady(n)              the unsteady branch of program main (src/fvm2d.f90:48-150)

There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Tuple

import numpy as np

from . import build as _build

RC_OK = 0
RC_ERR_ARG = 1024
RC_ERR = {1: "thermo T out of range", 2: "transport T out of range", 4: "negative rho/p/T in TimeStep",
          8: "negative rho/p at a face", 16: "NaN in WA(1,1)", 32: "unknown boundary code",
          64: "LU-SGS wait timed out", 128: "BDF2 cell system singular (dgesvx)",
          1024: "invalid argument", 2048: "CUDA error"}
RC_PREC_FP64, RC_PREC_MIXED, RC_PREC_MIXED_DC = 0, 1, 2
RC_CHEM_EXPLICIT, RC_CHEM_INTEGRATED, RC_CHEM_SURROGATE = 0, 1, 2

_i, _d, _l, _vp, _cp = ctypes.c_int, ctypes.c_double, ctypes.c_long, ctypes.c_void_p, ctypes.c_char_p
_IP, _DP = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)


class RcMesh(ctypes.Structure):
    _fields_ = [("NE", _i), ("NF", _i), ("NNT", _i), ("MaxNei", _i), ("Nghostcell", _i),
                ("KFace", _IP), ("Neighbor", _IP), ("FNode", _IP), ("FProperty", _IP), ("NeighF", _IP),
                ("Neigh", _IP), ("NeighC", _IP), ("Ghostcell", _IP), ("Num_ghostcell", _IP), ("Hostcell", _IP),
                ("BCtype_Ghostcell", _IP), ("COOR", _DP), ("VECX", _DP), ("SideOfs", _DP), ("VOL", _DP),
                ("CELLXY", _DP), ("reflen", _DP), ("wdis", _DP), ("AMLS", _DP), ("Coor_Ghostnode", _DP),
                ("total_volume", _d)]


class RcThermo(ctypes.Structure):
    _fields_ = [("Nsp", _i), ("Rconstant", _d), ("mole_weight", _DP), ("R_species", _DP),
                ("order_of_cp_polynomial", _i), ("thermo_lowest_tem", _d), ("thermo_critical_tem", _d),
                ("thermo_highest_tem", _d), ("low_coef_Cp_species", _DP), ("high_coef_Cp_species", _DP),
                ("low_enthalpy_b1", _DP), ("high_enthalpy_b1", _DP), ("transport_lowest_tem", _d),
                ("transport_critical_tem", _d), ("transport_highest_tem", _d), ("mu_K", _DP * 16),
                ("collision_diameter", _DP), ("LJ_energy", _DP), ("code_chemical_model", _i),
                ("coef_f_react", _DP), ("coef_r_react", _DP), ("Af_react", _d), ("E_react", _d),
                ("oxidizer_mass_fraction", _DP), ("oxidizer_temp_in", _d), ("oxidizer_mass_flow", _d),
                ("fuel_mass_fraction", _DP), ("fuel_temp_in", _d), ("fuel_mass_flow", _d)]


class RcConfig(ctypes.Structure):
    _fields_ = [("IfViscous", _i), ("If_turn_on_combustion", _i), ("limit_ID", _i), ("cfl", _d), ("p_out", _d),
                ("precision", _i), ("device", _i)]


# C-ABI symbol -> (restype, argtypes); the declarations of include/rc_gpu.h and rc_host.h
SIGNATURES = {
    "rc_init": (_i, [ctypes.POINTER(RcMesh), ctypes.POINTER(RcThermo), ctypes.POINTER(RcConfig),
                     ctypes.POINTER(_vp)]),
    "rc_finalize": (_i, [_vp]),
    "rc_set_state": (_i, [_vp, _DP, _DP]),
    "rc_get_state": (_i, [_vp, _DP, _DP]),
    "rc_timestep": (_i, [_vp]),
    "rc_reconstruction": (_i, [_vp]),
    "rc_flux_sourceterm": (_i, [_vp]),
    "rc_lusgs_steady": (_i, [_vp]),
    "rc_lusgs_stage": (_i, [_vp, _i]),
    "rc_residual": (_i, [_vp, _DP, _DP]),
    "rc_sync": (_i, [_vp]),
    "rc_get_array": (_i, [_vp, _cp, _DP]),
    "rc_set_array": (_i, [_vp, _cp, _DP]),
    "rc_set_stream": (_i, [_vp, _vp]),
    "rc_get_stream": (_vp, [_vp]),
    "rc_stats": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong), _IP, _IP]),
    "rc_last_error": (_cp, [_vp]),
    "rc_last_error_buf": (_i, [_vp, _cp, _i]),
    "rc_fp64_rate": (_i, [_vp, _i, _DP, _DP]),
    "rc_case_open": (_i, [_cp, ctypes.POINTER(_vp)]),
    "rc_case_error": (_cp, [_vp]),
    "rc_case_close": (None, [_vp]),
    "rc_case_views": (_i, [_vp, _i, _i, ctypes.POINTER(RcMesh), ctypes.POINTER(RcThermo),
                           ctypes.POINTER(RcConfig)]),
    "rc_case_dims": (None, [_vp, ctypes.POINTER(_l)]),
    "rc_case_PA": (_DP, [_vp]),
    "rc_case_WA": (_DP, [_vp]),
    "rc_case_array": (_vp, [_vp, _cp, ctypes.POINTER(_l)]),
    "rc_run_steady": (_i, [_vp, _i, _i, _l, _l, _DP]),
    "rc_case_set_state": (_i, [_vp, _DP, _DP]),
    "rc_case_write_backup": (_i, [_vp, _cp, _d]),
    "rc_case_write_vtk": (_i, [_vp, _cp]),
    "rc_run_steady_dc": (_i, [_vp, _i, _l, _l, _i, _DP, ctypes.POINTER(_l)]),
    "rc_residual_noalloc": (_i, [_vp, _vp, _vp, _i, _i, _d, _vp, _DP, _DP]),
    "rc_set_precision": (_i, [_vp, _i]),
    "rc_set_chemistry": (_i, [_vp, _i, _d, _i]),
    "rc_init_batch": (_i, [_i, ctypes.POINTER(RcMesh), ctypes.POINTER(RcThermo), ctypes.POINTER(RcConfig),
                           ctypes.POINTER(_vp)]),
    "rc_batch_info": (_i, [_vp, _IP, _IP]),
    "rc_residual_batch": (_i, [_vp, _DP, _DP]),
    "rc_autotune": (_i, [_vp, _i, _cp, _i]),
    "rc_set_wait_limit": (_i, [_vp, ctypes.c_uint]),
    "rc_clear_error": (_i, [_vp]),
    "rc_set_surrogate": (_i, [_vp, _vp, _d]),
    "rc_surrogate_stats": (_i, [_vp, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint)]),
    "rc_surrogate_freeze": (_i, [_vp, _i]),
    "rc_surrogate_samples": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "rc_mlp_create": (_i, [_i, ctypes.POINTER(_vp)]),
    "rc_mlp_destroy": (_i, [_vp]),
    "rc_mlp_set_params": (_i, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "rc_mlp_get_params": (_i, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "rc_mlp_set_norm": (_i, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                             ctypes.POINTER(ctypes.c_float)]),
    "rc_mlp_forward": (_i, [_vp, _vp, _i, _vp, _vp]),
    "rc_mlp_gradient": (_i, [_vp, _vp, _vp, _i, _vp, ctypes.POINTER(ctypes.c_float), _vp]),
    "rc_mlp_adam": (_i, [_vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _vp]),
    "rc_mlp_train": (_i, [_vp, _vp, _vp, ctypes.c_longlong, _i, _i, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, ctypes.c_float, ctypes.c_ulonglong, _vp, _vp]),
    "rc_mlp_last_error": (_cp, [_vp]),
    "rc_chem_substeps": (_i, [_vp, _IP]),
    "rc_chem_integrate": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _d, _i]),
    "rc_set_p_out": (_i, [_vp, _DP]),
    "rc_bdf2_stage": (_i, [_vp, _i, _d, _i, _d, _IP]),
    "rc_bdf2_lusgs": (_i, [_vp, _i, _d, _d]),
    "rc_euler_stage": (_i, [_vp, _i, _d, _i, _d, _IP]),
    "rc_euler_lusgs": (_i, [_vp, _i, _d]),
    "rc_case_unsteady": (_i, [_vp, _DP]),
    "rc_run_unsteady": (_i, [_vp, _i, _l, _l, _DP, _IP]),
    "rc_flow_plan_check": (_i, [_i, _i, _IP, _IP, ctypes.POINTER(ctypes.c_longlong)]),
    "rc_flow_plan_stats": (_i, [_i, _i, _IP, _IP, _i, _i, _i, ctypes.POINTER(ctypes.c_longlong)]),
}

_lib: Optional[ctypes.CDLL] = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load librc_gpu.so (building it first if asked); raises if unavailable."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB) or (build_if_missing and not _build.up_to_date()):
            if not build_if_missing:
                raise RuntimeError(f"{_build.LIB} is missing: run rocketcombustor_gb300.build.build()")
            _build.build()
        L = ctypes.CDLL(_build.LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class RcError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        bits = [v for k, v in RC_ERR.items() if code & k]
        super().__init__(f"RC status {code} ({', '.join(bits)}) {msg}".strip())
        self.code = code


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


_CASE_ARRAYS = {  # name -> (dtype, shape from dims NE,NF,NNT,NVar,Nsp,MaxNei,Ng)
    "KFace": (np.int32, lambda d: (d[0],)), "N": (np.int32, lambda d: (d[0], 4)),
    "Neighbor": (np.int32, lambda d: (d[1], 2)), "FNode": (np.int32, lambda d: (d[1], 2)),
    "FProperty": (np.int32, lambda d: (d[1],)), "NeighF": (np.int32, lambda d: (d[0], 4)),
    "Neigh": (np.int32, lambda d: (d[0],)), "NeighC": (np.int32, lambda d: (d[0], d[5] + 1)),
    "Ghostcell": (np.int32, lambda d: (d[0], d[5])), "Num_ghostcell": (np.int32, lambda d: (d[0],)),
    "Hostcell": (np.int32, lambda d: (d[6],)), "Hostface": (np.int32, lambda d: (d[6],)),
    "BCtype_Ghostcell": (np.int32, lambda d: (d[6],)), "COOR": (np.float64, lambda d: (d[2], 2)),
    "VECX": (np.float64, lambda d: (d[1], 2)), "SideOfs": (np.float64, lambda d: (d[1], 2)),
    "VOL": (np.float64, lambda d: (d[0],)), "CELLXY": (np.float64, lambda d: (d[0], 2)),
    "reflen": (np.float64, lambda d: (d[0], 2)), "wdis": (np.float64, lambda d: (d[0], d[5])),
    "AMLS": (np.float64, lambda d: (d[0], d[5], 2)), "Coor_Ghostnode": (np.float64, lambda d: (d[6], 4, 2)),
    "CellXY_Ghostcell": (np.float64, lambda d: (d[6], 2)), "vol_Ghostcell": (np.float64, lambda d: (d[6],)),
    "XYH": (np.float64, lambda d: (d[0], 2)), "PA": (np.float64, lambda d: (d[0], d[3])),
    "WA": (np.float64, lambda d: (d[0], d[3])),
}


def flow_plan_check(nface: np.ndarray, cother: np.ndarray, nblocks: int, groups: Optional[int] = None,
                    compact: bool = False, nvar: int = 7) -> dict:
    """The host-side check of the dataflow LU-SGS plan (rc_flow_plan_check; no
    GPU needed).  nface (NE,) faces per cell; cother (NE, 4) the cell across
    each face, -1 at a boundary.  Without `groups`: every plan rc_init builds,
    with the stats of the 8-position passes; with it: that one plan
    (rc_flow_plan_stats; compact for k_lusgs_flowc's, whose groups hold up to
    min(128 // nvar, 32) cells).  Raises RcError when a check fails."""
    nface = np.ascontiguousarray(nface, dtype=np.int32)
    ne = nface.shape[0]
    co = np.ascontiguousarray(np.asarray(cother, dtype=np.int32).reshape(ne, 4).T)  # [q * NE + i]
    stats = np.zeros(8, np.int64)
    sp = stats.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    if groups is None:
        st = load().rc_flow_plan_check(ne, int(nblocks), nface.ctypes.data_as(_IP), co.ctypes.data_as(_IP), sp)
    else:
        st = load().rc_flow_plan_stats(ne, int(nblocks), nface.ctypes.data_as(_IP), co.ctypes.data_as(_IP),
                                       int(groups), int(bool(compact)), int(nvar), sp)
    if st:
        raise RcError(st, "dataflow plan check failed" if st == 64 else "bad arguments")
    keys = ("passes_fwd", "passes_bwd", "deps", "max_deps", "steps", "levels_fwd", "levels_bwd", "cells_per_block")
    return dict(zip(keys, (int(v) for v in stats)))


class Case:
    """A case directory after the reference's start-up and set-up (host side)."""

    def __init__(self, case_dir: str):
        L = load()
        h = _vp()
        st = L.rc_case_open(case_dir.encode(), ctypes.byref(h))
        if st:
            raise RcError(st, L.rc_case_error(None).decode())
        self._h = h
        d = (_l * 9)()
        L.rc_case_dims(h, d)
        self.NE, self.NF, self.NNT, self.NVar, self.Nsp, self.MaxNei, self.Nghost, self.nstep_max, self.nscreen = list(d)
        self.dir = case_dir

    def array(self, name: str) -> np.ndarray:
        n = _l()
        p = load().rc_case_array(self._h, name.encode(), ctypes.byref(n))
        if not p:
            raise KeyError(name)
        dt, shp = _CASE_ARRAYS[name]
        dims = (self.NE, self.NF, self.NNT, self.NVar, self.Nsp, self.MaxNei, self.Nghost)
        buf = (ctypes.c_byte * (n.value * np.dtype(dt).itemsize)).from_address(p)
        return np.frombuffer(buf, dtype=dt).reshape(shp(dims))

    def set_state(self, PA: np.ndarray, WA: np.ndarray):
        """Replace the case's host state (PA, WA as (NE, NVar))."""
        PA = np.ascontiguousarray(PA, dtype=np.float64)
        WA = np.ascontiguousarray(WA, dtype=np.float64)
        if PA.shape != (self.NE, self.NVar) or WA.shape != (self.NE, self.NVar):
            raise ValueError("PA and WA must be (NE, NVar)")
        st = load().rc_case_set_state(self._h, _dp(PA), _dp(WA))
        if st:
            raise RcError(st, load().rc_case_error(self._h).decode())

    def write_backup(self, path: str, ttime: float = 0.0):
        """BackupData: restart file of the case's state (fvp format)."""
        st = load().rc_case_write_backup(self._h, path.encode(), float(ttime))
        if st:
            raise RcError(st, load().rc_case_error(self._h).decode())

    def write_vtk(self, path: str):
        """output_vtk: legacy ASCII VTK of the case's state."""
        st = load().rc_case_write_vtk(self._h, path.encode())
        if st:
            raise RcError(st, load().rc_case_error(self._h).decode())

    def run_steady(self, nsteps: int, every: int = 10, precision: int = RC_PREC_FP64, device: int = 0):
        """The steady driver (rc_run_steady): nsteps iterations on the GPU from
        the case's state, which it replaces; returns the residual history
        (nsteps // every rows of Res(1:NVar), romax)."""
        hist = np.zeros((nsteps // every, self.NVar + 1))
        st = load().rc_run_steady(self._h, int(precision), int(device), int(nsteps), int(every), _dp(hist))
        if st:
            raise RcError(st, load().rc_case_error(self._h).decode())
        return hist

    def run_steady_dc(self, nsteps: int, every: int = 10, window: int = 5, device: int = 0):
        """Mixed precision with the defect-correction switch (rc_run_steady_dc);
        returns (history, iteration of the switch or 0)."""
        hist = np.zeros((nsteps // every, self.NVar + 1))
        sw = _l(0)
        st = load().rc_run_steady_dc(self._h, int(device), int(nsteps), int(every), int(window), _dp(hist),
                                     ctypes.byref(sw))
        if st:
            raise RcError(st, load().rc_case_error(self._h).decode())
        return hist, int(sw.value)

    @property
    def unsteady(self) -> dict:
        """Time scheme of the case (flow_solver_info.in and the backup's time)."""
        o = np.zeros(11)
        load().rc_case_unsteady(self._h, _dp(o))
        return {"unsteady": bool(o[0]), "ttime": o[1], "dt": o[2], "totaltime": o[3], "nstep_max": int(o[4]),
                "inner_loop": int(o[5]), "rel_tol": o[6], "p_static": o[7], "A_p": o[8], "f_p": o[9],
                "method": int(o[10])}

    def run_unsteady(self, nsteps: int, every: int = 1, device: int = 0):
        """The unsteady BDF2 driver (rc_run_unsteady): up to nsteps physical
        steps from the case's state and time, which it advances; returns
        (residual history every `every` steps, inner iterations per step)."""
        hist = np.zeros((nsteps // every, self.NVar + 1))
        inner = np.zeros(nsteps, dtype=np.int32)
        st = load().rc_run_unsteady(self._h, int(device), int(nsteps), int(every), _dp(hist),
                                    inner.ctypes.data_as(_IP))
        if st:
            raise RcError(st, load().rc_case_error(self._h).decode())
        return hist, inner

    def views(self, precision: int = RC_PREC_FP64, device: int = 0):
        m, t, g = RcMesh(), RcThermo(), RcConfig()
        st = load().rc_case_views(self._h, precision, device, ctypes.byref(m), ctypes.byref(t), ctypes.byref(g))
        if st:
            raise RcError(st)
        return m, t, g

    def close(self):
        if getattr(self, "_h", None):
            load().rc_case_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Device-resident steady solver for one case (one CUDA stream)."""

    def __init__(self, case: Case, precision: int = RC_PREC_FP64, device: int = 0, stream: Optional[int] = None):
        L = load()
        self.case = case
        m, t, g = case.views(precision, device)
        self._keep = (m, t, g)
        h = _vp()
        st = L.rc_init(ctypes.byref(m), ctypes.byref(t), ctypes.byref(g), ctypes.byref(h))
        if st:
            raise RcError(st, "rc_init")
        self._h = h
        self.precision = int(precision)
        self.NE, self.NF, self.NVar, self.Nghost = case.NE, case.NF, case.NVar, case.Nghost
        if stream is not None:
            self._check(L.rc_set_stream(h, _vp(stream)))
        self.set_state(case.array("PA"), case.array("WA"))

    # -- status
    def _check(self, st: int):
        if st:
            raise RcError(st, load().rc_last_error(self._h).decode())
        return st

    # -- reference subroutines
    def timestep(self):
        return self._check(load().rc_timestep(self._h))

    def reconstruction(self):
        return self._check(load().rc_reconstruction(self._h))

    def flux_sourceterm(self):
        return self._check(load().rc_flux_sourceterm(self._h))

    def lu_sgs_steady(self):
        return self._check(load().rc_lusgs_steady(self._h))

    def lu_sgs_stage(self, istep: int = 1):
        return self._check(load().rc_lusgs_stage(self._h, int(istep)))

    def set_precision(self, precision: int):
        """RC_PREC_FP64, RC_PREC_MIXED or RC_PREC_MIXED_DC for the following calls."""
        self._check(load().rc_set_precision(self._h, int(precision)))
        self.precision = int(precision)

    def set_chemistry(self, mode: int, tol: float = 0.05, max_substeps: int = 200):
        """RC_CHEM_EXPLICIT (the reference's vol*omega) or RC_CHEM_INTEGRATED
        (mean rate of the per-cell integrator over the pseudo time step)."""
        self._check(load().rc_set_chemistry(self._h, int(mode), float(tol), int(max_substeps)))

    def set_wait_limit(self, polls: int):
        """Polls before a level wait of the persistent LU-SGS gives up (RC_ERR_SYNC)."""
        self._check(load().rc_set_wait_limit(self._h, int(polls)))

    def clear_error(self):
        self._check(load().rc_clear_error(self._h))

    def autotune(self, iters: int = 5) -> str:
        """Pick the fastest launch configuration on the current state (the
        state is restored); returns the timing report."""
        buf = ctypes.create_string_buffer(1024)
        self._check(load().rc_autotune(self._h, int(iters), buf, len(buf)))
        return buf.value.decode()

    def set_surrogate(self, net, spread_tol: float = 0.02):
        """Use the surrogate `net` (rocketcombustor_gb300.surrogate.MLP) for
        RC_CHEM_SURROGATE; it must outlive this solver's use of it."""
        self._check(load().rc_set_surrogate(self._h, net.handle, float(spread_tol)))
        self._net = net

    def surrogate_stats(self):
        """(cells served by the network, cells sent to the integrator) of the last source."""
        a, b = ctypes.c_uint(), ctypes.c_uint()
        self._check(load().rc_surrogate_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def surrogate_freeze(self, on: bool = True):
        """Freeze (record at the next stage, then keep) or free the surrogate's
        per-cell choice between the network and the integrator."""
        self._check(load().rc_surrogate_freeze(self._h, int(bool(on))))

    def surrogate_samples(self, P0, P1, dt):
        """Training pairs from states before (P0) and after (P1) dt: CUDA float64
        tensors (NVar, n) and (n,) -> raw features (n, 7) and targets (n, 4)."""
        import torch
        n = P0.shape[1]
        x = torch.empty((n, 7), dtype=torch.float32, device=P0.device)
        t = torch.empty((n, 4), dtype=torch.float32, device=P0.device)
        torch.cuda.synchronize(P0.device)
        self._check(load().rc_surrogate_samples(self._h, P0.contiguous().data_ptr(), P1.contiguous().data_ptr(),
                                                dt.contiguous().data_ptr(), n, x.data_ptr(), t.data_ptr()))
        self.sync()
        return x, t

    def chem_substeps(self) -> np.ndarray:
        out = np.zeros(self.NE, dtype=np.int32)
        self._check(load().rc_chem_substeps(self._h, out.ctypes.data_as(_IP)))
        return out

    def chem_integrate(self, P, dt, tol: float = 0.05, max_substeps: int = 200):
        """Integrate n primitive states (CUDA torch tensors: P (NVar, n) SoA,
        dt (n,), float64) on the solver's stream; returns (P_out, nsub) as
        CUDA tensors.  Synchronises the stream."""
        import torch
        if not (P.is_cuda and dt.is_cuda) or P.dtype != torch.float64 or dt.dtype != torch.float64:
            raise ValueError("P and dt must be float64 CUDA tensors")
        P = P.contiguous()
        dt = dt.contiguous()
        n = P.shape[1]
        if P.shape[0] != self.NVar or dt.shape != (n,):
            raise ValueError("P must be (NVar, n) and dt (n,)")
        out = torch.empty_like(P)
        nsub = torch.zeros(n, dtype=torch.int32, device=P.device)
        torch.cuda.synchronize(P.device)  # the tensors were made on torch's stream
        self._check(load().rc_chem_integrate(self._h, P.data_ptr(), dt.data_ptr(), n, out.data_ptr(),
                                             nsub.data_ptr(), float(tol), int(max_substeps)))
        self.sync()
        return out, nsub

    def run(self, nsteps: int):
        for it in range(1, nsteps + 1):
            self.lu_sgs_stage(it)
        return self.sync()

    def run_to_steady(self, tol: float = 1e-8, max_iters: int = 100000, every: int = 10, dc_window: int = 0,
                      start: int = 1, freeze_window: int = 0) -> dict:
        """The steady loop (fvm2d.f90:48-76) with the stopping test the
        reference does not have: iterate lu_sgs_stage until, for every case,
        max_k Res_k(n) / Res_k(1) <= tol, Res_k being the step_residual
        columns (residual.f90:61-97, sum of vol*|dU_k| over the total volume)
        and Res_k(1) their values after the first iteration.  The norms are
        read after the first iteration and then every `every` iterations.

        dc_window > 0 (mixed precision): once the level has not fallen below
        0.99 of its best for dc_window reads, switch to defect correction
        (RC_PREC_MIXED_DC, the FP64 residual driving the FP32 sweeps), whose
        fixed point is the FP64 one.  freeze_window > 0 (surrogate chemistry):
        the same stall test freezes the surrogate's per-cell choice between
        network and integrator (surrogate_freeze), whose switching otherwise
        keeps the source from settling.

        Returns {"iterations": last iteration run, "levels": per-case level at
        the end, "reached": per-case first iteration at or below tol (None if
        not), "history": [(iteration, per-case levels)], "switched_at":
        iteration of the switch or 0, "frozen_at": iteration of the freeze or
        0}."""
        res0 = mask = None
        hist, reached = [], None
        best, since, switched, frozen = np.inf, 0, 0, 0
        fbest, fsince = np.inf, 0
        it = start - 1
        for it in range(start, start + max_iters):
            self.lu_sgs_stage(it)
            if it != start and (it - start + 1) % every:
                continue
            r = np.atleast_2d(self.residual()[0])
            if res0 is None:
                mask = r > 0.0
                res0 = np.where(mask, r, 1.0)
                reached = [None] * r.shape[0]
            lv = np.where(mask, r / res0, 0.0).max(axis=1)
            hist.append((it, lv))
            for k in range(lv.shape[0]):
                if reached[k] is None and lv[k] <= tol:
                    reached[k] = it
            if all(x is not None for x in reached):
                break
            top = float(lv.max())
            if dc_window > 0 and not switched:
                if top < 0.99 * best:
                    best, since = top, 0
                else:
                    since += 1
                    if since >= dc_window:
                        self.set_precision(RC_PREC_MIXED_DC)
                        switched = it
            if freeze_window > 0 and not frozen:
                if top < 0.99 * fbest:
                    fbest, fsince = top, 0
                else:
                    fsince += 1
                    if fsince >= freeze_window:
                        self.surrogate_freeze(True)
                        frozen = it
        self.sync()
        return {"iterations": it - start + 1, "levels": hist[-1][1] if hist else None, "reached": reached,
                "history": hist, "switched_at": switched, "frozen_at": frozen}

    # -- unsteady dual-time BDF2
    def set_p_out(self, p_out: float):
        """Exit pressure for the following calls (compute_p_out's result)."""
        p = np.array([float(p_out)])
        self._check(load().rc_set_p_out(self._h, _dp(p)))

    def bdf2_lusgs(self, inner_rk: int, phi: float, dt: float):
        """BDF2_LU_SGS on the current residual (time levels from set_array("WP"/"WP2"))."""
        return self._check(load().rc_bdf2_lusgs(self._h, int(inner_rk), float(phi), float(dt)))

    def bdf2_stage(self, istep: int, dt: float, inner_loop: int, rel_tol: float) -> int:
        """BDF2_stage; returns the inner iterations taken."""
        n = ctypes.c_int()
        self._check(load().rc_bdf2_stage(self._h, int(istep), float(dt), int(inner_loop), float(rel_tol),
                                         ctypes.byref(n)))
        return n.value

    def euler_lusgs(self, inner_rk: int, dt: float):
        """backwardEuler_LU_SGS on the current residual."""
        return self._check(load().rc_euler_lusgs(self._h, int(inner_rk), float(dt)))

    def euler_stage(self, istep: int, dt: float, inner_loop: int, rel_tol: float) -> int:
        """backwardEuler_stage; returns the inner iterations taken."""
        n = ctypes.c_int()
        self._check(load().rc_euler_stage(self._h, int(istep), float(dt), int(inner_loop), float(rel_tol),
                                          ctypes.byref(n)))
        return n.value

    def residual(self) -> Tuple[np.ndarray, float]:
        r = np.zeros(self.NVar)
        m = np.zeros(1)
        self._check(load().rc_residual(self._h, _dp(r), _dp(m)))
        return r, float(m[0])

    def sync(self):
        return self._check(load().rc_sync(self._h))

    # -- state / arrays in the reference layout (numpy shape = reversed Fortran shape)
    def set_state(self, PA: np.ndarray, WA: np.ndarray):
        PA = np.ascontiguousarray(PA, dtype=np.float64)
        WA = np.ascontiguousarray(WA, dtype=np.float64)
        self._check(load().rc_set_state(self._h, _dp(PA), _dp(WA)))

    def get_state(self, PA: Optional[np.ndarray] = None, WA: Optional[np.ndarray] = None):
        """PA, WA (NE, NVar); writes into the given C-contiguous float64 buffers if any."""
        PA = np.zeros((self.NE, self.NVar)) if PA is None else PA
        WA = np.zeros((self.NE, self.NVar)) if WA is None else WA
        for a in (PA, WA):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != (self.NE, self.NVar):
                raise ValueError("state buffers must be C-contiguous float64 (NE, NVar)")
        self._check(load().rc_get_state(self._h, _dp(PA), _dp(WA)))
        return PA, WA

    _SHAPES = {"PA": lambda s: (s.NE, s.NVar), "WA": lambda s: (s.NE, s.NVar), "hWA": lambda s: (s.NE, s.NVar),
               "GradC": lambda s: (s.NE, s.NVar, 2), "GPA": lambda s: (s.Nghost, s.NVar),
               "alpaF": lambda s: (s.NF,), "step": lambda s: (s.NE,), "WP": lambda s: (s.NE, s.NVar),
               "WP2": lambda s: (s.NE, s.NVar)}

    def get_array(self, name: str) -> np.ndarray:
        out = np.zeros(self._SHAPES[name](self))
        self._check(load().rc_get_array(self._h, name.encode(), _dp(out)))
        return out

    def set_array(self, name: str, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(self._SHAPES[name](self))
        self._check(load().rc_set_array(self._h, name.encode(), _dp(a)))

    def write_backup(self, path: str, ttime: float = 0.0):
        """The device state as a restart file (BackupData, output.f90:256-273)."""
        PA, WA = self.get_state()
        self.case.set_state(PA, WA)
        self.case.write_backup(path, ttime)

    def write_vtk(self, path: str):
        """The device state as a VTK file (output_vtk, output.f90:5-227)."""
        PA, WA = self.get_state()
        self.case.set_state(PA, WA)
        self.case.write_vtk(path)

    def stream(self) -> int:
        return load().rc_get_stream(self._h) or 0

    def stats(self):
        n = ctypes.c_longlong()
        f, b = _i(), _i()
        load().rc_stats(self._h, ctypes.byref(n), ctypes.byref(f), ctypes.byref(b))
        return {"kernel_launches": n.value, "fwd_levels": f.value, "bwd_levels": b.value}

    def close(self):
        if getattr(self, "_h", None):
            load().rc_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver(Solver):
    """Several independent cases in one context: every kernel launch of an
    iteration covers all of them.  States are the cases' arrays concatenated
    (case k's cells after those of cases 0..k-1)."""

    def __init__(self, cases, precision: int = RC_PREC_FP64, device: int = 0, stream: Optional[int] = None):
        L = load()
        self.cases = list(cases)
        n = len(self.cases)
        views = [c.views(precision, device) for c in self.cases]
        ms = (RcMesh * n)(*[v[0] for v in views])
        ts = (RcThermo * n)(*[v[1] for v in views])
        gs = (RcConfig * n)(*[v[2] for v in views])
        self._keep = (views, ms, ts, gs)
        h = _vp()
        st = L.rc_init_batch(n, ms, ts, gs, ctypes.byref(h))
        if st:
            raise RcError(st, "rc_init_batch")
        self._h = h
        self.case = self.cases[0]
        self.precision = int(precision)
        self.ncase = n
        self.NE = sum(c.NE for c in self.cases)
        self.NF = sum(c.NF for c in self.cases)
        self.Nghost = sum(c.Nghost for c in self.cases)
        self.NVar = self.cases[0].NVar
        off = np.zeros(n + 1, dtype=np.int32)
        nc = _i()
        L.rc_batch_info(h, ctypes.byref(nc), off.ctypes.data_as(_IP))
        self.offsets = off
        if stream is not None:
            self._check(L.rc_set_stream(h, _vp(stream)))
        self.set_state(np.concatenate([c.array("PA") for c in self.cases]),
                       np.concatenate([c.array("WA") for c in self.cases]))

    def residual(self):
        """Per-case norms: (ncase, NVar) and romax (ncase,)."""
        r = np.zeros((self.ncase, self.NVar))
        m = np.zeros(self.ncase)
        self._check(load().rc_residual_batch(self._h, _dp(r), _dp(m)))
        return r, m

    def case_slice(self, k: int) -> slice:
        return slice(int(self.offsets[k]), int(self.offsets[k + 1]))
