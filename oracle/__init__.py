"""Test infrastructure: CPU FP64 oracle of the RocketCombustor steady hot path.

Only the tests, the smoke check and the CPU-baseline leg of the benchmark use
this package.  `build()` compiles rc_oracle.cpp; `Oracle` wraps its C API.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "librc_oracle.so")
SRC = os.path.join(HERE, "rc_oracle.cpp")

# The oracle's arithmetic must not contract a*b+c into FMA: the reference's
# x86-64 build (src/Makefile:43, no -march) has no FMA.
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CXXFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-std=c++17", f"-I{INCLUDE}"]


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/librc_oracle.so (seconds)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [SRC, os.path.join(INCLUDE, "rc_math.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(x) for x in srcs):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run(["g++", *CXXFLAGS, "-o", tmp, SRC], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, cp, i, l, d = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_long)
        L.orc_open.restype = vp; L.orc_open.argtypes = [cp]
        L.orc_last_error.restype = cp; L.orc_last_error.argtypes = [vp]
        L.orc_close.argtypes = [vp]
        L.orc_set_threads.argtypes = [vp, i]
        L.orc_max_threads.restype = i
        L.orc_dims.argtypes = [vp, lp]
        L.orc_scalars.argtypes = [vp, dp]
        L.orc_array.restype = vp; L.orc_array.argtypes = [vp, cp, lp]
        L.orc_call.restype = i; L.orc_call.argtypes = [vp, cp]
        L.orc_run.restype = i; L.orc_run.argtypes = [vp, l, dp]
        L.orc_residual.argtypes = [vp, dp, dp]
        L.orc_clear_error.argtypes = [vp]
        L.orc_gas.argtypes = [vp, dp, d, dp]
        L.orc_enthalpy.argtypes = [vp, d, dp]
        L.orc_transport.argtypes = [vp, d, dp, dp]
        L.orc_diffusion.argtypes = [vp, d, d, dp, dp]
        L.orc_production.argtypes = [vp, d, d, dp, dp]
        L.orc_newton.restype = d; L.orc_newton.argtypes = [vp, d, dp, d]
        L.orc_math.argtypes = [i, dp, dp, dp, l]
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_con_to_pri_jaco.argtypes = [vp, dp, dp]
        L.orc_dwdp.argtypes = [vp, dp, dp]
        L.orc_chem_integrate.restype = i
        L.orc_chem_integrate.argtypes = [vp, l, dp, dp, dp, ip, d, i]
        L.orc_set_chemistry.argtypes = [vp, i, d, i]
        L.orc_chem_nsub.restype = ip; L.orc_chem_nsub.argtypes = [vp]
        L.orc_unsteady_scalars.argtypes = [vp, dp]
        L.orc_bdf2_lusgs.restype = i; L.orc_bdf2_lusgs.argtypes = [vp, i, d]
        L.orc_euler_lusgs.restype = i; L.orc_euler_lusgs.argtypes = [vp, i]
        L.orc_unsteady_step.restype = i; L.orc_unsteady_step.argtypes = [vp, l, ip, ip]
        L.orc_dgesvx.restype = i; L.orc_dgesvx.argtypes = [i, dp, dp, dp, cp, dp]
        _lib = L
    return _lib


def math(which: str, x, y=None) -> np.ndarray:
    """include/rc_math.h exp/log/pow evaluated on the host, elementwise."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_math({"exp": 0, "log": 1, "pow": 2}[which], _dp(x), _dp(y), _dp(out), x.size)
    return out


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# name -> (dtype, shape builder from dims) ; dims = NE,NF,NNT,NVar,Nsp,MaxNei,Ng
_SHAPES = {
    "PA": (np.float64, lambda d: (d[0], d[3])), "WA": (np.float64, lambda d: (d[0], d[3])),
    "hWA": (np.float64, lambda d: (d[0], d[3])), "GradC": (np.float64, lambda d: (d[0], d[3], 2)),
    "GPA": (np.float64, lambda d: (d[6], d[3])), "alpaF": (np.float64, lambda d: (d[1],)),
    "step": (np.float64, lambda d: (d[0],)), "VOL": (np.float64, lambda d: (d[0],)),
    "CELLXY": (np.float64, lambda d: (d[0], 2)), "reflen": (np.float64, lambda d: (d[0], 2)),
    "COOR": (np.float64, lambda d: (d[2], 2)), "VECX": (np.float64, lambda d: (d[1], 2)),
    "SideOfs": (np.float64, lambda d: (d[1], 2)), "wdis": (np.float64, lambda d: (d[0], d[5])),
    "AMLS": (np.float64, lambda d: (d[0], d[5], 2)), "XYH": (np.float64, lambda d: (d[0], 2)),
    "Coor_Ghostnode": (np.float64, lambda d: (d[6], 4, 2)),
    "CellXY_Ghostcell": (np.float64, lambda d: (d[6], 2)), "vol_Ghostcell": (np.float64, lambda d: (d[6],)),
    "N": (np.int32, lambda d: (d[0], 4)), "KFace": (np.int32, lambda d: (d[0],)),
    "NeighF": (np.int32, lambda d: (d[0], 4)), "NeighC": (np.int32, lambda d: (d[0], d[5] + 1)),
    "Neigh": (np.int32, lambda d: (d[0],)), "FNode": (np.int32, lambda d: (d[1], 2)),
    "Neighbor": (np.int32, lambda d: (d[1], 2)), "FProperty": (np.int32, lambda d: (d[1],)),
    "Ghostcell": (np.int32, lambda d: (d[0], d[5])), "Num_ghostcell": (np.int32, lambda d: (d[0],)),
    "Hostcell": (np.int32, lambda d: (d[6],)), "Hostface": (np.int32, lambda d: (d[6],)),
    "BCtype_Ghostcell": (np.int32, lambda d: (d[6],)),
    "WP": (np.float64, lambda d: (d[0], d[3])), "WP2": (np.float64, lambda d: (d[0], d[3])),
    "fixed": (np.float64, lambda d: (d[0], d[3])),
}


def dgesvx(a, b):
    """The oracle's restatement of LAPACK dgesvx('E', 'N') on one system:
    returns (x, info, equed, rcond)."""
    a = np.asfortranarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = b.shape[0]
    x = np.zeros(n)
    eq = ctypes.create_string_buffer(1)
    rc = np.zeros(1)
    info = lib().orc_dgesvx(n, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _dp(b), _dp(x), eq, _dp(rc))
    return x, info, eq.raw.decode(), float(rc[0])


class Oracle:
    """Handle on one case loaded by the oracle (start-up, mesh, initial field
    and reconstruction matrices done, as before the reference's main loop)."""

    def __init__(self, case_dir: str, threads: int = 1):
        L = lib()
        self._h = L.orc_open(case_dir.encode())
        if not self._h:
            raise RuntimeError("oracle: " + L.orc_last_error(None).decode())
        d = (ctypes.c_long * 9)()
        L.orc_dims(self._h, d)
        self.NE, self.NF, self.NNT, self.NVar, self.Nsp, self.MaxNei, self.Nghost, self.nlev_fwd, self.nlev_bwd = list(d)
        s = (ctypes.c_double * 8)()
        L.orc_scalars(self._h, s)
        self.total_volume, self.p_out, self.cfl = s[0], s[1], s[2]
        self.oxidizer_mass_flow, self.fuel_mass_flow = s[3], s[4]
        self.viscous, self.combustion, self.limit_id = bool(s[5]), bool(s[6]), int(s[7])
        self.set_threads(threads)

    def close(self):
        if self._h:
            lib().orc_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int):
        lib().orc_set_threads(self._h, int(n))

    @staticmethod
    def max_threads() -> int:
        return lib().orc_max_threads()

    def array(self, name: str) -> np.ndarray:
        """Live view of an internal array, indexed [last Fortran dim, ..., first]
        (the transpose of the Fortran shape; PA is (NE, NVar))."""
        n = ctypes.c_long()
        p = lib().orc_array(self._h, name.encode(), ctypes.byref(n))
        if not p:
            raise KeyError(name)
        dt, shp = _SHAPES[name]
        dims = (self.NE, self.NF, self.NNT, self.NVar, self.Nsp, self.MaxNei, self.Nghost)
        shape = shp(dims)
        buf = (ctypes.c_byte * (n.value * np.dtype(dt).itemsize)).from_address(p)
        return np.frombuffer(buf, dtype=dt).reshape(shape)

    def call(self, sub: str) -> int:
        return lib().orc_call(self._h, sub.encode())

    def run(self, nsteps: int, history: bool = False):
        hist = np.zeros((nsteps, self.NVar + 1)) if history else None
        e = lib().orc_run(self._h, nsteps, _dp(hist) if history else None)
        if e:
            raise RuntimeError(f"oracle error {e}: " + lib().orc_last_error(self._h).decode())
        return hist

    def residual(self):
        r = np.zeros(self.NVar)
        m = np.zeros(1)
        lib().orc_residual(self._h, _dp(r), _dp(m))
        return r, float(m[0])

    def last_error(self) -> str:
        return lib().orc_last_error(self._h).decode()

    def clear_error(self):
        lib().orc_clear_error(self._h)

    # point functions
    def gas(self, Y, T):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        o = np.zeros(3)
        lib().orc_gas(self._h, _dp(Y), float(T), _dp(o))
        return o  # Cp, gama, Rcpcv

    def enthalpy(self, T):
        o = np.zeros(self.Nsp)
        lib().orc_enthalpy(self._h, float(T), _dp(o))
        return o

    def transport(self, T, Y):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        o = np.zeros(2)
        lib().orc_transport(self._h, float(T), _dp(Y), _dp(o))
        return o

    def diffusion(self, p, T, Y):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        o = np.zeros(self.Nsp)
        lib().orc_diffusion(self._h, float(p), float(T), _dp(Y), _dp(o))
        return o

    def production(self, T, rho, Y):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        o = np.zeros(self.Nsp)
        lib().orc_production(self._h, float(T), float(rho), _dp(Y), _dp(o))
        return o

    def con_to_pri_jaco(self, pri):
        pri = np.ascontiguousarray(pri, dtype=np.float64)
        o = np.zeros((self.NVar, self.NVar))
        lib().orc_con_to_pri_jaco(self._h, _dp(pri), _dp(o))
        return o

    def dwdp(self, pri):
        pri = np.ascontiguousarray(pri, dtype=np.float64)
        o = np.zeros((self.Nsp - 1, self.NVar))
        lib().orc_dwdp(self._h, _dp(pri), _dp(o))
        return o

    def chem_integrate(self, P, dt, tol=0.05, maxsub=200):
        """Integrate n primitive states (n x NVar) over dt (n); returns
        (states after dt, accepted substep counts)."""
        P = np.ascontiguousarray(np.atleast_2d(P), dtype=np.float64)
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (P.shape[0],)))
        out = np.empty_like(P)
        nsub = np.zeros(P.shape[0], dtype=np.int32)
        e = lib().orc_chem_integrate(self._h, P.shape[0], _dp(P), _dp(dt), _dp(out),
                                     nsub.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), float(tol), int(maxsub))
        if e:
            raise RuntimeError(f"oracle error {e}: " + self.last_error())
        return out, nsub

    def set_chemistry(self, mode, tol=0.05, maxsub=200):
        """Source mode: 0 explicit rate (the reference), 1 integrated over the
        cell's pseudo time step."""
        lib().orc_set_chemistry(self._h, int(mode), float(tol), int(maxsub))

    def chem_nsub(self):
        p = lib().orc_chem_nsub(self._h)
        if not p:
            return None
        return np.ctypeslib.as_array(p, shape=(self.NE,)).copy()

    # unsteady dual-time BDF2
    def unsteady(self) -> dict:
        s = np.zeros(12)
        lib().orc_unsteady_scalars(self._h, _dp(s))
        return {"ttime": s[0], "dt": s[1], "p_out": s[2], "p_static": s[3], "rel_tol": s[4],
                "inner_loop": int(s[5]), "steady": bool(s[6]), "A_p": s[7], "f_p": s[8],
                "totaltime": s[9], "nstep_max": int(s[10]), "method": int(s[11])}

    def bdf2_lusgs(self, inner_rk: int, phi: float) -> int:
        return lib().orc_bdf2_lusgs(self._h, int(inner_rk), float(phi))

    def euler_lusgs(self, inner_rk: int) -> int:
        return lib().orc_euler_lusgs(self._h, int(inner_rk))

    def unsteady_step(self, istep: int):
        """One physical step of the case's implicit scheme (BDF2 or backward
        Euler); returns (inner iterations, last step)."""
        inner = ctypes.c_int()
        stop = ctypes.c_int()
        e = lib().orc_unsteady_step(self._h, int(istep), ctypes.byref(inner), ctypes.byref(stop))
        if e:
            raise RuntimeError(f"oracle error {e}: " + self.last_error())
        return inner.value, bool(stop.value)

    def newton(self, et, Y, t0):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        return lib().orc_newton(self._h, float(et), _dp(Y), float(t0))
