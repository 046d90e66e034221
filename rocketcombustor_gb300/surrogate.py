"""Learned chemistry surrogate: host side of include/rc_mlp.h.

The network maps (T, p, Y_1..Y_4, dt) to the normalised changes z_k of the
per-cell integrator (include/rc_mlp.h: dY_k over the progress scale of the
global reaction, the smaller of its explicit progress and the progress that
exhausts the limiting reactant); it is trained on
the GPU by the project's own kernels (forward, backward, Adam) on pairs the
integrator produces from solver states.  Nothing here is in the reference.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import RcError, load

NIN, NOUT, HID = 7, 4, 128
NPARAM = 51076
_FP = ctypes.POINTER(ctypes.c_float)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_FP)


def param_slices():
    """Name -> (slice, shape) of the flat parameter vector."""
    out, o = {}, 0
    for name, shp in (("W0", (HID, NIN)), ("b0", (HID,)), ("W1", (HID, HID)), ("b1", (HID,)), ("W2", (HID, HID)),
                      ("b2", (HID,)), ("W3", (HID, HID)), ("b3", (HID,)), ("W4", (NOUT, HID)), ("b4", (NOUT,))):
        n = int(np.prod(shp))
        out[name] = (slice(o, o + n), shp)
        o += n
    assert o == NPARAM
    return out


def init_params(seed: int = 0) -> np.ndarray:
    """Seeded initialisation: weights uniform in +-sqrt(6/(fan_in+fan_out)), biases 0."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    for name, (sl, shp) in param_slices().items():
        if name.startswith("W"):
            lim = np.sqrt(6.0 / (shp[0] + shp[1]))
            p[sl] = rng.uniform(-lim, lim, size=int(np.prod(shp))).astype(np.float32)
    return p


class MLP:
    """The surrogate network on one GPU (opaque rc_mlp handle)."""

    def __init__(self, device: int = 0, seed: int = 0):
        L = load()
        h = ctypes.c_void_p()
        st = L.rc_mlp_create(int(device), ctypes.byref(h))
        if st:
            raise RcError(st, "rc_mlp_create")
        self.handle = h
        self.device = device
        self.set_params(init_params(seed))
        self.mean = np.zeros(NIN, dtype=np.float32)
        self.std = np.ones(NIN, dtype=np.float32)
        self.domain = np.array([*T_RANGE, *P_RANGE, *DT_RANGE], dtype=np.float32)

    def _check(self, st):
        if st:
            raise RcError(st, load().rc_mlp_last_error(self.handle).decode())

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == NPARAM
        self._check(load().rc_mlp_set_params(self.handle, _fp(p)))

    def get_params(self) -> np.ndarray:
        p = np.zeros(NPARAM, dtype=np.float32)
        self._check(load().rc_mlp_get_params(self.handle, _fp(p)))
        return p

    def set_norm(self, mean, std, domain=None):
        self.mean = np.ascontiguousarray(mean, dtype=np.float32)
        self.std = np.ascontiguousarray(std, dtype=np.float32)
        if domain is not None:
            self.domain = np.ascontiguousarray(domain, dtype=np.float32)
        self._check(load().rc_mlp_set_norm(self.handle, _fp(self.mean), _fp(self.std), _fp(self.domain)))

    def fit_norm(self, x):
        """Feature mean/std of raw samples x (torch (n, 7)); the features are
        (1000/T, log10 p, log10(Y_k + 1e-10), log10 dt)."""
        f = features(x)
        m = f.mean(0).cpu().numpy()
        s = f.std(0).cpu().numpy()
        s = np.where(s > 1e-6, s, 1.0)
        self.set_norm(m, s, self.domain)

    def forward(self, x):
        """x: CUDA float32 (n, 7) raw features -> (n, 4) on torch's current stream."""
        import torch
        x = x.contiguous()
        y = torch.empty((x.shape[0], NOUT), dtype=torch.float32, device=x.device)
        s = torch.cuda.current_stream(x.device).cuda_stream
        self._check(load().rc_mlp_forward(self.handle, x.data_ptr(), x.shape[0], y.data_ptr(), ctypes.c_void_p(s)))
        return y

    def gradient(self, x, t, sync_loss: bool = True):
        """Mean squared error and its parameter gradient for n (multiple of 128) samples."""
        import torch
        g = torch.empty(NPARAM, dtype=torch.float32, device=x.device)
        loss = ctypes.c_float(0.0)
        s = torch.cuda.current_stream(x.device).cuda_stream
        self._check(load().rc_mlp_gradient(self.handle, x.contiguous().data_ptr(), t.contiguous().data_ptr(),
                                           x.shape[0], g.data_ptr(), ctypes.byref(loss) if sync_loss else None,
                                           ctypes.c_void_p(s)))
        return g, float(loss.value)

    def adam(self, g, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        import torch
        s = torch.cuda.current_stream(g.device).cuda_stream
        self._check(load().rc_mlp_adam(self.handle, g.data_ptr(), lr, beta1, beta2, eps, ctypes.c_void_p(s)))

    def train(self, x, t, steps: int, batch: int = 8192, lr: float = 2e-3, lr_end: float = 1e-4, seed: int = 0,
              log_every: int = 0, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        """Adam on random batches (multiples of 128, drawn on the device) with
        a cosine learning-rate decay from lr to lr_end, all steps in one call
        of rc_mlp_train (one CUDA graph launch per step); returns the loss
        history (one (step, loss) per log point)."""
        import torch
        if steps <= 0:
            return []
        x, t = x.contiguous(), t.contiguous()
        n = x.shape[0]
        batch = max(128, (min(batch, n) // 128) * 128)
        loss = torch.empty(steps, dtype=torch.float32, device=x.device)
        s = torch.cuda.current_stream(x.device).cuda_stream
        self._check(load().rc_mlp_train(self.handle, x.data_ptr(), t.data_ptr(), n, steps, batch, lr, lr_end, beta1,
                                        beta2, eps, seed, loss.data_ptr(), ctypes.c_void_p(s)))
        if not log_every:
            return []
        h = loss.cpu().tolist()
        return [(it, h[it]) for it in range(steps) if it % log_every == 0 or it == steps - 1]

    def close(self):
        if getattr(self, "handle", None):
            load().rc_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def features(x):
    """Un-normalised network features of raw samples (torch (n, 7): T, p, Y_1..Y_4, dt)."""
    f = x.double().clone()
    f[:, 0] = 1000.0 / f[:, 0].clamp_min(1.0)
    f[:, 1] = f[:, 1].clamp_min(1e-30).log10()
    f[:, 2:6] = (f[:, 2:6].clamp_min(0.0) + 1e-10).log10()
    f[:, 6] = f[:, 6].clamp_min(1e-30).log10()
    return f


# sampled training domain: T, p, dt (the solver's nozzle states reach 6000 K
# in the exit corner and 1e2 Pa at the exit of the large area ratios)
T_RANGE, P_RANGE, DT_RANGE = (300.0, 6000.0), (1.0e2, 2.0e7), (1.0e-10, 1.0e-4)


def sample_states(pool, n: int, seed: int, t_range=T_RANGE, p_range=P_RANGE, dt_range=DT_RANGE,
                  keep: float = 0.5):
    """n (state, dt) samples from a pool of solver states (torch (NVar, m),
    float64, CUDA): species from the pool, T and p kept with probability
    `keep` and otherwise drawn uniform / log-uniform over the ranges, dt
    log-uniform."""
    import torch
    g = torch.Generator(device=pool.device)
    g.manual_seed(seed)
    dev = pool.device
    idx = torch.randint(0, pool.shape[1], (n,), generator=g, device=dev)
    P = pool[:, idx].clone()
    u = lambda: torch.rand(n, generator=g, device=dev, dtype=torch.float64)  # noqa: E731
    newT = t_range[0] + (t_range[1] - t_range[0]) * u()
    newp = torch.exp(np.log(p_range[0]) + (np.log(p_range[1]) - np.log(p_range[0])) * u())
    P[3] = torch.where(u() < keep, P[3].clamp(*t_range), newT)
    P[0] = torch.where(u() < keep, P[0].clamp(*p_range), newp)
    dt = torch.exp(np.log(dt_range[0]) + (np.log(dt_range[1]) - np.log(dt_range[0])) * u())
    return P.contiguous(), dt.contiguous()


def collect_pool(solver, iters: int, every: int):
    """Solver states (NVar, NE * snapshots) on the GPU, one snapshot every
    `every` iterations of `iters` (the solver keeps its chemistry mode)."""
    import torch
    snaps = []
    for it in range(1, iters + 1):
        solver.lu_sgs_stage(it)
        if it % every == 0:
            PA, _ = solver.get_state()
            snaps.append(torch.tensor(PA.T.copy(), device="cuda"))
    return torch.cat(snaps, 1).contiguous()


def build_dataset(solver, pool, n: int, seed: int, tol: float = 0.005, max_substeps: int = 2000,
                  chunk: int = 1 << 20):
    """n training pairs: states sampled from `pool` (sample_states), integrated
    over their dt by the FP64 integrator of `solver` at a tolerance ten times
    tighter than the solver's default (the targets then carry about a tenth
    of the integrator's own error), turned into raw features and normalised
    changes.  Returns (x (n', 7), t (n', 4), substeps); samples
    whose target is not finite or outside [-1, 10] are dropped."""
    import torch
    xs, ts, ns = [], [], []
    for k in range(0, n, chunk):
        m = min(chunk, n - k)
        P0, dt = sample_states(pool, m, seed * 7919 + k)
        P1, nsub = solver.chem_integrate(P0, dt, tol, max_substeps)
        x, t = solver.surrogate_samples(P0, P1, dt)
        ok = torch.isfinite(t).all(1) & (t[:, :3] > -1).all(1) & (t[:, :3] < 10).all(1)
        xs.append(x[ok]); ts.append(t[ok]); ns.append(nsub[ok])
    return torch.cat(xs).contiguous(), torch.cat(ts).contiguous(), torch.cat(ns)


def validate(net, x, t):
    """Errors of the network's normalised changes against the integrator's on
    held-out pairs: max and 99th percentile of |r - r_int| over the reacting
    species, and the fraction the error indicator's spread test would accept."""
    import torch
    y = net.forward(x)
    e = (y[:, :3] - t[:, :3]).abs().max(1).values
    rbar = y[:, :3].mean(1, keepdim=True)
    spread = (y[:, :3] - rbar).abs().max(1).values
    return {"max_abs_err": float(e.max()), "p99_abs_err": float(torch.quantile(e.float(), 0.99)),
            "median_abs_err": float(e.median()), "spread_p99": float(torch.quantile(spread.float(), 0.99))}
