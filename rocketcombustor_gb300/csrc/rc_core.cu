// GB300 (sm_103a) kernels and C ABI for the steady LU-SGS iteration of
// RocketCombustor (lu_sgs_stage, src/Time_LUSGS_steady.f90:4-30).
//
// Device layout (structure of arrays, reference cell/face order, 0-based):
//   cell arrays  X[k*NE + i]  (PA, WA, hWA, cell gas state, sources)
//   gradients    G[(2k+r)*NE + i]  (r = x, y in reflen-scaled coordinates)
//   face arrays  F[k*NF + f]  (inviscid and viscous face fluxes)
//   stencils     per cell up to 4 slots, slot q at [q*NE + i], in NeighF order.
//
// One iteration is five kernel kinds (captured in one CUDA graph):
//   k_ts_face   per face:  spectral radius of TimeStep                (TimeStep.f90:16-92)
//   k_cell      per cell:  local step and LU-SGS diagonal, ghost states, LS gradient,
//                          Barth limiter, cell gas state, chemical source
//   k_face_flux per face:  Lax/Rusanov flux and viscous flux           (flux_lax.f90, flux_viscous.f90)
//   k_sweep     per level: forward sweep (with the residual gather) / backward sweep
//   k_update    per cell:  WA += dU and the Newton temperature update
// Face contributions are gathered per cell in NeighF order, which is the
// reference's scatter order, so no atomics are used and the sums are the
// reference's sums.  The sweeps run level by level over the reference cell
// order and compute the reference's Gauss-Seidel recurrences exactly.
//
// Built with --fmad=false: no FMA contraction, matching the reference build.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "rc_gpu.h"
#include "rc_mlp.h"
#include "rc_dev.cuh"
#include "rc_div.cuh"

namespace rc {

// oxidizer_inlet_bc / fuel_inlet_bc (oxidizer.f90:53-68, fuel.f90:54-69)
// with the inlet data of row bc of the case table (w = 0 oxidizer, 1 fuel).
template <int NSP>
__device__ __forceinline__ void inlet_bc(const ThermoDev<NSP>& th, const double* bc, int w, double pl, double& pr,
                                         double& ur, double& vr, double& tr, double& rr, double* Yr, double& Cpr,
                                         double& gamar, double& Rcpcvr, unsigned& err) {
#pragma unroll
  for (int k = 0; k < NSP; ++k) Yr[k] = bc[BC_Y + w * BC_NSPMAX + k];
  tr = bc[BC_T + w];
  gas<NSP>(th, Yr, tr, Cpr, gamar, Rcpcvr, err);
  pr = pl;
  rr = pr / (Rcpcvr * tr);
  ur = bc[BC_MFLOW + w] / rr;
  vr = 0.0;
}

// ----------------------------------------------------------- TimeStep ------
template <int NSP, bool VISC>
__global__ void __launch_bounds__(128) k_ts_face(const Dev d, const ThermoDev<NSP> th) {
  constexpr int V = 3 + NSP;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= d.NF) return;
  unsigned err = 0;
  const int NE = d.NE, NL = d.fNL[f], NR = d.fNR[f];
  double P[V], yy[NSP];
  if (NR >= 0) {
#pragma unroll
    for (int k = 0; k < V; ++k) P[k] = 0.5 * (d.PA[k * NE + NL] + d.PA[k * NE + NR]);
  } else {
#pragma unroll
    for (int k = 0; k < V; ++k) P[k] = d.PA[k * NE + NL];
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { yy[k] = P[4 + k]; s = s + yy[k]; }
  yy[NSP - 1] = 1.0 - s;
  const double pp = P[0], uu = P[1], vv = P[2], tt = P[3];
  double Cp, gama, Rcpcv;
  gas<NSP>(th, yy, tt, Cp, gama, Rcpcv, err);
  const double rr = pp / (Rcpcv * tt);
  if (rr < 0. || pp < 0. || tt < 0.) err |= ERR_NEG_TIMESTEP;
  const double unormal = uu * d.fvec[f] + vv * d.fvec[d.NF + f];
  const double alpa = fabs(unormal) + sqrt(gama * pp / rr) * d.fss[f];
  d.alpa[f] = alpa;
  if (VISC) {
    double vmul, akmu;
    transport<NSP>(th, tt, yy, vmul, akmu, err);
    const double prl = vmul * Cp / akmu;
    const double alpaVis = 2. * d.fs2[f] * fmax2(4. / 3., gama / prl) * vmul / rr;
    const double vl = alpaVis / d.vol[NL];
    d.visL[f] = vl;
    d.visR[f] = (NR >= 0) ? alpaVis / d.vol[NR] : 0.0;
    d.alpaF[f] = alpa + vl;
  } else {
    d.alpaF[f] = alpa;
  }
  flag(d, err);
}

// --------------------------------------------------------- cell kernel -----
// step/dd (TimeStep.f90:94-96, Time_LUSGS_steady.f90:46-53), ghost states
// (update_flow_variables.f90:90-269), gradient (gradient.f90:4-45), Barth
// limiter (limiter.f90:5-107), cell gas state and source (sourceterm.f90:2-70).
template <int NSP>
__global__ void __launch_bounds__(128) k_cell(const Dev d, const ThermoDev<NSP> th, int do_step, int do_recon,
                                              int limit, int comb, int visc) {
  constexpr int V = 3 + NSP;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE;
  unsigned err = 0;
  const int nf = d.nface[i];
  const double vol = d.vol[i];
  if (do_step) {
    const unsigned lb = d.cleft[i];
    double acc = 0.0;
    for (int q = 0; q < nf; ++q) {
      const int f = d.cface[q * NE + i];
      if (visc) acc = acc + d.alpa[f] + (((lb >> q) & 1u) ? d.visL[f] : d.visR[f]);
      else acc = acc + d.alpa[f];
    }
    const double st = th.cfl * vol / acc;
    double dsum = 0.0;
    for (int q = 0; q < nf; ++q) dsum = dsum + 0.5 * d.alpaF[d.cface[q * NE + i]];
    d.step[i] = st;
    const double ddv = dsum + vol / st;
    d.dd[i] = ddv;
    const Recip rd = recip_of(ddv);
    d.rcp[4 * NE + i] = rd.h;
    d.rcp[5 * NE + i] = rd.l;
  }
  if (!do_recon) { flag(d, err); return; }
  double P[V], Y[NSP];
#pragma unroll
  for (int k = 0; k < V; ++k) P[k] = d.PA[k * NE + i];
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { Y[k] = P[4 + k]; s = s + Y[k]; }
  Y[NSP - 1] = 1.0 - s;
  double Cp, gama, Rcpcv, entha[NSP];
  gas<NSP>(th, Y, P[3], Cp, gama, Rcpcv, err);
  const double rr = P[0] / (Rcpcv * P[3]);
  enthalpy<NSP>(th, P[3], entha, err);
  double hh = 0.0;
#pragma unroll
  for (int k = 0; k < NSP; ++k) hh = hh + Y[k] * entha[k];
  d.cst[0 * NE + i] = rr;
  d.cst[1 * NE + i] = gama;
  {
    const Recip a = recip_of(rr), b = recip_of(gama - 1);
    d.rcp[0 * NE + i] = a.h; d.rcp[1 * NE + i] = a.l; d.rcp[2 * NE + i] = b.h; d.rcp[3 * NE + i] = b.l;
  }
  d.cst[2 * NE + i] = rr * (hh + 0.5 * (P[1] * P[1] + P[2] * P[2])) - P[0];
#pragma unroll
  for (int k = 0; k < NSP; ++k) d.cst[(3 + k) * NE + i] = entha[k];

  // gradient with running min/max of the stencil
  double g0[V], g1[V], mn[V], mx[V];
#pragma unroll
  for (int k = 0; k < V; ++k) { g0[k] = 0.0; g1[k] = 0.0; mn[k] = P[k]; mx[k] = P[k]; }
  const int nn = d.nnei[i];
  for (int q = 0; q < nn; ++q) {
    const int j = d.cnei[q * NE + i];
    const double w = d.wdis[q * NE + i], a0 = d.amls[(2 * q) * NE + i], a1 = d.amls[(2 * q + 1) * NE + i];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const double x = d.PA[k * NE + j];
      const double c = w * (x - P[k]);
      g0[k] = g0[k] + a0 * c;
      g1[k] = g1[k] + a1 * c;
      mn[k] = fmin2(mn[k], x);
      mx[k] = fmax2(mx[k], x);
    }
  }
  const int ng = d.ngh[i];
  for (int q = 0; q < ng; ++q) {
    const int gj = d.cgh[q * NE + i];
    const double s1n = d.gsn[gj], s2n = d.gsn[d.NG + gj];
    const double pl = P[0], ul = P[1], vl = P[2], tl = P[3];
    const double ac = sqrt(gama * pl / rr);
    double G[V], Yr[NSP];
    double pr = pl, ur = ul, vr = vl, tr = tl, vn;
#pragma unroll
    for (int k = 0; k < NSP; ++k) Yr[k] = Y[k];
    switch (d.gtype[gj]) {
      case 1: ur = -ul; vr = -vl; break;
      case 2:
      case 6:
        vn = ul * s1n + vl * s2n;
        ur = ul - 2 * vn * s1n;
        vr = vl - 2 * vn * s2n;
        break;
      case 3:
      case 4: {
        double rrb, Cpb, gab, Rb;
        inlet_bc<NSP>(th, bc_row(d, d.gcase, gj), d.gtype[gj] == 3 ? 0 : 1, pl, pr, ur, vr, tr, rrb, Yr, Cpb, gab,
                      Rb, err);
        break;
      }
      case 5:
        vn = ul * s1n + vl * s2n;
        if (!(fabs(vn) > ac)) pr = bc_row(d, d.gcase, gj)[BC_POUT];
        break;
      default: err |= ERR_BCTYPE;
    }
    G[0] = pr; G[1] = ur; G[2] = vr; G[3] = tr;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) G[4 + k] = Yr[k];
#pragma unroll
    for (int k = 0; k < V; ++k) d.GPA[k * d.NG + gj] = G[k];
    const int m = nn + q;
    const double w = d.wdis[m * NE + i], a0 = d.amls[(2 * m) * NE + i], a1 = d.amls[(2 * m + 1) * NE + i];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const double c = w * (G[k] - P[k]);
      g0[k] = g0[k] + a0 * c;
      g1[k] = g1[k] + a1 * c;
      mn[k] = fmin2(mn[k], G[k]);
      mx[k] = fmax2(mx[k], G[k]);
    }
  }
  if (limit > 0) {
    double lv0[MAXF], lv1[MAXF];
    for (int q = 0; q < nf; ++q) { lv0[q] = d.lvvh[(2 * q) * NE + i]; lv1[q] = d.lvvh[(2 * q + 1) * NE + i]; }
#pragma unroll
    for (int k = 0; k < V; ++k) {
      double phi = 1.0;
      for (int q = 0; q < nf; ++q) {
        const double fv = P[k] + (g0[k] * lv0[q] + g1[k] * lv1[q]);
        double pf;
        if (fv > P[k]) pf = fmin2(1.0, (mx[k] - P[k]) / (fv - P[k]));
        else if (fv < P[k]) pf = fmin2(1.0, (mn[k] - P[k]) / (fv - P[k]));
        else pf = 1.0;
        phi = fmin2(phi, pf);
      }
      g0[k] = phi * g0[k];
      g1[k] = phi * g1[k];
    }
  }
#pragma unroll
  for (int k = 0; k < V; ++k) {
    d.grad[(2 * k) * NE + i] = g0[k];
    d.grad[(2 * k + 1) * NE + i] = g1[k];
  }
  if (comb) {
    double prod[NSP];
    production<NSP>(th, P[3], rr, Y, prod);
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) d.src[k * NE + i] = vol * prod[k];
  }
  flag(d, err);
}

// ------------------------------------------------------------ face flux ----
template <int NSP>
__device__ __forceinline__ void recon(const Dev& d, int c, double v0, double v1, double* u) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
#pragma unroll
  for (int k = 0; k < V; ++k)
    u[k] = d.PA[k * NE + c] + (d.grad[(2 * k) * NE + c] * v0 + d.grad[(2 * k + 1) * NE + c] * v1);
}

template <int NSP, bool VISC>
__global__ void __launch_bounds__(128) k_face_flux(const Dev d, const ThermoDev<NSP> th) {
  constexpr int V = 3 + NSP;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= d.NF) return;
  unsigned err = 0;
  const int NE = d.NE, NF = d.NF;
  const int NL = d.fNL[f], NR = d.fNR[f];
  const double sav1 = d.fvec[f], sav2 = d.fvec[NF + f], sav = d.fsav[f];
  const double sav1n = d.fsn[f], sav2n = d.fsn[NF + f];
  double uL[V], uR[V], Yl0[NSP], Yr0[NSP];
  recon<NSP>(d, NL, d.fvL[f], d.fvL[NF + f], uL);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { Yl0[k] = uL[4 + k]; s = s + Yl0[k]; }
  Yl0[NSP - 1] = 1.0 - s;
  double Cpl0, gamal0, Rl0;
  gas<NSP>(th, Yl0, uL[3], Cpl0, gamal0, Rl0, err);
  const double rl0 = uL[0] / (Rl0 * uL[3]);
  double Cpr0 = 0.0, gamar0 = 0.0, Rr0 = 0.0, rr0 = 0.0;
  if (NR >= 0) {
    recon<NSP>(d, NR, d.fvR[f], d.fvR[NF + f], uR);
    s = 0.0;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { Yr0[k] = uR[4 + k]; s = s + Yr0[k]; }
    Yr0[NSP - 1] = 1.0 - s;
    gas<NSP>(th, Yr0, uR[3], Cpr0, gamar0, Rr0, err);
    rr0 = uR[0] / (Rr0 * uR[3]);
  } else {
#pragma unroll
    for (int k = 0; k < V; ++k) uR[k] = uL[k];
  }

  // ---- Lax/Rusanov flux (flux_lax.f90:17-293)
  {
    double pl = uL[0], ul = uL[1], vl = uL[2], tl = uL[3], rl = rl0, gamal = gamal0, Rcl = Rl0, Cpl = Cpl0;
    double pr, ur, vr, tr, rr, gamar, Rcr, Cpr, vn;
    double Yl[NSP], Yr[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) Yl[k] = Yl0[k];
    if (NR >= 0) {
      pr = uR[0]; ur = uR[1]; vr = uR[2]; tr = uR[3]; rr = rr0; gamar = gamar0; Rcr = Rr0; Cpr = Cpr0;
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = Yr0[k];
    } else if (NR == -3 || NR == -4) {
      inlet_bc<NSP>(th, bc_row(d, d.fcase, f), NR == -3 ? 0 : 1, pl, pr, ur, vr, tr, rr, Yr, Cpr, gamar, Rcr, err);
      pl = pr; ul = ur; vl = vr; tl = tr; rl = rr;
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yl[k] = Yr[k];
      Cpl = Cpr; gamal = gamar; Rcl = Rcr;
    } else {
      rr = rl; pr = pl; tr = tl; ur = ul; vr = vl;
      if (NR == -1) { ur = -ul; vr = -vl; }
      else if (NR == -2 || NR == -6) {
        vn = ul * sav1n + vl * sav2n;
        ur = ul - 2 * vn * sav1n;
        vr = vl - 2 * vn * sav2n;
      } else if (NR == -5) {
        const double ac = sqrt(gamal * pl / rl);
        vn = ul * sav1n + vl * sav2n;
        if (!(fabs(vn) > ac)) {
          pr = bc_row(d, d.fcase, f)[BC_POUT];
          ur = ul + sav1n * (pl - pr) / (rl * ac);
          vr = vl + sav2n * (pl - pr) / (rl * ac);
          rr = rl + (pr - pl) / (ac * ac);
          tr = pr / (Rcl * rr);
          pl = pr; ul = ur; vl = vr; tl = tr; rl = rr;
        }
      } else {
        err |= ERR_BCTYPE;
      }
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = Yl[k];
      gamar = gamal; Rcr = Rcl; Cpr = Cpl;
    }
    (void)Cpr; (void)Rcr; (void)Cpl;
    if (rl < 0. || pl < 0. || (NR >= 0 && (rr < 0. || pr < 0.))) err |= ERR_NEG_FACE;
    double entha[NSP];
    enthalpy<NSP>(th, tl, entha, err);
    double hl = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) hl = hl + Yl[k] * entha[k];
    enthalpy<NSP>(th, tr, entha, err);
    double hr = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) hr = hr + Yr[k] * entha[k];
    const double vaml = ul * ul + vl * vl, vamr = ur * ur + vr * vr;
    hl = hl + 0.5 * vaml;
    hr = hr + 0.5 * vamr;
    const double el = hl - pl / rl, er = hr - pr / rr;
    const double acl = sqrt(gamal * pl / rl), acr = sqrt(gamar * pr / rr);
    const double ulnormal = (sav1 * ul + sav2 * vl), urnormal = (sav1 * ur + sav2 * vr);
    const double coex = fmax2(fabs(ulnormal) + acl * sav, fabs(urnormal) + acr * sav);
    const double rul = rl * ulnormal, rur = rr * urnormal;
    d.Finv[0 * NF + f] = 0.5 * (rul + rur - coex * (rr - rl));
    d.Finv[1 * NF + f] = 0.5 * (rul * ul + rur * ur + sav1 * (pl + pr) - coex * (rr * ur - rl * ul));
    d.Finv[2 * NF + f] = 0.5 * (rul * vl + rur * vr + sav2 * (pl + pr) - coex * (rr * vr - rl * vl));
    d.Finv[3 * NF + f] = 0.5 * (rul * hl + rur * hr - coex * (rr * er - rl * el));
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k)
      d.Finv[(4 + k) * NF + f] = 0.5 * (rul * Yl[k] + rur * Yr[k] - coex * (rr * Yr[k] - rl * Yl[k]));
  }

  // ---- viscous flux (flux_viscous.f90:25-343)
  if (VISC) {
    double pl = uL[0], ul = uL[1], vl = uL[2], tl = uL[3], rl = rl0;
    double pr, ur, vr, tr;
    double Yl[NSP], Yr[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) Yl[k] = Yl0[k];
    if (NR >= 0) {
      pr = uR[0]; ur = uR[1]; vr = uR[2]; tr = uR[3];
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = Yr0[k];
    } else if (NR == -3 || NR == -4) {
      double rr, Cpr, gamar, Rcr;
      inlet_bc<NSP>(th, bc_row(d, d.fcase, f), NR == -3 ? 0 : 1, pl, pr, ur, vr, tr, rr, Yr, Cpr, gamar, Rcr, err);
      pl = pr; ul = ur; vl = vr; tl = tr; rl = rr;
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yl[k] = Yr[k];
    } else {
      if (NR == -1) { ul = 0.; vl = 0.; }
      else if (NR == -2 || NR == -6 || NR == -7) removedirection(ul, vl, sav1n, sav2n);
      pr = pl; tr = tl; ur = ul; vr = vl;
      if (NR == -5) {
        const double ac = sqrt(gamal0 * pl / rl);
        const double vn = ul * sav1n + vl * sav2n;
        if (!(fabs(vn) > ac)) {
          pr = bc_row(d, d.fcase, f)[BC_POUT];
          ur = ul + sav1n * (pl - pr) / (rl * ac);
          vr = vl + sav2n * (pl - pr) / (rl * ac);
          const double rrb = rl + (pr - pl) / (ac * ac);
          tr = pr / (Rl0 * rrb);
          pl = pr; ul = ur; vl = vr; tl = tr;
        }
      } else if (NR == -7) {
        pr = 2.0e6; tr = 700; ur = -100; vr = 0;
      }
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = Yl[k];
    }
    (void)rl;
    const double pp = 0.5 * (pl + pr), uu = 0.5 * (ul + ur), vv = 0.5 * (vl + vr), tem = 0.5 * (tl + tr);
    double YY[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) YY[k] = 0.5 * (Yl[k] + Yr[k]);
    double Cp, gama, Rcpcv;
    gas<NSP>(th, YY, tem, Cp, gama, Rcpcv, err);
    const double rr = pp / (Rcpcv * tem);
    // face gradient (flux_viscous.f90:201-224), signed zeros of the dropped
    // g*0.0 basis terms aside
    double t0[V], t1[V];
    {
      const double dxl = d.rinv[NL], dyl = d.rinv[NE + NL];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        t0[k] = d.grad[(2 * k) * NE + NL] * dxl;
        t1[k] = d.grad[(2 * k + 1) * NE + NL] * dyl;
      }
    }
    if (NR >= 0) {
      const double dxk = d.fdxk[f], y1 = d.fysn[f], y2 = d.fysn[NF + f];
      const double rkh = d.fdxkr[f], rkl = d.fdxkr[NF + f];
      const double dxr = d.rinv[NR], dyr = d.rinv[NE + NR];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const double du = uR[k] - uL[k];
        t0[k] = 0.5 * (t0[k] + d.grad[(2 * k) * NE + NR] * dxr) + div_rn(y1 * du, dxk, rkh, rkl);
        t1[k] = 0.5 * (t1[k] + d.grad[(2 * k + 1) * NE + NR] * dyr) + div_rn(y2 * du, dxk, rkh, rkl);
      }
    }
    double dudx = t0[1], dudy = t1[1], dvdx = t0[2], dvdy = t1[2], dtdx = t0[3], dtdy = t1[3];
    double dYdx[NSP], dYdy[NSP];
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { dYdx[k] = t0[4 + k]; dYdy[k] = t1[4 + k]; }
    if (NR == -1 || NR == -6) removedirection(dtdx, dtdy, sav1n, sav2n);
    if (NR == -2) {
      const double snx = sav1n, sny = sav2n, stx = -sny, sty = snx;
      removedirection(dtdx, dtdy, snx, sny);
#pragma unroll
      for (int k = 0; k < NSP - 1; ++k) removedirection(dYdx[k], dYdy[k], snx, sny);
      double dutdx = dudx * stx + dvdx * sty, dutdy = dudy * stx + dvdy * sty;
      double dundx = dudx * snx + dvdx * sny, dundy = dudy * snx + dvdy * sny;
      removedirection(dutdx, dutdy, snx, sny);
      removedirection(dundx, dundy, stx, sty);
      dudx = dutdx * stx + dundx * snx;
      dudy = dutdy * stx + dundy * snx;
      dvdx = dutdx * sty + dundx * sny;
      dvdy = dutdy * sty + dundy * sny;
    }
    {
      double sx = 0.0, sy = 0.0;
#pragma unroll
      for (int k = 0; k < NSP - 1; ++k) { sx = sx + dYdx[k]; sy = sy + dYdy[k]; }
      dYdx[NSP - 1] = -sx;
      dYdy[NSP - 1] = -sy;
    }
    double entha[NSP], Dk[NSP], vmulc, akmu;
    enthalpy<NSP>(th, tem, entha, err);
    transport<NSP>(th, tem, YY, vmulc, akmu, err);
    diffusion<NSP>(th, pp, tem, YY, Dk);
    double uicx = 0.0, uicy = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) uicx = uicx + Dk[k] * dYdx[k];
#pragma unroll
    for (int k = 0; k < NSP; ++k) uicy = uicy + Dk[k] * dYdy[k];
    const double vlac = -2. / 3. * vmulc;
    const double div = dudx + dvdy;
    const double txx = 2. * vmulc * dudx + vlac * div;
    const double tyy = 2. * vmulc * dvdy + vlac * div;
    const double txy = vmulc * (dudy + dvdx);
    double sx = 0.0, sy = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) sx = sx + (Dk[k] * dYdx[k] - YY[k] * uicx) * entha[k];
#pragma unroll
    for (int k = 0; k < NSP; ++k) sy = sy + (Dk[k] * dYdy[k] - YY[k] * uicy) * entha[k];
    const double qx = -akmu * dtdx - rr * sx;
    const double qy = -akmu * dtdy - rr * sy;
    const double btx = uu * txx + vv * txy - qx;
    const double bty = uu * txy + vv * tyy - qy;
    d.Fvis[0 * NF + f] = -(sav1 * txx + sav2 * txy);
    d.Fvis[1 * NF + f] = -(sav1 * txy + sav2 * tyy);
    d.Fvis[2 * NF + f] = -(sav1 * btx + sav2 * bty);
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) {
      const double spx = rr * (Dk[k] * dYdx[k] - YY[k] * uicx);
      const double spy = rr * (Dk[k] * dYdy[k] - YY[k] * uicy);
      d.Fvis[(3 + k) * NF + f] = -(sav1 * spx + sav2 * spy);
    }
  }
  flag(d, err);
}

// Residual of cell i: inviscid faces, then viscous faces, in NeighF order,
// then the chemical source (fvm2d.f90:196-224, sourceterm.f90:51).
template <int NSP>
__device__ __forceinline__ void gather_residual(const Dev& d, int i, int visc, int comb, double* R) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE, NF = d.NF, nf = d.nface[i];
  const unsigned lb = d.cleft[i];
#pragma unroll
  for (int k = 0; k < V; ++k) R[k] = 0.0;
  for (int q = 0; q < nf; ++q) {
    const int f = d.cface[q * NE + i];
    const bool left = (lb >> q) & 1u;
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const double F = d.Finv[k * NF + f];
      R[k] = left ? R[k] - F : R[k] + F;
    }
  }
  if (visc)
    for (int q = 0; q < nf; ++q) {
      const int f = d.cface[q * NE + i];
      const bool left = (lb >> q) & 1u;
#pragma unroll
      for (int k = 1; k < V; ++k) {
        const double F = d.Fvis[(k - 1) * NF + f];
        R[k] = left ? R[k] - F : R[k] + F;
      }
    }
  if (comb) {
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) R[4 + k] = R[4 + k] + d.src[k * NE + i];
  }
}

template <int NSP>
__global__ void __launch_bounds__(128) k_gather(const Dev d, int visc, int comb) {
  constexpr int V = 3 + NSP;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  double R[V];
  gather_residual<NSP>(d, i, visc, comb, R);
#pragma unroll
  for (int k = 0; k < V; ++k) d.hWA[k * d.NE + i] = R[k];
}

// ---------------------------------------------------------------- LU-SGS ---
// LU-SGS forward / backward sweeps (Time_LUSGS_steady.f90:55-190).
// A quad of 4 lanes handles one cell: lane q evaluates the dflux term of the
// neighbour in face slot q, the terms are added in slot order (the NeighF
// order of the reference) and the lanes share the final divisions.  The
// residual R is already in hWA (the gather runs before, fully parallel).
// sweep_load / sweep_compute: the cell at level position t (t >= tend: lanes
// that only join the reduction).  sweep_load reads what the sweep does not
// change (tables, the neighbour's state and gas state, the face, the
// diagonal), so it can be issued before the previous level is complete;
// sweep_compute reads the residuals / increments and does the reference's
// arithmetic in the reference's order.  Called by whole warps.
template <int NSP>
struct SweepPre {
  int i;
  bool valid, act;
  int j;
  double dx, dy, pp, uu, vv, tt, rr, gama, roe, aF, ddi;
  // reciprocal pairs (recip_of) of rr, gama - 1 and ddi: the divisions below
  // by div_rn give the bits of the IEEE divisions
  double rrh, rrl, gmh, gml, ddh, ddl;
  // products of the constants above, formed before the wait with the same
  // operations as the reference expressions use them
  double rou, rov, gm1, roepp, unormal;
  double cs[NSP];          // h_k of the neighbour (cst planes 3..)
  double ry[NSP > 1 ? NSP - 1 : 1];  // rr * Y_k of the neighbour
};
template <int NSP, bool FWD>
__device__ __forceinline__ SweepPre<NSP> sweep_load(const Dev& d, int t, int tend, int q) {
  constexpr int DIR = FWD ? 0 : 1;
  SweepPre<NSP> p;
  p.valid = t < tend;
  const int NE = d.NE, NF = d.NF;
  p.i = p.valid ? d.swi[DIR][t] : 0;
  p.j = p.valid ? d.swj[DIR][q * NE + t] : -1;
  const int fs = p.valid ? d.swf[DIR][q * NE + t] : 0;
  p.ddi = p.valid ? d.dd[p.i] : 1.0;
  p.ddh = p.valid ? d.rcp[4 * NE + p.i] : 1.0;
  p.ddl = p.valid ? d.rcp[5 * NE + p.i] : 0.0;
  p.rrh = 1.0; p.rrl = 0.0; p.gmh = 1.0; p.gml = 0.0;
  p.act = p.j >= 0;
  if (p.act) {
    const int j = p.j, f = fs >= 0 ? fs : ~fs;
    p.dx = d.fvec[f];
    p.dy = d.fvec[NF + f];
    if (fs < 0) { p.dx = -p.dx; p.dy = -p.dy; }
    p.pp = d.PA[0 * NE + j]; p.uu = d.PA[1 * NE + j]; p.vv = d.PA[2 * NE + j]; p.tt = d.PA[3 * NE + j];
    p.rr = d.cst[0 * NE + j]; p.gama = d.cst[1 * NE + j]; p.roe = d.cst[2 * NE + j];
    p.rrh = d.rcp[0 * NE + j]; p.rrl = d.rcp[1 * NE + j]; p.gmh = d.rcp[2 * NE + j]; p.gml = d.rcp[3 * NE + j];
    p.aF = d.alpaF[f];
#pragma unroll
    for (int k = 0; k < NSP; ++k) p.cs[k] = d.cst[(3 + k) * NE + j];
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) p.ry[k] = p.rr * d.PA[(4 + k) * NE + j];
    p.rou = p.rr * p.uu;
    p.rov = p.rr * p.vv;
    p.gm1 = p.gama - 1;
    p.roepp = p.roe + p.pp;
    p.unormal = p.uu * p.dx + p.vv * p.dy;
  }
  return p;
}
template <int NSP, bool FWD>
__device__ __forceinline__ void sweep_compute(const Dev& d, const ThermoDev<NSP>& th, const SweepPre<NSP>& p, int q,
                                              double* wsm) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
  double R0 = 0.0, R1 = 0.0;
  if (p.valid) {  // own residual (variables q and q+4)
    R0 = d.hWA[q * NE + p.i];
    if (q + 4 < V) R1 = d.hWA[(q + 4) * NE + p.i];
  }
  double c[V];
#pragma unroll
  for (int k = 0; k < V; ++k) c[k] = 0.0;
  if (p.act) {
    const int j = p.j;
    const double dx = p.dx, dy = p.dy, uu = p.uu, vv = p.vv, tt = p.tt, rr = p.rr, gama = p.gama;
    const double rou = p.rou, rov = p.rov;
    const double drr = d.hWA[0 * NE + j], dru = d.hWA[1 * NE + j], drv = d.hWA[2 * NE + j],
                 dre = d.hWA[3 * NE + j];
    double dry[NSP], s = 0.0;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { dry[k] = d.hWA[(4 + k) * NE + j]; s = s + dry[k]; }
    dry[NSP - 1] = drr - s;
    const double duu = div_rn(dru - uu * drr, rr, p.rrh, p.rrl);
    const double dvv = div_rn(drv - vv * drr, rr, p.rrh, p.rrl);
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) s1 = s1 + p.cs[k] * dry[k];
#pragma unroll
    for (int k = 0; k < NSP; ++k) s2 = s2 + th.R[k] * dry[k];
    const double gm1 = p.gm1;
    const double dpp =
        gm1 * (dre - s1 + div_rn(tt * s2 * gama, gm1, p.gmh, p.gml) - 0.5 * (dru * uu + duu * rou + drv * vv + dvv * rov));
    const double unormal = p.unormal;
    const double dunormal = duu * dx + dvv * dy;
    const double aF = p.aF;
    c[0] = 0.5 * (-aF * drr + dru * dx + drv * dy);
    c[1] = 0.5 * (-aF * dru + dru * unormal + rou * dunormal + dpp * dx);
    c[2] = 0.5 * (-aF * drv + drv * unormal + rov * dunormal + dpp * dy);
    c[3] = 0.5 * (-aF * dre + dunormal * p.roepp + unormal * (dre + dpp));
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) c[4 + k] = 0.5 * (-aF * dry[k] + dry[k] * unormal + p.ry[k] * dunormal);
  }
  // terms in slot order (NeighF order) through the warp's shared scratch; lane
  // q sums its variables q and q+4 over the 4 slots of its quad.  Inactive
  // slots contribute +0.0, which leaves the sums bit-identical to adding the
  // active terms only (the sums start at +0.0, so -0.0 never occurs).
  const int lane = threadIdx.x & 31, base = lane & ~3;
  __syncwarp();
#pragma unroll
  for (int k = 0; k < V; ++k) wsm[k * 32 + lane] = c[k];
  __syncwarp();
  double df0 = 0.0, df1 = 0.0;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl) {
    df0 = df0 + wsm[q * 32 + base + sl];
    if (q + 4 < V) df1 = df1 + wsm[(q + 4) * 32 + base + sl];
  }
  if (!p.valid) return;
  const double ddi = p.ddi;
  d.hWA[q * NE + p.i] = FWD ? div_rn(R0 - df0, ddi, p.ddh, p.ddl) : R0 - div_rn(df0, ddi, p.ddh, p.ddl);
  if (q + 4 < V)
    d.hWA[(q + 4) * NE + p.i] = FWD ? div_rn(R1 - df1, ddi, p.ddh, p.ddl) : R1 - div_rn(df1, ddi, p.ddh, p.ddl);
}
// The terms of one face slot split in two parts: the terms that need dp (c1,
// c2, c3; dpart) or the others (c0, c4..); both parts compute the velocity
// increments they share.  The same expressions in the same order as
// sweep_compute, so the same bits.
template <int NSP>
__device__ __forceinline__ void sweep_terms(const Dev& d, const ThermoDev<NSP>& th, const SweepPre<NSP>& p,
                                            bool dpart, double* c) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
#pragma unroll
  for (int k = 0; k < V; ++k) c[k] = 0.0;
  if (!p.act) return;
  const int j = p.j;
  const double dx = p.dx, dy = p.dy, uu = p.uu, vv = p.vv, rr = p.rr;
  const double drr = d.hWA[0 * NE + j], dru = d.hWA[1 * NE + j], drv = d.hWA[2 * NE + j];
  double dry[NSP], s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { dry[k] = d.hWA[(4 + k) * NE + j]; s = s + dry[k]; }
  dry[NSP - 1] = drr - s;
  const double duu = div_rn(dru - uu * drr, rr, p.rrh, p.rrl);
  const double dvv = div_rn(drv - vv * drr, rr, p.rrh, p.rrl);
  const double unormal = p.unormal;
  const double dunormal = duu * dx + dvv * dy;
  const double aF = p.aF;
  if (dpart) {
    const double dre = d.hWA[3 * NE + j], tt = p.tt, gama = p.gama, rou = p.rou, rov = p.rov;
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) s1 = s1 + p.cs[k] * dry[k];
#pragma unroll
    for (int k = 0; k < NSP; ++k) s2 = s2 + th.R[k] * dry[k];
    const double gm1 = p.gm1;
    const double dpp = gm1 * (dre - s1 + div_rn(tt * s2 * gama, gm1, p.gmh, p.gml) -
                              0.5 * (dru * uu + duu * rou + drv * vv + dvv * rov));
    c[1] = 0.5 * (-aF * dru + dru * unormal + rou * dunormal + dpp * dx);
    c[2] = 0.5 * (-aF * drv + drv * unormal + rov * dunormal + dpp * dy);
    c[3] = 0.5 * (-aF * dre + dunormal * p.roepp + unormal * (dre + dpp));
  } else {
    c[0] = 0.5 * (-aF * drr + dru * dx + drv * dy);
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) c[4 + k] = 0.5 * (-aF * dry[k] + dry[k] * unormal + p.ry[k] * dunormal);
  }
}
// write a part's terms of slot q into the cell's [k][slot] scratch
template <int NSP>
__device__ __forceinline__ void sweep_put(double* w, bool dpart, int q, const double* c) {
  constexpr int V = 3 + NSP;
  if (dpart) {
#pragma unroll
    for (int k = 1; k < 4; ++k) w[k * 4 + q] = c[k];
  } else {
    w[q] = c[0];
#pragma unroll
    for (int k = 4; k < V; ++k) w[k * 4 + q] = c[k];
  }
}
// The same cell step with 8 lanes per cell: lanes r = 0..3 (slot r) form the
// dp part, lanes r = 4..7 (slot r-4) the other part; then lane r adds
// variable r over the 4 slots in slot order and divides.  wsm: 4 cells x V x
// 4 slots.
template <int NSP, bool FWD>
__device__ __forceinline__ void sweep_compute8(const Dev& d, const ThermoDev<NSP>& th, const SweepPre<NSP>& p,
                                               int r, int cell, double* wsm) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE, q = r & 3;
  const bool dpart = r < 4;
  double R = 0.0;
  if (p.valid && r < V) R = d.hWA[r * NE + p.i];
  double c[V];
  sweep_terms<NSP>(d, th, p, dpart, c);
  double* w = wsm + cell * V * 4;  // [k][slot]
  __syncwarp();
  sweep_put<NSP>(w, dpart, q, c);
  __syncwarp();
  if (!p.valid || r >= V) return;
  double df = 0.0;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl) df = df + w[r * 4 + sl];
  const double ddi = p.ddi;
  d.hWA[r * NE + p.i] = FWD ? div_rn(R - df, ddi, p.ddh, p.ddl) : R - div_rn(df, ddi, p.ddh, p.ddl);
}

template <int NSP, bool FWD>
__device__ __forceinline__ void sweep_step(const Dev& d, const ThermoDev<NSP>& th, int t, int tend, int q,
                                           double* wsm) {
  const SweepPre<NSP> p = sweep_load<NSP, FWD>(d, t, tend, q);
  sweep_compute<NSP, FWD>(d, th, p, q, wsm);
}

// one level of a sweep: block b (one warp) takes cells t0 + b*cpw .. + cpw-1.
// Launched as a programmatic dependent of the previous level: it lets the
// next level start, loads what the sweep does not change, and only then
// waits for the previous level.
// one level with 8 lanes per cell: block b (one warp) takes cells t0 + 4b .. + 3
template <int NSP, bool FWD>
__global__ void __launch_bounds__(32) k_sweep8(const Dev d, const ThermoDev<NSP> th, int t0, int t1) {
  pdl_launch_dependents();
  const int cell = threadIdx.x >> 3, r = threadIdx.x & 7;
  __shared__ double wsm[4 * (3 + NSP) * 4];
  const SweepPre<NSP> p = sweep_load<NSP, FWD>(d, t0 + blockIdx.x * 4 + cell, t1, r & 3);
  pdl_wait();
  sweep_compute8<NSP, FWD>(d, th, p, r, cell, wsm);
}
// one level with the two parts of each slot in two warps (two SM sub-partitions,
// each with its own FP64 pipe): block b (64 threads) takes cells t0 + 8b .. + 7;
// warp 0 forms the dp part of every slot of the 8 cells (lane = 4 cell + slot),
// warp 1 the other part; after a block barrier warp h finishes cells 4h .. 4h+3
// (8 lanes per cell, lane r adds variable r over the slots and divides).  On
// GB300 a warp's FP64 instruction occupies its sub-partition's FP64 pipe for
// 64 cycles whatever its active lanes, so the per-warp instruction count sets
// the level's time: the split cuts it by the other part's share.
template <int NSP, bool FWD>
__global__ void __launch_bounds__(64) k_sweep2w(const Dev d, const ThermoDev<NSP> th, int t0, int t1) {
  constexpr int V = 3 + NSP, DIR = FWD ? 0 : 1;
  pdl_launch_dependents();
  const int NE = d.NE, role = threadIdx.x >> 5, lane = threadIdx.x & 31, cell = lane >> 2, q = lane & 3;
  __shared__ double wsm[8 * V * 4];
  const SweepPre<NSP> p = sweep_load<NSP, FWD>(d, t0 + blockIdx.x * 8 + cell, t1, q);
  const int fcell = role * 4 + (lane >> 3), r = lane & 7, ft = t0 + blockIdx.x * 8 + fcell;
  const bool fvalid = ft < t1 && r < V;
  const int fi = fvalid ? d.swi[DIR][ft] : 0;
  double fdd = 1.0, fddh = 1.0, fddl = 0.0;
  if (fvalid) { fdd = d.dd[fi]; fddh = d.rcp[4 * NE + fi]; fddl = d.rcp[5 * NE + fi]; }
  pdl_wait();
  const double R = fvalid ? d.hWA[r * NE + fi] : 0.0;
  double c[V];
  sweep_terms<NSP>(d, th, p, role == 0, c);
  sweep_put<NSP>(wsm + cell * V * 4, role == 0, q, c);
  __syncthreads();
  if (!fvalid) return;
  const double* w = wsm + fcell * V * 4;
  double df = 0.0;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl) df = df + w[r * 4 + sl];
  d.hWA[r * NE + fi] = FWD ? div_rn(R - df, fdd, fddh, fddl) : R - div_rn(df, fdd, fddh, fddl);
}
// one level with the work of each slot in four warps: block b (128 threads)
// takes cells t0 + 8b .. + 7, lane = 4 cell + slot in every warp, in three
// phases between named barriers 5 (all warps), 6 and 7:
//   A  warp 0: s1 = sum h_k dY_k and c0     warp 1: s2 = sum R_k dY_k and
//      Q = T s2 gamma / (gamma-1)           warp 2: du      warp 3: dv
//   B  warp 2: X = du u + du rho u + dv v + dv rho v,
//      dp = (gamma-1)((dE - s1 + Q) - X/2)
//      warp 3: dun = du nx + dv ny (published before barrier 6), then the
//      species terms
//   C  warps 0-2: c1, c2, c3
// then warps 0 and 1 finish cells 0-3 and 4-7 (8 lanes per cell).  The SM's
// FP64 pipe is shared by the four warps (an FP64 instruction of a full warp
// holds it for 16 cycles on GB300), so each quantity is formed once, in one
// warp, and exchanged through shared memory.  Every expression is the one of
// sweep_terms in the same order, so the same bits.
// hWA as the sweeps read it: through L2 (ld.global.cg) where other SMs write
// it during the launch (the dataflow schedule), else a plain load
template <bool L2>
__device__ __forceinline__ double ldh(const double* p) {
  if (L2) return __ldcg(p);
  return *p;
}
// What finishing a cell needs besides the terms: the cell (-1: no cell at
// this position), dd and its reciprocal pair.
struct Fin4w {
  int i;
  double dd, ddh, ddl;
};
template <bool FWD>
__device__ __forceinline__ Fin4w fin_load(const Dev& d, int ft, int t1) {
  Fin4w f = {-1, 1.0, 1.0, 0.0};
  if (ft < t1) {
    const int i = d.swi[FWD ? 0 : 1][ft];
    f.i = i;
    f.dd = d.dd[i];
    f.ddh = d.rcp[4 * d.NE + i];
    f.ddl = d.rcp[5 * d.NE + i];
  }
  return f;
}
// The sweep step of the 8 cells of one pass on threads 0..127 (four warps,
// lane = 4 cell + slot): p is the thread's (cell, slot) data from sweep_load,
// nbv the hWA of its neighbour (V values; unused when the slot is inactive),
// fn the data of the cell it finishes (warps 0 and 1, 8 lanes per cell).
// A block may hold NG such groups of four warps (threads 128 g .. 128 g +
// 127), each with its own shared scratch and named barriers 5 + 3g, 6 + 3g
// and 7 + 3g.
template <int NSP, bool FWD, bool L2, int NG = 1>
__device__ __forceinline__ void sweep4w_compute(const Dev& d, const ThermoDev<NSP>& th, const SweepPre<NSP>& p,
                                                const double* nbv, const Fin4w& fn) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE, gi = NG > 1 ? (int)(threadIdx.x >> 7) : 0, role = (threadIdx.x >> 5) & 3,
            lane = threadIdx.x & 31, cell = lane >> 2, q = lane & 3;
  __shared__ double wsm_g[NG][8 * V * 4];
  __shared__ double xs1_g[NG][32], xq_g[NG][32], xdp_g[NG][32], xdu_g[NG][32], xdv_g[NG][32], xdn_g[NG][32];
  double* wsm = wsm_g[gi];
  double *xs1 = xs1_g[gi], *xq = xq_g[gi], *xdp = xdp_g[gi], *xdu = xdu_g[gi], *xdv = xdv_g[gi], *xdn = xdn_g[gi];
  const int b5 = 5 + 3 * gi, b6 = 6 + 3 * gi, b7 = 7 + 3 * gi;
  const int fcell = (role & 1) * 4 + (lane >> 3), r = lane & 7;
  const bool fvalid = role < 2 && fn.i >= 0 && r < V;
  const int fi = fvalid ? fn.i : 0;
  const double fdd = fn.dd, fddh = fn.ddh, fddl = fn.ddl;
  const double R = fvalid ? ldh<L2>(d.hWA + r * NE + fi) : 0.0;
  double* w = wsm + cell * V * 4;
  const double aF = p.aF, unormal = p.unormal;
  const double drr = nbv[0], dru = nbv[1], drv = nbv[2], dre = nbv[3];
  double dry[NSP];
#pragma unroll
  for (int k = 0; k < NSP; ++k) dry[k] = 0.0;
  if (role != 2) {  // the species increments: warps 0, 1 and 3
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { dry[k] = nbv[4 + k]; s = s + dry[k]; }
    dry[NSP - 1] = drr - s;
  }
  // A
  if (role == 0) {
    if (p.act) {
      double s1 = 0.0;
#pragma unroll
      for (int k = 0; k < NSP; ++k) s1 = s1 + p.cs[k] * dry[k];
      xs1[lane] = s1;
    }
    w[q] = p.act ? 0.5 * (-aF * drr + dru * p.dx + drv * p.dy) : 0.0;
  } else if (role == 1) {
    if (p.act) {
      double s2 = 0.0;
#pragma unroll
      for (int k = 0; k < NSP; ++k) s2 = s2 + th.R[k] * dry[k];
      xq[lane] = div_rn(p.tt * s2 * p.gama, p.gm1, p.gmh, p.gml);
    }
  } else if (role == 2) {
    if (p.act) xdu[lane] = div_rn(dru - p.uu * drr, p.rr, p.rrh, p.rrl);
  } else {
    if (p.act) xdv[lane] = div_rn(drv - p.vv * drr, p.rr, p.rrh, p.rrl);
  }
  bar_named(b5, 128);
  // B
  if (role == 3) {
    double dunormal = 0.0;
    if (p.act) {
      dunormal = xdu[lane] * p.dx + xdv[lane] * p.dy;
      xdn[lane] = dunormal;
    }
    bar_arrive(b6, 128);
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k)
      w[(4 + k) * 4 + q] = p.act ? 0.5 * (-aF * dry[k] + dry[k] * unormal + p.ry[k] * dunormal) : 0.0;
  } else {
    if (role == 2 && p.act) {
      const double duu = xdu[lane], dvv = xdv[lane];
      const double X = dru * p.uu + duu * p.rou + drv * p.vv + dvv * p.rov;
      xdp[lane] = p.gm1 * (dre - xs1[lane] + xq[lane] - 0.5 * X);
    }
    bar_named(b6, 128);
    // C
    double ck = 0.0;
    if (p.act) {
      const double dpp = xdp[lane], dunormal = xdn[lane];
      if (role == 0) ck = 0.5 * (-aF * dru + dru * unormal + p.rou * dunormal + dpp * p.dx);
      else if (role == 1) ck = 0.5 * (-aF * drv + drv * unormal + p.rov * dunormal + dpp * p.dy);
      else ck = 0.5 * (-aF * dre + dunormal * p.roepp + unormal * (dre + dpp));
    }
    w[(1 + role) * 4 + q] = ck;
  }
  bar_named(b7, 128);
  if (!fvalid) return;
  const double* wf = wsm + fcell * V * 4;
  double df = 0.0;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl) df = df + wf[r * 4 + sl];
  d.hWA[r * NE + fi] = FWD ? div_rn(R - df, fdd, fddh, fddl) : R - div_rn(df, fdd, fddh, fddl);
}
template <int NSP, bool FWD>
__global__ void __launch_bounds__(128) k_sweep4w(const Dev d, const ThermoDev<NSP> th, int t0, int t1) {
  pdl_launch_dependents();
  const int lane = threadIdx.x & 31, role = threadIdx.x >> 5, tb = t0 + blockIdx.x * 8;
  const SweepPre<NSP> p = sweep_load<NSP, FWD>(d, tb + (lane >> 2), t1, lane & 3);
  const Fin4w fn = role < 2 ? fin_load<FWD>(d, tb + (role & 1) * 4 + (lane >> 3), t1) : Fin4w{-1, 1.0, 1.0, 0.0};
  pdl_wait();
  constexpr int V = 3 + NSP;
  double nbv[V];
#pragma unroll
  for (int k = 0; k < V; ++k) nbv[k] = p.act ? d.hWA[k * d.NE + p.j] : 0.0;
  sweep4w_compute<NSP, FWD, false>(d, th, p, nbv, fn);
}
// Both LU-SGS sweeps as a dataflow over one cooperative launch, one block per
// SM.  Block b owns a contiguous range of cells; its cells of one level, in
// runs of at most 8 consecutive sweep positions, form a pass, and the block
// runs its forward passes, then its backward passes, in level order.  A pass
// waits (bounded) only for the passes of other blocks that hold its lower
// (forward) or upper (backward) neighbours; neighbours in the block itself
// were done by an earlier pass.  Warps 0-3 of each compute group compute the
// passes (the four-warp step of k_sweep4w, hWA read through L2); the last warp
// runs one pass ahead of them:
// while they compute it stages the next pass's sweep_load data in shared
// memory and looks once at the flags that pass waits for; when they are done
// (barrier 4) it hands the next pass over (barrier 3) at once if those flags
// were set, and publishes the finished pass's flag = this launch's epoch;
// otherwise it publishes first and then waits for the flags, so that no
// block waits while holding a finished pass that others may need.  The last block to finish advances the
// epoch counter (ctr[0]; ctr[1] counts finished blocks), so the flags need no
// reset between launches.  After a failed wait (ERR_SYNC latched) no flag is
// published any more and every block runs to the end.  The Newton update
// follows as its own launch.
// With G groups a pass holds up to 8 G consecutive positions: G groups of
// four compute warps each take 8 of them (a group without cells in the pass
// only joins the hand-over), and the last warp stages all of them.  On a wide
// mesh a block's cells of one level then form one pass instead of several
// (the 2,000,000-cell nozzle: 6,689 protocol steps with G = 1, 4,420 with 2,
// 2,402 = its levels with 3).  G = 3 has 13 warps, 4 of them on one SM
// sub-partition, which caps a thread at 128 registers (the kernel spills);
// rc_autotune picks G.
constexpr int FLOW_GMAX = 3;
__host__ __device__ constexpr int flow_threads(int G) { return 128 * G + 32; }
template <int NSP, int G>
constexpr int flow_dsmem() { return (int)(2 * 32 * G * sizeof(SweepPre<NSP>)); }
template <int NSP, int G>
__global__ void __launch_bounds__(flow_threads(G), 1) k_lusgs_flow(const Dev d, const ThermoDev<NSP> th, const FlowDev f) {
  constexpr int V = 3 + NSP, FLOW_G = G, FLOW_THREADS = flow_threads(G);
  extern __shared__ __align__(16) uint8_t flow_smem[];
  SweepPre<NSP>(*s_pre)[32 * FLOW_G] = reinterpret_cast<SweepPre<NSP>(*)[32 * FLOW_G]>(flow_smem);
  __shared__ Fin4w s_fin[2][8 * FLOW_G];
  __shared__ unsigned s_epoch;
  __shared__ int s_bad;
  if (threadIdx.x == 0) {
    s_epoch = ld_acquire(f.ctr) + 1u;
    s_bad = 0;
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  const int b = blockIdx.x, lane = threadIdx.x & 31;
  const int f0 = f.boff[0][b], b0 = f.boff[1][b];
  const int nf = f.boff[0][b + 1] - f0, n = nf + (f.boff[1][b + 1] - b0);
  auto pass_of = [&](int k) { return k < nf ? f.blist[0][f0 + k] : f.blist[1][b0 + k - nf]; };
  if (threadIdx.x >= 128 * FLOW_G) {
    // the data of pass k that the sweep does not change
    auto stage = [&](int k) {
      const int pz = pass_of(k), t0 = f.pstart[pz], t1 = t0 + f.pcount[pz];
#pragma unroll
      for (int g = 0; g < FLOW_G; ++g) {
        const int tg = t0 + 8 * g;
        SweepPre<NSP> pl;
        if (k < nf) {
          pl = sweep_load<NSP, true>(d, tg + (lane >> 2), t1, lane & 3);
          if (lane < 8) s_fin[k & 1][8 * g + lane] = fin_load<true>(d, tg + lane, t1);
        } else {
          pl = sweep_load<NSP, false>(d, tg + (lane >> 2), t1, lane & 3);
          if (lane < 8) s_fin[k & 1][8 * g + lane] = fin_load<false>(d, tg + lane, t1);
        }
        s_pre[k & 1][32 * g + lane] = pl;
      }
    };
    auto poll = [&](int k) {
      if (s_bad) return;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && wait_flag(f.pflag + f.deps[d0 + u], epoch, d.err, d.spin_limit);
      if (__any_sync(0xffffffffu, !ok) && lane == 0) s_bad = 1;
      __syncwarp();
    };
    // one look at the flags of pass k, without waiting
    auto ready = [&](int k) -> bool {
      if (s_bad) return true;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && ld_acquire(f.pflag + f.deps[d0 + u]) >= epoch;
      return __all_sync(0xffffffffu, ok) != 0;
    };
    if (n > 0) {
      stage(0);
      poll(0);
      bar_arrive(3, FLOW_THREADS);
    }
    // Never wait for other blocks while holding a finished, unpublished pass:
    // if the next pass's flags are not all set yet, publish first.
    for (int k = 0; k < n; ++k) {
      const bool more = k + 1 < n;
      bool go = false;
      if (more) {
        stage(k + 1);
        go = ready(k + 1);
      }
      bar_named(4, FLOW_THREADS);
      if (go) bar_arrive(3, FLOW_THREADS);
      if (lane == 0 && !s_bad) st_release(f.pflag + pass_of(k), epoch);
      if (more && !go) {
        poll(k + 1);
        bar_arrive(3, FLOW_THREADS);
      }
    }
  } else {
    const int gi = threadIdx.x >> 7, role = (threadIdx.x >> 5) & 3;
    for (int k = 0; k < n; ++k) {
      bar_named(3, FLOW_THREADS);
      // the group's first position holds a cell iff the group has work in
      // this pass; all 128 threads of the group read the same entry
      if (s_fin[k & 1][8 * gi].i >= 0) {
        const SweepPre<NSP> p = s_pre[k & 1][32 * gi + lane];
        const Fin4w fn = s_fin[k & 1][8 * gi + (role & 1) * 4 + (lane >> 3)];
        double nbv[V];
#pragma unroll
        for (int v = 0; v < V; ++v) nbv[v] = p.act ? __ldcg(d.hWA + (size_t)v * d.NE + p.j) : 0.0;
        if (k < nf) sweep4w_compute<NSP, true, true, FLOW_G>(d, th, p, nbv, fn);
        else sweep4w_compute<NSP, false, true, FLOW_G>(d, th, p, nbv, fn);
      }
      bar_arrive(4, FLOW_THREADS);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(f.ctr + 1, 1u) == gridDim.x - 1) {
      f.ctr[1] = 0u;
      __threadfence();
      st_release(f.ctr, epoch);
    }
  }
}

// ---- compact dataflow LU-SGS (k_lusgs_flowc) ----
// In a sweep only the faces to lower (forward) or upper (backward) neighbours
// carry a term: on a triangulation about 1.5 of a cell's 3 slots.  The
// per-slot lanes of k_lusgs_flow spend the other lanes' FP64 issue on terms
// that are zero.  Here a group of four warps takes up to 32 ACTIVE (cell,
// slot) pairs of up to 16 consecutive cells, one pair per lane, so one
// group holds about twice the cells of a k_lusgs_flow group on the same
// FP64 instruction count.  The finishing sums add only the active slots, in
// slot order: a sum that starts at +0.0 is never -0.0, so leaving out the
// +0.0 terms of the inactive slots leaves its bits unchanged.
constexpr int FLOWC_GMAX = 2;
constexpr int FLOWC_STAGERS = 2, FLOWC_NBUF = 4;
// compute groups, the coordinator warp, the staging warps
__host__ __device__ constexpr int flowc_threads(int G) { return 128 * G + 32 + 32 * FLOWC_STAGERS; }
// What the sweep step of one active pair needs (the neighbour j's gas state
// and its products, the face), staged before the pass may start: the fields
// of SweepPre that the step reads, formed with the same expressions.
template <int NSP>
struct PairPre {
  int j;   // the neighbour (-1: no pair in this lane)
  int cs;  // the pair's cell within its group << 2 | its slot
  double dx, dy, uu, vv, tt, rr, gama, aF;
  double rrh, rrl, gmh, gml;
  double rou, rov, gm1, roepp, unormal;
  double cs_h[NSP];
  double ry[NSP > 1 ? NSP - 1 : 1];
};
template <int NSP, bool FWD>
__device__ __forceinline__ PairPre<NSP> pair_load(const Dev& d, int t, int q, int tg) {
  constexpr int DIR = FWD ? 0 : 1;
  const int NE = d.NE, NF = d.NF;
  PairPre<NSP> p;
  const int j = d.swj[DIR][q * NE + t], fs = d.swf[DIR][q * NE + t], f = fs >= 0 ? fs : ~fs;
  p.j = j;
  p.cs = ((t - tg) << 2) | q;
  p.dx = d.fvec[f];
  p.dy = d.fvec[NF + f];
  if (fs < 0) { p.dx = -p.dx; p.dy = -p.dy; }
  const double pp = d.PA[0 * NE + j];
  p.uu = d.PA[1 * NE + j]; p.vv = d.PA[2 * NE + j]; p.tt = d.PA[3 * NE + j];
  p.rr = d.cst[0 * NE + j]; p.gama = d.cst[1 * NE + j];
  const double roe = d.cst[2 * NE + j];
  p.rrh = d.rcp[0 * NE + j]; p.rrl = d.rcp[1 * NE + j]; p.gmh = d.rcp[2 * NE + j]; p.gml = d.rcp[3 * NE + j];
  p.aF = d.alpaF[f];
#pragma unroll
  for (int k = 0; k < NSP; ++k) p.cs_h[k] = d.cst[(3 + k) * NE + j];
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) p.ry[k] = p.rr * d.PA[(4 + k) * NE + j];
  p.rou = p.rr * p.uu;
  p.rov = p.rr * p.vv;
  p.gm1 = p.gama - 1;
  p.roepp = roe + pp;
  p.unormal = p.uu * p.dx + p.vv * p.dy;
  return p;
}
// one ring slot: G groups of 32 pairs and 16 cells
template <int NSP, int G>
__host__ __device__ constexpr int flowc_slot_bytes() {
  return (int)(32 * G * sizeof(PairPre<NSP>) + flowc_cells(3 + NSP) * G * 32);
}
template <int NSP, int G>
__host__ __device__ constexpr int flowc_dsmem() { return FLOWC_NBUF * flowc_slot_bytes<NSP, G>(); }
// The cell a finishing lane needs: its index, dd and dd's reciprocal pair,
// and its active slots (bit q: slot q has a neighbour in this sweep).
struct FinC {
  int i, mask;
  double dd, ddh, ddl;
};
template <bool FWD>
__device__ __forceinline__ FinC finc_load(const Dev& d, int t) {
  constexpr int DIR = FWD ? 0 : 1;
  FinC f;
  const int NE = d.NE;
  f.i = d.swi[DIR][t];
  f.dd = d.dd[f.i];
  f.ddh = d.rcp[4 * NE + f.i];
  f.ddl = d.rcp[5 * NE + f.i];
  f.mask = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) f.mask |= (d.swj[DIR][q * NE + t] >= 0 ? 1 : 0) << q;
  return f;
}
// One group's step (threads 128 g .. 128 g + 127): in the term phases lane l
// holds the group's l-th active pair (p; p.j < 0 past the last pair) and nbv
// its neighbour's hWA; in the finishing phase the group's thread x = 32 role
// + lane finishes variable x % V of local cell x / V (fn: that cell, fn.i < 0
// past the last cell).  The expressions are sweep4w_compute's, each rounded
// operation the same in the same order, but the parts of every term that do
// not wait for du, dv, dp or dun are formed in phase A, where the four warps
// have room, so that fewer dependent FP64 operations follow (on GB300 a
// warp's FP64 instruction holds its sub-partition's FP64 unit for 64
// cycles, so the count per warp on the critical path sets the step's time):
//   A  warp 0: s = 0 + dY_0 + dY_1 + dY_2, dY_3 = drho - s; s1 = 0 + sum h_k dY_k;
//      es1 = dE - s1; S_k = -aF dY_k + dY_k un for k = 0, 1
//      warp 1: dY; s2 = 0 + sum R_k dY_k; Q = (T s2) gamma / (gamma - 1)
//      warp 2: du = (drho u - u drho) / rho; c0; a1 = drho u * u, a3 = drho v * v;
//      P1 = -aF drho u + drho u un
//      warp 3: dY; dv; P2 = -aF drho v + drho v un; A3 = -aF dE; S_2
//   B  warp 3: dun = du nx + dv ny (barrier B6 to warps 0, 1), then the species
//      terms half(S_k + ry_k dun)
//      warp 2: X = ((a1 + du rho u) + a3) + dv rho v, dp = gm1 ((es1 + Q) - X / 2)
//      (barrier B8 to warps 0, 1)
//      warp 0: c1p = P1 + rho u dun; warp 1: c2p = P2 + rho v dun, c3p = A3 + dun (rho E + p)
//   C  warp 0: c1 = half(c1p + dp nx); warp 1: c2 = half(c2p + dp ny);
//      warp 2: c3 = half(c3p + un (dE + dp))
// with 0 + x and 0.5 x on the integer pipe (plus_zero, half_of: the same bits).
template <int NSP, bool FWD, int G>
__device__ __forceinline__ void sweepc_compute(const Dev& d, const ThermoDev<NSP>& th, const PairPre<NSP>& p,
                                               const double* nbv, const FinC& fn) {
  constexpr int V = 3 + NSP, NS = NSP > 1 ? NSP - 1 : 1;
  const int NE = d.NE, gi = G > 1 ? (int)(threadIdx.x >> 7) : 0, role = (threadIdx.x >> 5) & 3,
            lane = threadIdx.x & 31, q = p.cs & 3;
  const bool act = p.j >= 0;
  constexpr int CAP = flowc_cells(V);
  __shared__ double wsc_g[G][CAP * V * 4];
  // per pair: es1, Q, du, dv, dun, dp, P1, P2, A3, c3p, S_0, S_1
  __shared__ double xc_g[G][12][32];
  double* wsm = wsc_g[gi];
  double(*xc)[32] = xc_g[gi];
  enum { ES1, XQ, XDU, XDV, XDN, XDP, XP1, XP2, XA3, XC3, XS0, XS1 };
  const int B5 = 5 + 4 * gi, B6 = B5 + 1, B7 = B5 + 2, B8 = B5 + 3;
  const int x = role * 32 + lane, fc = x / V, r = x - fc * V;
  const bool fvalid = fc < CAP && fn.i >= 0;
  const int fi = fvalid ? fn.i : 0;
  const double R = fvalid ? __ldcg(d.hWA + r * NE + fi) : 0.0;
  double* w = wsm + min(p.cs >> 2, CAP - 1) * V * 4;
  const double aF = p.aF, un = p.unormal;
  const double drr = nbv[0], dru = nbv[1], drv = nbv[2], dre = nbv[3];
  // the species increments dY_k (warps 0, 1 and 3)
  double dry[NSP];
#pragma unroll
  for (int k = 0; k < NSP; ++k) dry[k] = 0.0;
  if (role != 2 && act) {
    double s = 0.0;
    if (NSP > 1) {
      dry[0] = nbv[4];
      s = plus_zero(dry[0]);
#pragma unroll
      for (int k = 1; k < NSP - 1; ++k) { dry[k] = nbv[4 + k]; s = s + dry[k]; }
    }
    dry[NSP - 1] = drr - s;
  }
  // A
  double S2 = 0.0;  // warp 3: S_{NSP-2}
  if (act) {
    if (role == 0) {
      double s1 = plus_zero(p.cs_h[0] * dry[0]);
#pragma unroll
      for (int k = 1; k < NSP; ++k) s1 = s1 + p.cs_h[k] * dry[k];
      xc[ES1][lane] = dre - s1;
      if (NSP > 1) xc[XS0][lane] = -aF * dry[0] + dry[0] * un;
      if (NSP > 2) xc[XS1][lane] = -aF * dry[1] + dry[1] * un;
    } else if (role == 1) {
      double s2 = plus_zero(th.R[0] * dry[0]);
#pragma unroll
      for (int k = 1; k < NSP; ++k) s2 = s2 + th.R[k] * dry[k];
      xc[XQ][lane] = div_rn(p.tt * s2 * p.gama, p.gm1, p.gmh, p.gml);
    } else if (role == 2) {
      xc[XDU][lane] = div_rn(dru - p.uu * drr, p.rr, p.rrh, p.rrl);
      w[q] = half_of(-aF * drr + dru * p.dx + drv * p.dy);
      xc[XP1][lane] = -aF * dru + dru * un;
    } else {
      xc[XDV][lane] = div_rn(drv - p.vv * drr, p.rr, p.rrh, p.rrl);
      xc[XP2][lane] = -aF * drv + drv * un;
      xc[XA3][lane] = -aF * dre;
      if (NSP > 3) S2 = -aF * dry[2] + dry[2] * un;
    }
  }
  // the X partials of warp 2, formed while the others finish phase A
  double a1 = 0.0, a3 = 0.0;
  if (role == 2 && act) {
    a1 = dru * p.uu;
    a3 = drv * p.vv;
  }
  bar_named(B5, 128);
  // B, C
  if (role == 3) {
    double dun = 0.0;
    if (act) {
      dun = xc[XDU][lane] * p.dx + xc[XDV][lane] * p.dy;
      xc[XDN][lane] = dun;
    }
    bar_arrive(B6, 96);
    if (act) {
#pragma unroll
      for (int k = 0; k < NSP - 1; ++k) {
        const double Sk = k == 0 ? xc[XS0][lane] : k == 1 ? xc[XS1][lane] : S2;
        w[(4 + k) * 4 + q] = half_of(Sk + p.ry[k] * dun);
      }
    }
  } else if (role == 2) {
    double dpp = 0.0;
    if (act) {
      const double duu = xc[XDU][lane], dvv = xc[XDV][lane];
      const double X = a1 + duu * p.rou + a3 + dvv * p.rov;
      dpp = p.gm1 * (xc[ES1][lane] + xc[XQ][lane] - half_of(X));
      xc[XDP][lane] = dpp;
    }
    bar_named(B8, 96);
    if (act) w[3 * 4 + q] = half_of(xc[XC3][lane] + un * (dre + dpp));
  } else {
    bar_named(B6, 96);
    double cp = 0.0;
    if (act) {
      const double dun = xc[XDN][lane];
      if (role == 0) {
        cp = xc[XP1][lane] + p.rou * dun;
      } else {
        cp = xc[XP2][lane] + p.rov * dun;
        xc[XC3][lane] = xc[XA3][lane] + dun * p.roepp;
      }
    }
    bar_named(B8, 96);
    if (act) {
      const double dpp = xc[XDP][lane];
      if (role == 0) w[1 * 4 + q] = half_of(cp + dpp * p.dx);
      else w[2 * 4 + q] = half_of(cp + dpp * p.dy);
    }
  }
  (void)NS;
  bar_named(B7, 128);
  if (!fvalid) return;
  const double* wf = wsm + fc * V * 4;
  double df = 0.0;
  bool first = true;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl)
    if ((fn.mask >> sl) & 1) {
      df = first ? plus_zero(wf[r * 4 + sl]) : df + wf[r * 4 + sl];
      first = false;
    }
  d.hWA[r * NE + fi] = FWD ? div_rn(R - df, fn.dd, fn.ddh, fn.ddl) : R - div_rn(df, fn.dd, fn.ddh, fn.ddl);
}
// Both LU-SGS sweeps as a dataflow over one cooperative launch with compact
// passes: block b owns cells [bC, (b+1)C); a pass is a run of consecutive
// positions of one level owned by the block, split into G groups of at most
// 16 cells and 32 active pairs, group g on warps 4g .. 4g+3.  The work
// around a pass is spread over more warps than k_lusgs_flow's single staging
// warp, whose gathers, polls and publishing took longer than a pass:
//  - FLOWC_STAGERS staging warps: warp s stages passes s, s + STAGERS, ...
//    (pair_load / finc_load) into a ring of FLOWC_NBUF shared slots, once
//    the pass that held the slot before is finished (s_consumed); s_slot[b]
//    = k + 1 marks pass k staged in slot b;
//  - the coordinator warp (4G): looks at the flags of the next pass, hands
//    it to the compute warps (barrier 3) once it is staged, its flags are
//    set and the current pass is done (barrier 4), and publishes the
//    finished pass (flag = this launch's epoch), before any blocking wait, so
//    no block waits while holding a finished pass.
// With each hand-over the coordinator writes s_go[slot]: 0 after any wait
// gave up (ERR_SYNC), when the staging may have stopped; all warps of a group
// read the same s_go and skip the pass together, so the group's barriers
// stay matched.  Every wait is bounded.  A group without cells in the pass
// only joins the hand-over.
template <int NSP, int G>
__global__ void __launch_bounds__(flowc_threads(G), 1) k_lusgs_flowc(const Dev d, const ThermoDev<NSP> th, const FlowDev f) {
  constexpr int V = 3 + NSP, T34 = 128 * G + 32, SLOT = flowc_slot_bytes<NSP, G>(), CAP = flowc_cells(V);
  extern __shared__ __align__(16) uint8_t flowc_smem[];
  auto slot_pre = [&](int s) { return reinterpret_cast<PairPre<NSP>*>(flowc_smem + s * SLOT); };
  auto slot_fin = [&](int s) {
    return reinterpret_cast<FinC*>(flowc_smem + s * SLOT + 32 * G * sizeof(PairPre<NSP>));
  };
  __shared__ unsigned s_epoch;
  __shared__ volatile int s_bad, s_consumed;
  __shared__ volatile int s_slot[FLOWC_NBUF], s_go[FLOWC_NBUF];
  if (threadIdx.x == 0) {
    s_epoch = ld_acquire(f.ctr) + 1u;
    s_bad = 0;
    s_consumed = 0;
    for (int s = 0; s < FLOWC_NBUF; ++s) { s_slot[s] = 0; s_go[s] = 0; }
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  const int b = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int f0 = f.boff[0][b], b0 = f.boff[1][b];
  const int nf = f.boff[0][b + 1] - f0, n = nf + (f.boff[1][b + 1] - b0);
  auto pass_of = [&](int k) { return k < nf ? f.blist[0][f0 + k] : f.blist[1][b0 + k - nf]; };
  auto give_up = [&]() {
    if (lane == 0) {
      s_bad = 1;
      atomicOr(d.err, ERR_SYNC);
    }
    __syncwarp();
  };
  if (warp > 4 * G) {
    // staging warp s: the data of its passes that the sweep does not change
    const int s = warp - 4 * G - 1;
    for (int k = s; k < n && !s_bad; k += FLOWC_STAGERS) {
      for (unsigned spin = 0; s_consumed < k - FLOWC_NBUF + 1 && !s_bad; ++spin)
        if (spin >= d.spin_limit) give_up();
      if (s_bad) break;
      const int pz = pass_of(k), sl = k % FLOWC_NBUF;
      PairPre<NSP>* pre = slot_pre(sl);
      FinC* fin = slot_fin(sl);
      int tg = f.pstart[pz];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int nc = f.gcell[pz * G + g], e0 = f.poff[pz * G + g], np = f.poff[pz * G + g + 1] - e0;
        PairPre<NSP> pl;
        pl.j = -1;
        pl.cs = 0;
        if (lane < np) {
          const int e = f.plist[e0 + lane];
          pl = k < nf ? pair_load<NSP, true>(d, e >> 2, e & 3, tg) : pair_load<NSP, false>(d, e >> 2, e & 3, tg);
        }
        pre[32 * g + lane] = pl;
        if (lane < CAP) {
          FinC fc = {-1, 0, 1.0, 1.0, 0.0};
          if (lane < nc) fc = k < nf ? finc_load<true>(d, tg + lane) : finc_load<false>(d, tg + lane);
          fin[CAP * g + lane] = fc;
        }
        tg += nc;
      }
      __syncwarp();
      __threadfence_block();
      if (lane == 0) s_slot[sl] = k + 1;
      __syncwarp();
    }
  } else if (warp == 4 * G) {
    // the coordinator
    auto staged = [&](int k) {  // wait (bounded) until pass k is staged
      for (unsigned spin = 0; s_slot[k % FLOWC_NBUF] != k + 1 && !s_bad; ++spin)
        if (spin >= d.spin_limit) give_up();
      __threadfence_block();
    };
    auto poll = [&](int k) {
      if (s_bad) return;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && wait_flag(f.pflag + f.deps[d0 + u], epoch, d.err, d.spin_limit);
      if (__any_sync(0xffffffffu, !ok)) give_up();
    };
    auto ready = [&](int k) -> bool {
      if (s_bad) return true;
      if (s_slot[k % FLOWC_NBUF] != k + 1) return false;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && ld_acquire(f.pflag + f.deps[d0 + u]) >= epoch;
      return __all_sync(0xffffffffu, ok) != 0;
    };
    // hand pass k over: the compute warps run it iff nothing gave up
    auto hand_over = [&](int k) {
      if (lane == 0) s_go[k % FLOWC_NBUF] = s_bad ? 0 : 1;
      __syncwarp();
      __threadfence_block();
      bar_arrive(3, T34);
    };
    if (n > 0) {
      staged(0);
      poll(0);
      hand_over(0);
    }
    for (int k = 0; k < n; ++k) {
      const bool more = k + 1 < n;
      const bool go = more && ready(k + 1);
      if (go) __threadfence_block();
      bar_named(4, T34);
      __threadfence_block();
      if (lane == 0) s_consumed = k + 1;  // pass k's slot is free
      if (go) hand_over(k + 1);
      if (lane == 0 && !s_bad) st_release(f.pflag + pass_of(k), epoch);
      if (more && !go) {
        poll(k + 1);
        staged(k + 1);
        hand_over(k + 1);
      }
    }
  } else {
    const int gi = threadIdx.x >> 7, role = (threadIdx.x >> 5) & 3;
    for (int k = 0; k < n; ++k) {
      bar_named(3, T34);
      const int sl = k % FLOWC_NBUF;
      // the group's first cell exists iff the group has work in this pass
      if (s_go[sl] && slot_fin(sl)[CAP * gi].i >= 0) {
        const PairPre<NSP> p = slot_pre(sl)[32 * gi + lane];
        const FinC fn = slot_fin(sl)[CAP * gi + min((role * 32 + lane) / V, CAP - 1)];
        double nbv[V];
#pragma unroll
        for (int v = 0; v < V; ++v) nbv[v] = p.j >= 0 ? __ldcg(d.hWA + (size_t)v * d.NE + p.j) : 0.0;
        if (k < nf) sweepc_compute<NSP, true, G>(d, th, p, nbv, fn);
        else sweepc_compute<NSP, false, G>(d, th, p, nbv, fn);
      }
      bar_arrive(4, T34);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(f.ctr + 1, 1u) == gridDim.x - 1) {
      f.ctr[1] = 0u;
      __threadfence();
      st_release(f.ctr, epoch);
    }
  }
}

template <int NSP, bool FWD>
__global__ void __launch_bounds__(32) k_sweep4(const Dev d, const ThermoDev<NSP> th, int t0, int t1) {
  pdl_launch_dependents();
  const int lt = threadIdx.x >> 2;
  __shared__ double wsm[32 * (3 + NSP)];
  const SweepPre<NSP> p = sweep_load<NSP, FWD>(d, lt < d.cpw ? t0 + blockIdx.x * d.cpw + lt : t1, t1, threadIdx.x & 3);
  pdl_wait();
  sweep_compute<NSP, FWD>(d, th, p, threadIdx.x & 3, wsm);
}

template <int NSP>
__global__ void __launch_bounds__(128) k_update(const Dev d, const ThermoDev<NSP> th) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  unsigned err = 0;
  update_cell<NSP>(d, th, i, err);
  flag(d, err);
}

// Both LU-SGS sweeps and the Newton update in one cooperative launch.  The
// levels of the forward sweep, then of the backward sweep, are cut into
// chunks of cpw cells (4 lanes each) dealt to the warps of the grid; a warp
// loads its next chunk's constant data, waits (bounded) until every chunk of
// the previous level is counted done, computes and counts its chunk.  Only
// warps with work in a level wait for the one before it, and each level's
// wait implies all earlier levels (each warp runs its levels in order).  The
// Newton update of all cells follows the last backward level.  cnt holds one
// counter per level (nf + nb), zeroed before the launch.
constexpr int PERS_THREADS = 256;
template <int NSP>
__global__ void __launch_bounds__(PERS_THREADS) k_lusgs_persistent(const Dev d, const ThermoDev<NSP> th,
                                                                   const int* __restrict__ foff, int nf,
                                                                   const int* __restrict__ boff, int nb,
                                                                   unsigned* cnt) {
  const int G = gridDim.x, wpb = PERS_THREADS / 32, w = threadIdx.x >> 5;
  const int gw = blockIdx.x + w * G, nw = G * wpb;
  const int lt = (threadIdx.x & 31) >> 2, q = threadIdx.x & 3;
  __shared__ double wsm_all[PERS_THREADS / 32][32 * (3 + NSP)];
  double* wsm = wsm_all[w];
  const int nl = nf + nb;
  // level L covers positions [lo(L), lo(L) + len(L)) of its sweep's tables
  auto lo = [&](int L) { return L < nf ? foff[L] : boff[L - nf]; };
  const int cpw = d.cpw;
  auto nchunks = [&](int L) {
    const int a = L < nf ? foff[L] : boff[L - nf], b = L < nf ? foff[L + 1] : boff[L - nf + 1];
    return (unsigned)((b - a + cpw - 1) / cpw);
  };
  for (int L = 0; L < nl; ++L) {
    const bool fwd = L < nf;
    const int t0 = lo(L), t1 = fwd ? foff[L + 1] : boff[L - nf + 1];
    const int nch = (t1 - t0 + cpw - 1) / cpw;
    if (gw >= nch) continue;
    bool waited = L == 0;
    for (int c = gw; c < nch; c += nw) {
      const int t = lt < cpw ? t0 + c * cpw + lt : t1;
      if (fwd) {
        const SweepPre<NSP> p = sweep_load<NSP, true>(d, t, t1, q);
        if (!waited) {
          if (!wait_count(cnt + L - 1, nchunks(L - 1), d.err, d.spin_limit)) return;
          waited = true;
        }
        sweep_compute<NSP, true>(d, th, p, q, wsm);
      } else {
        const SweepPre<NSP> p = sweep_load<NSP, false>(d, t, t1, q);
        if (!waited) {
          if (!wait_count(cnt + L - 1, nchunks(L - 1), d.err, d.spin_limit)) return;
          waited = true;
        }
        sweep_compute<NSP, false>(d, th, p, q, wsm);
      }
      count_done(cnt + L);
    }
  }
  // the update needs the whole backward sweep
  if (!wait_count(cnt + nl - 1, nchunks(nl - 1), d.err, d.spin_limit)) return;
  unsigned err = 0;
  for (int i = blockIdx.x * PERS_THREADS + threadIdx.x; i < d.NE; i += G * PERS_THREADS) update_cell<NSP>(d, th, i, err);
  flag(d, err);
}

// ------------------------------------------------------------ utilities ----
// Residual norms: fixed-shape deterministic reduction (block partials then one
// block over the partials).  out[k] = sum vol*|hWA_k|, out[V] = max WA_1.
constexpr int NRM_BLOCKS = 304, NRM_THREADS = 256;
// Case blockIdx.y covers cells [coff[y], coff[y+1]) (coff null: [0, NE)); the
// arrays have plane stride NE.  The order of the sums depends only on the
// case's own cells, so a case gives the same norms alone and in a batch.
__global__ void __launch_bounds__(NRM_THREADS) k_norm_partial(const double* __restrict__ hWA,
                                                              const double* __restrict__ WA,
                                                              const double* __restrict__ vol, int NE, int V,
                                                              const int* __restrict__ coff, double* part) {
  __shared__ double sh[NRM_THREADS];
  const int c0 = coff ? coff[blockIdx.y] : 0, n = coff ? coff[blockIdx.y + 1] - c0 : NE;
  part += (size_t)blockIdx.y * (V + 1) * NRM_BLOCKS;
  const int per = (n + NRM_BLOCKS - 1) / NRM_BLOCKS;
  const int lo = blockIdx.x * per, hi = min(n, lo + per);
  for (int k = 0; k <= V; ++k) {
    double a = (k == V) ? 0.0 : 0.0;
    for (int ii = lo + threadIdx.x; ii < hi; ii += NRM_THREADS) {
      const int i = c0 + ii;
      a = (k == V) ? fmax2(a, WA[i]) : a + vol[i] * fabs(hWA[k * NE + i]);
    }
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int w = NRM_THREADS / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sh[threadIdx.x] = (k == V) ? fmax2(sh[threadIdx.x], sh[threadIdx.x + w])
                                                      : sh[threadIdx.x] + sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[k * NRM_BLOCKS + blockIdx.x] = sh[0];
    __syncthreads();
  }
}
__global__ void k_norm_final(const double* part, int V, const double* __restrict__ total_volume, double* out) {
  const int k = threadIdx.x;
  if (k > V) return;
  part += (size_t)blockIdx.x * (V + 1) * NRM_BLOCKS;
  out += (size_t)blockIdx.x * (V + 1);
  double a = 0.0;
  for (int b = 0; b < NRM_BLOCKS; ++b) a = (k == V) ? fmax2(a, part[k * NRM_BLOCKS + b]) : a + part[k * NRM_BLOCKS + b];
  out[k] = (k == V) ? a : a / total_volume[blockIdx.x];
}

// Fortran (V,N) <-> device (V planes of N)
__global__ void k_aos_to_soa(const double* __restrict__ a, double* __restrict__ s, int N, int V) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * V) return;
  const int i = (int)(t / V), k = (int)(t % V);
  s[(long)k * N + i] = a[t];
}
__global__ void k_soa_to_aos(const double* __restrict__ s, double* __restrict__ a, int N, int V) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * V) return;
  const int i = (int)(t / V), k = (int)(t % V);
  a[t] = s[(long)k * N + i];
}

// Mixed-precision launchers (rc_mixed.cu).
template <int NSP> void mixed_ts_face(const Dev&, const void*, int, cudaStream_t);
template <int NSP> void mixed_cell(const Dev&, const void*, const ThermoDev<NSP>&, int, int, int, int, cudaStream_t);
template <int NSP> void mixed_face_flux(const Dev&, const void*, int, cudaStream_t);
template <int NSP> void mixed_gather(const Dev&, int, int, cudaStream_t);
template <int NSP> void mixed_pack(const Dev&, cudaStream_t);
template <int NSP> void mixed_sweep(const Dev&, const void*, bool, int, int, cudaStream_t);
template <int NSP> size_t mixed_thermo(const void*, void*);
template <int NSP>
cudaError_t mixed_lusgs_persistent(const Dev&, const void*, const int*, int, const int*, int, unsigned*, int,
                                   cudaStream_t);
template <int NSP> int mixed_persistent_occupancy();
template <int NSP>
cudaError_t mixed_lusgs_flow(const Dev&, const void*, const void*, const FlowDev&, int, cudaStream_t);
template <int NSP> int mixed_flow_occupancy();
template <int NSP>
cudaError_t mixed_lusgs_flowc(const Dev&, const void*, const void*, const FlowDev&, int, int, cudaStream_t);
template <int NSP> int mixed_flowc_occupancy(int);
template <int NSP>
void chem_source(const Dev&, const void*, double, int, int*, int*, unsigned*, unsigned*, cudaStream_t);
template <int NSP>
void chem_batch(const void*, const double*, const double*, int, double*, int*, double, int, unsigned*, unsigned*,
                cudaStream_t);
template <int NSP>
void chem_list(const Dev&, const void*, double, int, int*, const int*, const unsigned*, unsigned*, cudaStream_t);
template <int NSP> void bdf2_fixed(const Dev&, int, int, cudaStream_t);
template <int NSP> void bdf2_prep(const Dev&, const void*, int, cudaStream_t);
template <int NSP> void bdf2_sweep(const Dev&, const void*, bool, int, int, int, cudaStream_t);
template <int NSP> void bdf2_update(const Dev&, const void*, int, cudaStream_t);
template <int NSP> int bdf2_nbq();
template <int NSP> cudaError_t bdf2_flow(const Dev&, const void*, const FlowDev&, int, cudaStream_t);
template <int NSP> int bdf2_flow_occupancy();
cudaError_t surrogate_source(const Dev&, const void*, const rc_mlp*, float, int*, unsigned*, unsigned*, const int*,
                             unsigned char*, cudaStream_t);
cudaError_t surrogate_prepare();
cudaError_t surrogate_samples(const void*, const double*, const double*, const double*, int, float*, float*,
                              cudaStream_t);

}  // namespace rc

// ======================================================== host context =====
using namespace rc;

struct rc_ctx {
  int NE = 0, NF = 0, NG = 0, NSP = 0, V = 0;
  int visc = 0, comb = 0, limit = 0, precision = 0, device = 0;
  double total_volume = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Dev d{};
  std::vector<void*> allocs;
  std::vector<char> thermo;    // ThermoDev<NSP> bytes
  std::vector<char> thermo32;  // ThermoDev32<NSP> bytes (mixed precision)
  int mode = RC_PREC_FP64;     // current precision mode
  int* fwd_cells = nullptr;
  int* bwd_cells = nullptr;
  std::vector<int> fwd_off, bwd_off;
  bool persistent = false;      // LU-SGS sweeps as one cooperative launch with level counters
  bool can_persistent = false;  // the device can co-schedule the persistent LU-SGS grid
  int wide = 0;                 // FP64 per-level sweeps: 4 lanes per cell (0), 8 lanes (1, k_sweep8),
                                // the two parts of a slot in two warps (2, k_sweep2w) or four (3, k_sweep4w);
                                // 4: the dataflow launches k_lusgs_flow / k_lusgs_flow32 (where they
                                // cannot run: as 3 for FP64, the per-level sweeps for the mixed forms)
  bool can_flow[FLOW_GMAX] = {};  // the device can co-schedule the k_lusgs_flow grid (per G)
  bool can_flow32 = false;      // ... and the k_lusgs_flow32 grid (mixed forms)
  int flow_grid = 0;            // its blocks (one per SM)
  FlowDev flows[FLOW_GMAX] = {};  // its pass tables for G = 1..3 groups (passes of up to 8 G cells;
                                  // G = 1 is also the mixed forms' k_lusgs_flow32)
  int flow_g = 1;                 // the groups of the FP64 dataflow launch
  bool can_flowc[FLOWC_GMAX] = {};  // the device can co-schedule the k_lusgs_flowc grid (per G)
  FlowDev flowc[FLOWC_GMAX] = {};   // compact pass tables for G = 1, 2 groups
  bool flow_c = false;              // the dataflow launch is k_lusgs_flowc / k_lusgs_flowc32 (flow_g groups)
  bool can_flowc32[FLOWC_GMAX] = {};  // the device can co-schedule the k_lusgs_flowc32 grid (per G)
  int pers_grid = 0;             // blocks of the persistent launch (one per SM)
  unsigned* lvl_count = nullptr; // per-level completion counters of the persistent launch
  int nlevels = 0;
  int* fwd_off_dev = nullptr;
  int* bwd_off_dev = nullptr;
  // batch of independent cases sharing the numbering (ncase == 1: one case)
  int ncase = 1;
  std::vector<int> case_off;         // [ncase+1] cell offsets
  std::vector<double> case_vol;      // [ncase] total_volume of each case
  int* case_off_dev = nullptr;
  double* case_vol_dev = nullptr;
  // chemistry source mode (RC_CHEM_*) and the integrator's work arrays
  int chem = RC_CHEM_EXPLICIT;
  double chem_tol = 0.05;
  int chem_maxsub = 200;
  int* chem_nsub = nullptr;           // [NE] accepted substeps of the last integrated source
  int* chem_order = nullptr;          // [NE] cells by previous substeps, descending
  unsigned* chem_hist = nullptr;      // [256] bucket counts / cursors of that sort
  unsigned* chem_counter = nullptr;   // work-queue counter
  const rc_mlp* net = nullptr;        // surrogate (RC_CHEM_SURROGATE)
  float spread_tol = 0.02f;
  int* sur_list = nullptr;            // [NE] cells handed back to the integrator
  unsigned* sur_counts = nullptr;     // [2]: fallback cells, surrogate cells
  int* sur_mode = nullptr;            // [1]: 0 each cell decided per call, 1 decide and record, 2 recorded
  unsigned char* sur_dec = nullptr;   // [NE]: recorded decision, 1 = integrator
  bool sur_freeze_pending = false;    // switch sur_mode to 2 after the next stage
  cudaStream_t stream2 = nullptr;     // side stream: the integrated source runs beside the face fluxes
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

  // unsteady dual-time BDF2 (allocated by the first BDF2 call)
  bool bdf2_ready = false;
  int bdf2_cpw = 4;                        // BDF2 sweep cells per warp (1, 2 or 4; RC_BDF2_CPW)
  bool bdf2_flow = false;                  // BDF2 sweeps as one dataflow launch on flows[0]
                                           // (RC_BDF2_SCHEDULE=levels: one launch per level)
  double* bpar_dev = nullptr;              // {dt, phi}
  cudaGraphExec_t bdf2_graph = nullptr;    // one inner iteration and its norms
  long long bdf2_graph_kernels = 0;

  double* norm_part = nullptr;
  double* norm_out = nullptr;
  double* staging = nullptr;  // (V*max(NE,NF,NG)) for layout conversion
  cudaGraphExec_t graph = nullptr;       // graph of the current mode
  cudaGraphExec_t graphs[3] = {nullptr, nullptr, nullptr};
  long long graph_kernels_of[3] = {0, 0, 0};
  long long graph_kernels = 0;
  long long launches = 0;
  std::string err;
  int latched = 0;
};

namespace {

int cuda_fail(rc_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RC_OK;
  if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return RC_ERR_CUDA;
}
#define RC_CU(call)                                         \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call);  \
  } while (0)

// Allocations are filled on the context's stream and waited for: the stream
// is non-blocking, so a fill on the legacy stream would not be ordered before
// the context's kernels (and a pageable cudaMemcpy may return before its DMA
// has landed).
template <class T>
int dev_upload(rc_ctx* c, const std::vector<T>& h, T** out) {
  void* p = nullptr;
  size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
  RC_CU(cudaMalloc(&p, bytes));
  c->allocs.push_back(p);
  if (!h.empty()) {
    RC_CU(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    RC_CU(cudaStreamSynchronize(c->stream));
  }
  *out = static_cast<T*>(p);
  return RC_OK;
}
template <class T>
int dev_zeros(rc_ctx* c, size_t n, T** out) {
  void* p = nullptr;
  RC_CU(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  c->allocs.push_back(p);
  RC_CU(cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(T), c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  *out = static_cast<T*>(p);
  return RC_OK;
}

double hmax(double a, double b) { return (b > a) ? b : a; }

// ---- LU-SGS planning (host only)
// The level order of both sweeps over the reference cell order: forward, the
// level of cell i is 1 + the largest level of its neighbours j < i; backward,
// of its neighbours j > i.  cells[d] lists the cells level by level (ascending
// index inside a level), off[d] the level boundaries.  nface[i] faces,
// cother[q*NE + i] the cell across face q (-1 at a boundary).
struct SweepOrder {
  std::vector<int> cells[2], off[2];
};
template <class NF>
SweepOrder sweep_order(int NE, const NF& nface, const std::vector<int>& cother) {
  std::vector<int> lev[2] = {std::vector<int>(NE, 0), std::vector<int>(NE, 0)};
  int mx[2] = {0, 0};
  for (int i = 0; i < NE; ++i) {
    int l = 0;
    for (int q = 0; q < nface[i]; ++q) {
      const int j = cother[(size_t)q * NE + i];
      if (j >= 0 && j < i) l = std::max(l, lev[0][j] + 1);
    }
    lev[0][i] = l; mx[0] = std::max(mx[0], l);
  }
  for (int i = NE - 1; i >= 0; --i) {
    int l = 0;
    for (int q = 0; q < nface[i]; ++q) {
      const int j = cother[(size_t)q * NE + i];
      if (j > i) l = std::max(l, lev[1][j] + 1);
    }
    lev[1][i] = l; mx[1] = std::max(mx[1], l);
  }
  SweepOrder so;
  for (int d = 0; d < 2; ++d) {
    std::vector<int>& off = so.off[d];
    off.assign(mx[d] + 2, 0);
    for (int i = 0; i < NE; ++i) off[lev[d][i] + 1]++;
    for (int l = 0; l <= mx[d]; ++l) off[l + 1] += off[l];
    so.cells[d].assign(NE, 0);
    std::vector<int> pos(off.begin(), off.end() - 1);
    for (int i = 0; i < NE; ++i) so.cells[d][pos[lev[d][i]]++] = i;
  }
  return so;
}
// The dataflow schedule (k_lusgs_flow) over G blocks: block b owns the cells
// [b*C, (b+1)*C), C = ceil(NE/G); a pass is a run of at most `width`
// consecutive positions of one level whose cells one block owns (24 for the
// FP64 launch, three groups of 8; 8 for the mixed forms'); a block's passes are
// listed forward then backward in level order; a pass depends on the passes
// (same sweep) of the neighbours it reads that other blocks own.
//
// Compact passes (groups > 0, k_lusgs_flowc): the run is cut into up to
// `groups` groups of consecutive positions, each of at most `cap` cells
// and FLOWC_PAIRS active (position, slot) pairs, filled greedily; plist
// lists each group's pairs in (position, slot) order.
struct FlowPlan {
  int C = 1;
  std::vector<int> pstart, pcount, pdir, powner, plevel, doff, deps;
  std::vector<int> boff[2], blist[2];
  std::vector<int> cellpass[2];
  int groups = 0;
  std::vector<int> gcell, poff, plist;
};
// the slot q of cell i has a neighbour in sweep dir (0 forward: a lower one)
template <class NF>
inline bool sweep_slot(int NE, const NF& nface, const std::vector<int>& cother, int dir, int i, int q) {
  if (q >= nface[i]) return false;
  const int j = cother[(size_t)q * NE + i];
  return j >= 0 && (dir == 0 ? j < i : j > i);
}
template <class NF>
FlowPlan flow_plan(int NE, int G, const NF& nface, const std::vector<int>& cother, const SweepOrder& so,
                   int width = 8, int groups = 0, int cap = 0) {
  FlowPlan fp;
  fp.C = (NE + G - 1) / G;
  const int C = fp.C;
  fp.doff.assign(1, 0);
  fp.groups = groups;
  if (groups > 0) fp.poff.assign(1, 0);
  for (int dir = 0; dir < 2; ++dir) {
    const std::vector<int>& lst = so.cells[dir];
    const std::vector<int>& off = so.off[dir];
    fp.cellpass[dir].assign(NE, 0);
    std::vector<std::vector<int>> per(G);
    for (size_t l = 0; l + 1 < off.size(); ++l)
      for (int t = off[l]; t < off[l + 1];) {
        const int own = lst[t] / C;
        int e = t + 1;
        if (groups > 0) {
          e = t;
          for (int g = 0; g < groups; ++g) {
            int nc = 0, np = 0;
            while (e < off[l + 1] && lst[e] / C == own && nc < cap) {
              int a = 0;
              for (int q = 0; q < 4; ++q) a += sweep_slot(NE, nface, cother, dir, lst[e], q) ? 1 : 0;
              if (np + a > FLOWC_PAIRS) break;
              for (int q = 0; q < 4; ++q)
                if (sweep_slot(NE, nface, cother, dir, lst[e], q)) fp.plist.push_back(e << 2 | q);
              np += a;
              ++nc;
              ++e;
            }
            fp.gcell.push_back(nc);
            fp.poff.push_back((int)fp.plist.size());
          }
        } else {
          while (e < off[l + 1] && e - t < width && lst[e] / C == own) ++e;
        }
        const int pz = (int)fp.pstart.size();
        fp.pstart.push_back(t); fp.pcount.push_back(e - t); fp.pdir.push_back(dir); fp.powner.push_back(own);
        fp.plevel.push_back((int)l);
        per[own].push_back(pz);
        for (int u = t; u < e; ++u) fp.cellpass[dir][lst[u]] = pz;
        t = e;
      }
    fp.boff[dir].assign(1, 0);
    for (int bb = 0; bb < G; ++bb) {
      fp.blist[dir].insert(fp.blist[dir].end(), per[bb].begin(), per[bb].end());
      fp.boff[dir].push_back((int)fp.blist[dir].size());
    }
  }
  for (size_t pz = 0; pz < fp.pstart.size(); ++pz) {
    const int dir = fp.pdir[pz];
    const std::vector<int>& lst = so.cells[dir];
    const size_t d0 = fp.deps.size();
    for (int u = fp.pstart[pz]; u < fp.pstart[pz] + fp.pcount[pz]; ++u) {
      const int i = lst[u];
      for (int q = 0; q < nface[i]; ++q) {
        const int j = cother[(size_t)q * NE + i];
        if (j < 0 || (dir == 0 ? j >= i : j <= i) || j / C == fp.powner[pz]) continue;
        const int dp = fp.cellpass[dir][j];
        if (std::find(fp.deps.begin() + (long)d0, fp.deps.end(), dp) == fp.deps.end()) fp.deps.push_back(dp);
      }
    }
    fp.doff.push_back((int)fp.deps.size());
  }
  return fp;
}

template <int NSP>
void fill_thermo(const rc_thermo* t, const rc_config* g, ThermoDev<NSP>& th) {
  std::memset(&th, 0, sizeof(th));
  for (int i = 0; i < NSP; ++i) { th.R[i] = t->R_species[i]; th.mw[i] = t->mole_weight[i]; }
  th.Rconstant = t->Rconstant;
  th.tlo = t->thermo_lowest_tem; th.tcrit = t->thermo_critical_tem; th.thi = t->thermo_highest_tem;
  for (int j = 0; j < 7; ++j)
    for (int i = 0; i < NSP; ++i) {
      th.cl[j][i] = t->low_coef_Cp_species[j + 7 * i];
      th.ch[j][i] = t->high_coef_Cp_species[j + 7 * i];
    }
  for (int i = 0; i < NSP; ++i) { th.b1l[i] = t->low_enthalpy_b1[i]; th.b1h[i] = t->high_enthalpy_b1[i]; }
  th.trlo = t->transport_lowest_tem; th.trcrit = t->transport_critical_tem; th.trhi = t->transport_highest_tem;
  for (int a = 0; a < 4; ++a)
    for (int i = 0; i < NSP; ++i) {
      th.mu[0][a][i] = t->mu_K[a][i];
      th.mu[1][a][i] = t->mu_K[4 + a][i];
      th.kk[0][a][i] = t->mu_K[8 + a][i];
      th.kk[1][a][i] = t->mu_K[12 + a][i];
    }
  for (int i = 0; i < NSP; ++i)
    for (int j = 0; j < NSP; ++j) {
      const double mi = t->mole_weight[i], mj = t->mole_weight[j];
      th.wc[i][j] = rcm::pow(mj / mi, 0.25);
      th.wd[i][j] = std::sqrt(1. + mi / mj);
      th.dlj[i][j] = std::sqrt(t->LJ_energy[i] * t->LJ_energy[j]);
      th.dmw[i][j] = std::sqrt(2. / (1. / mi + 1. / mj) * 1000);
      const double cd = 0.5 * (t->collision_diameter[i] + t->collision_diameter[j]);
      th.dcd[i][j] = cd * cd;
    }
  th.model = t->code_chemical_model;
  th.Af = t->Af_react; th.E = t->E_react;
  for (int k = 0; k < NSP; ++k)
    th.prodc[k] = 1000 * t->mole_weight[k] * (t->coef_r_react[k] - t->coef_f_react[k]);
  th.mw1000[0] = t->mole_weight[0] * 1000;
  th.mw1000[1] = t->mole_weight[NSP > 1 ? 1 : 0] * 1000;
  th.cfl = g->cfl;
  // the device's recip_of, on the host (IEEE division, a correctly rounded FMA)
  auto rp = [](double x, double* r) {
    r[0] = 1.0 / x;
    r[1] = std::fma(-x, r[0], 1.0) * r[0];
  };
  for (int i = 0; i < NSP; ++i) {
    rp(th.mw[i], th.mwr[i]);
    for (int j = 0; j < NSP; ++j) {
      rp(th.wd[i][j], th.wdr[i][j]);
      rp(th.dlj[i][j], th.dljr[i][j]);
    }
  }
  rp(th.mw1000[0], th.mw1000r[0]);
  rp(th.mw1000[1], th.mw1000r[1]);
}

inline unsigned blocks(long n, int t) { return (unsigned)((n + t - 1) / t); }

template <int NSP>
const ThermoDev<NSP>& TH(const rc_ctx* c) { return *reinterpret_cast<const ThermoDev<NSP>*>(c->thermo.data()); }

// --- the pieces of one iteration, enqueued on c->stream
template <int NSP>
void q_timestep_face(rc_ctx* c) {
  if (c->visc) k_ts_face<NSP, true><<<blocks(c->NF, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, TH<NSP>(c));
  else k_ts_face<NSP, false><<<blocks(c->NF, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, TH<NSP>(c));
  c->launches++;
}
template <int NSP>
void q_cell(rc_ctx* c, int do_step, int do_recon) {
  k_cell<NSP><<<blocks(c->NE, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, TH<NSP>(c), do_step, do_recon, c->limit,
                                                          c->comb && c->chem == RC_CHEM_EXPLICIT, c->visc);
  c->launches++;
}
template <int NSP>
void q_face_flux(rc_ctx* c) {
  if (c->visc) k_face_flux<NSP, true><<<blocks(c->NF, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, TH<NSP>(c));
  else k_face_flux<NSP, false><<<blocks(c->NF, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, TH<NSP>(c));
  c->launches++;
}
template <int NSP>
void q_persistent(rc_ctx* c) {
  cudaMemsetAsync(c->lvl_count, 0, sizeof(unsigned) * c->nlevels, c->stream);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c->pers_grid);
  cfg.blockDim = dim3(PERS_THREADS);
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_lusgs_persistent<NSP>, c->d, TH<NSP>(c), (const int*)c->fwd_off_dev,
                     (int)c->fwd_off.size() - 1, (const int*)c->bwd_off_dev, (int)c->bwd_off.size() - 1,
                     c->lvl_count);
  c->launches++;
}
template <int NSP, int G>
void q_flow_g(rc_ctx* c) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c->flow_grid);
  cfg.blockDim = dim3(flow_threads(G));
  cfg.dynamicSmemBytes = (size_t)flow_dsmem<NSP, G>();
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_lusgs_flow<NSP, G>, c->d, TH<NSP>(c), c->flows[G - 1]);
}
template <int NSP, int G>
void q_flowc_g(rc_ctx* c) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c->flow_grid);
  cfg.blockDim = dim3(flowc_threads(G));
  cfg.dynamicSmemBytes = (size_t)flowc_dsmem<NSP, G>();
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_lusgs_flowc<NSP, G>, c->d, TH<NSP>(c), c->flowc[G - 1]);
}
// the FP64 dataflow launch the context runs, if the device can hold its grid
bool flow_runs(const rc_ctx* c) {
  return c->wide == 4 && (c->flow_c ? c->flow_g <= FLOWC_GMAX && c->can_flowc[c->flow_g - 1] : c->can_flow[c->flow_g - 1]);
}
template <int NSP>
void q_flow(rc_ctx* c) {
  if (c->flow_c) {
    if (c->flow_g == 2) q_flowc_g<NSP, 2>(c);
    else q_flowc_g<NSP, 1>(c);
  } else if (c->flow_g == 3) q_flow_g<NSP, 3>(c);
  else if (c->flow_g == 2) q_flow_g<NSP, 2>(c);
  else q_flow_g<NSP, 1>(c);
  c->launches++;
  launch_pdl(k_update<NSP>, blocks(c->NE, c->d.bs), c->d.bs, c->stream, c->d, TH<NSP>(c));
  c->launches++;
}
template <int NSP>
void q_sweeps(rc_ctx* c, int gather) {
  if (gather) {
    k_gather<NSP><<<blocks(c->NE, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, c->visc, c->comb);
    c->launches++;
  }
  if (c->persistent) { q_persistent<NSP>(c); return; }
  if (flow_runs(c)) { q_flow<NSP>(c); return; }
  for (size_t l = 0; l + 1 < c->fwd_off.size(); ++l) {
    const int n = c->fwd_off[l + 1] - c->fwd_off[l];
    if (c->wide >= 3) launch_pdl(k_sweep4w<NSP, true>, blocks(n, 8), 128, c->stream, c->d, TH<NSP>(c),
                                 c->fwd_off[l], c->fwd_off[l + 1]);
    else if (c->wide == 2) launch_pdl(k_sweep2w<NSP, true>, blocks(n, 8), 64, c->stream, c->d, TH<NSP>(c),
                                      c->fwd_off[l], c->fwd_off[l + 1]);
    else if (c->wide) launch_pdl(k_sweep8<NSP, true>, blocks(n, 4), 32, c->stream, c->d, TH<NSP>(c),
                                 c->fwd_off[l], c->fwd_off[l + 1]);
    else launch_pdl(k_sweep4<NSP, true>, blocks(n, c->d.cpw), 32, c->stream, c->d, TH<NSP>(c), c->fwd_off[l],
                    c->fwd_off[l + 1]);
    c->launches++;
  }
  for (size_t l = 0; l + 1 < c->bwd_off.size(); ++l) {
    const int n = c->bwd_off[l + 1] - c->bwd_off[l];
    if (c->wide >= 3) launch_pdl(k_sweep4w<NSP, false>, blocks(n, 8), 128, c->stream, c->d, TH<NSP>(c),
                                 c->bwd_off[l], c->bwd_off[l + 1]);
    else if (c->wide == 2) launch_pdl(k_sweep2w<NSP, false>, blocks(n, 8), 64, c->stream, c->d, TH<NSP>(c),
                                      c->bwd_off[l], c->bwd_off[l + 1]);
    else if (c->wide) launch_pdl(k_sweep8<NSP, false>, blocks(n, 4), 32, c->stream, c->d, TH<NSP>(c),
                                 c->bwd_off[l], c->bwd_off[l + 1]);
    else launch_pdl(k_sweep4<NSP, false>, blocks(n, c->d.cpw), 32, c->stream, c->d, TH<NSP>(c), c->bwd_off[l],
                    c->bwd_off[l + 1]);
    c->launches++;
  }
  launch_pdl(k_update<NSP>, blocks(c->NE, c->d.bs), c->d.bs, c->stream, c->d, TH<NSP>(c));
  c->launches++;
}
// Integrated chemical source on the side stream, forked after the cell pass
// and joined before the gather, so that it overlaps the face fluxes.
// With the surrogate, the network serves every cell it can and the
// integrator takes the cells its error indicator rejects.
template <int NSP>
void q_chem_fork(rc_ctx* c) {
  if (!c->comb || c->chem == RC_CHEM_EXPLICIT) return;
  cudaEventRecord(c->ev_fork, c->stream);
  cudaStreamWaitEvent(c->stream2, c->ev_fork, 0);
  if (c->chem == RC_CHEM_SURROGATE) {
    cudaMemsetAsync(c->sur_counts, 0, 2 * sizeof(unsigned), c->stream2);
    surrogate_source(c->d, c->thermo.data(), c->net, c->spread_tol, c->sur_list, c->sur_counts, c->sur_counts + 1,
                     c->sur_mode, c->sur_dec, c->stream2);
    chem_list<NSP>(c->d, c->thermo.data(), c->chem_tol, c->chem_maxsub, c->chem_nsub, c->sur_list, c->sur_counts,
                   c->chem_counter, c->stream2);
    c->launches += 2;
  } else {
    chem_source<NSP>(c->d, c->thermo.data(), c->chem_tol, c->chem_maxsub, c->chem_nsub, c->chem_order,
                     c->chem_hist, c->chem_counter, c->stream2);
    c->launches += 4;
  }
  cudaEventRecord(c->ev_join, c->stream2);
}
void q_chem_join(rc_ctx* c) {
  if (!c->comb || c->chem == RC_CHEM_EXPLICIT) return;
  cudaStreamWaitEvent(c->stream, c->ev_join, 0);
}
template <int NSP>
void q_gather(rc_ctx* c) {
  k_gather<NSP><<<blocks(c->NE, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, c->visc, c->comb);
  c->launches++;
}
// Sweeps of the mixed-precision modes: FP32 off-diagonal terms, FP64 division.
template <int NSP>
void q_sweeps32(rc_ctx* c) {
  if (!c->persistent && c->wide == 4 && c->flow_c && c->flow_g <= FLOWC_GMAX && c->can_flowc32[c->flow_g - 1]) {
    // compact passes; the Newton update runs inside the dataflow launch
    mixed_lusgs_flowc<NSP>(c->d, c->thermo32.data(), c->thermo.data(), c->flowc[c->flow_g - 1], c->flow_g,
                           c->flow_grid, c->stream);
    c->launches += 1;
    return;
  }
  if (!c->persistent && c->wide == 4 && c->can_flow32) {
    // the Newton update runs inside the dataflow launch
    mixed_lusgs_flow<NSP>(c->d, c->thermo32.data(), c->thermo.data(), c->flows[0], c->flow_grid, c->stream);
    c->launches += 1;
    return;
  }
  if (c->persistent) {
    cudaMemsetAsync(c->lvl_count, 0, sizeof(unsigned) * c->nlevels, c->stream);
    mixed_lusgs_persistent<NSP>(c->d, c->thermo32.data(), c->fwd_off_dev, (int)c->fwd_off.size() - 1, c->bwd_off_dev,
                                (int)c->bwd_off.size() - 1, c->lvl_count, c->pers_grid, c->stream);
    k_update<NSP><<<blocks(c->NE, c->d.bs), c->d.bs, 0, c->stream>>>(c->d, TH<NSP>(c));
    c->launches += 2;
    return;
  }
  for (size_t l = 0; l + 1 < c->fwd_off.size(); ++l) {
    mixed_sweep<NSP>(c->d, c->thermo32.data(), true, c->fwd_off[l], c->fwd_off[l + 1], c->stream);
    c->launches++;
  }
  for (size_t l = 0; l + 1 < c->bwd_off.size(); ++l) {
    mixed_sweep<NSP>(c->d, c->thermo32.data(), false, c->bwd_off[l], c->bwd_off[l + 1], c->stream);
    c->launches++;
  }
  launch_pdl(k_update<NSP>, blocks(c->NE, c->d.bs), c->d.bs, c->stream, c->d, TH<NSP>(c));
  c->launches++;
}
// The subroutines of one iteration in the current precision mode.
template <int NSP>
void q_timestep_mode(rc_ctx* c) {
  if (c->mode == RC_PREC_FP64) { q_timestep_face<NSP>(c); q_cell<NSP>(c, 1, 0); return; }
  mixed_ts_face<NSP>(c->d, c->thermo32.data(), c->visc, c->stream);
  c->launches++;
  q_cell<NSP>(c, 1, 0);
}
template <int NSP>
void q_reconstruction_mode(rc_ctx* c) {
  if (c->mode == RC_PREC_MIXED) {
    mixed_cell<NSP>(c->d, c->thermo32.data(), TH<NSP>(c), 0, c->limit, c->comb && c->chem == RC_CHEM_EXPLICIT,
                    c->visc, c->stream);
    c->launches++;
  } else {
    q_cell<NSP>(c, 0, 1);
    if (c->mode == RC_PREC_MIXED_DC) {
      mixed_pack<NSP>(c->d, c->stream);
      c->launches++;
    }
  }
}
template <int NSP>
void q_flux_mode(rc_ctx* c) {
  q_chem_fork<NSP>(c);
  if (c->mode == RC_PREC_MIXED) {
    mixed_face_flux<NSP>(c->d, c->thermo32.data(), c->visc, c->stream);
    q_chem_join(c);
    mixed_gather<NSP>(c->d, c->visc, c->comb, c->stream);
    c->launches += 2;
  } else {
    q_face_flux<NSP>(c);
    q_chem_join(c);
    q_gather<NSP>(c);
  }
}
template <int NSP>
void q_lusgs_mode(rc_ctx* c) {
  if (c->mode == RC_PREC_FP64) q_sweeps<NSP>(c, 0);
  else q_sweeps32<NSP>(c);
}
template <int NSP>
void q_stage(rc_ctx* c) {
  if (c->mode == RC_PREC_FP64) {
    q_timestep_face<NSP>(c);
    q_cell<NSP>(c, 1, 1);
    q_chem_fork<NSP>(c);
    q_face_flux<NSP>(c);
    q_chem_join(c);
    q_sweeps<NSP>(c, 1);
    return;
  }
  mixed_ts_face<NSP>(c->d, c->thermo32.data(), c->visc, c->stream);
  c->launches++;
  if (c->mode == RC_PREC_MIXED) {
    mixed_cell<NSP>(c->d, c->thermo32.data(), TH<NSP>(c), 1, c->limit, c->comb && c->chem == RC_CHEM_EXPLICIT,
                    c->visc, c->stream);
    c->launches++;
  } else {
    q_cell<NSP>(c, 1, 1);
    mixed_pack<NSP>(c->d, c->stream);
    c->launches++;
  }
  q_flux_mode<NSP>(c);
  q_sweeps32<NSP>(c);
}

// BDF2_LU_SGS after the residual assembly: per-cell set-up, the sweeps (one
// dataflow launch, or one launch per level), the primitive update.
template <int NSP>
void q_bdf2_lusgs(rc_ctx* c) {
  bdf2_prep<NSP>(c->d, c->thermo.data(), c->d.bs, c->stream);
  c->launches++;
  if (c->bdf2_flow) {
    bdf2_flow<NSP>(c->d, c->thermo.data(), c->flows[0], c->flow_grid, c->stream);
    c->launches++;
  }
  for (size_t l = 0; !c->bdf2_flow && l + 1 < c->fwd_off.size(); ++l) {
    bdf2_sweep<NSP>(c->d, c->thermo.data(), true, c->fwd_off[l], c->fwd_off[l + 1], c->bdf2_cpw, c->stream);
    c->launches++;
  }
  for (size_t l = 0; !c->bdf2_flow && l + 1 < c->bwd_off.size(); ++l) {
    bdf2_sweep<NSP>(c->d, c->thermo.data(), false, c->bwd_off[l], c->bwd_off[l + 1], c->bdf2_cpw, c->stream);
    c->launches++;
  }
  bdf2_update<NSP>(c->d, c->thermo.data(), c->d.bs, c->stream);
  c->launches++;
}
// Norms of every case into norm_out ([case][V+1]), enqueued.
void q_norms(rc_ctx* c) {
  const int nc = c->ncase;
  k_norm_partial<<<dim3(NRM_BLOCKS, nc), NRM_THREADS, 0, c->stream>>>(c->d.hWA, c->d.WA, c->d.vol, c->NE, c->V,
                                                                       nc > 1 ? c->case_off_dev : nullptr,
                                                                       c->norm_part);
  k_norm_final<<<nc, 32, 0, c->stream>>>(c->norm_part, c->V, c->case_vol_dev, c->norm_out);
  c->launches += 2;
}
// One inner iteration of BDF2_stage (Time_BDF2.f90:25-46) and the norms of
// inner_iteration_residual.
template <int NSP>
void q_bdf2_inner(rc_ctx* c) {
  q_timestep_face<NSP>(c);
  q_cell<NSP>(c, 1, 1);
  q_chem_fork<NSP>(c);
  q_face_flux<NSP>(c);
  q_chem_join(c);
  q_gather<NSP>(c);
  q_bdf2_lusgs<NSP>(c);
  q_norms(c);
}
// The residual assembly after the last inner iteration (Time_BDF2.f90:51-52).
template <int NSP>
void q_bdf2_final(rc_ctx* c) {
  q_cell<NSP>(c, 0, 1);
  q_chem_fork<NSP>(c);
  q_face_flux<NSP>(c);
  q_chem_join(c);
  q_gather<NSP>(c);
}

#define RC_DISPATCH(c, fn, ...)                  \
  switch ((c)->NSP) {                            \
    case 1: fn<1>(__VA_ARGS__); break;           \
    case 4: fn<4>(__VA_ARGS__); break;           \
    default: break;                              \
  }

int check_launch(rc_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  return cuda_fail(c, e, what);
}

int latch(rc_ctx* c) {
  unsigned h = 0;
  RC_CU(cudaMemcpyAsync(&h, c->d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  c->latched |= (int)h;
  if (h && c->err.empty()) c->err = "device-detected stop condition, code " + std::to_string(h);
  return c->latched;
}

}  // namespace

// ================================================================ C ABI =====
extern "C" {

}  // extern "C"

namespace {

// Boundary data and case layout of a context: one row of bctab per case (the
// BC_* offsets of rc_dev.cuh); fcase / gcase / case_off only for batches.
struct BatchDesc {
  std::vector<double> bctab;
  std::vector<int> fcase, gcase, case_off;
  std::vector<double> case_vol;
  int ncase() const { return (int)case_vol.size(); }
};

void bc_row_of(const rc_thermo* t, const rc_config* g, std::vector<double>& tab) {
  const size_t r = tab.size();
  tab.resize(r + BCS, 0.0);
  for (int k = 0; k < t->Nsp && k < BC_NSPMAX; ++k) {
    tab[r + BC_Y + k] = t->oxidizer_mass_fraction[k];
    tab[r + BC_Y + BC_NSPMAX + k] = t->fuel_mass_fraction[k];
  }
  tab[r + BC_T] = t->oxidizer_temp_in;
  tab[r + BC_T + 1] = t->fuel_temp_in;
  tab[r + BC_MFLOW] = t->oxidizer_mass_flow;
  tab[r + BC_MFLOW + 1] = t->fuel_mass_flow;
  tab[r + BC_POUT] = g->p_out;
}

// The module arrays of several cases renumbered into one mesh: cells, faces,
// nodes and ghosts of case c follow those of cases 0..c-1; every 1-based id is
// shifted by its case's offset, boundary codes (negative) are kept.
struct MergedMesh {
  rc_mesh m{};
  std::vector<int> KFace, Neighbor, FNode, FProperty, NeighF, Neigh, NeighC, Ghostcell, Num_ghostcell, Hostcell,
      BCtype;
  std::vector<double> COOR, VECX, SideOfs, VOL, CELLXY, reflen, wdis, AMLS, CoorG;
};

std::string merge_meshes(int n, const rc_mesh* ms, MergedMesh& o, BatchDesc& b) {
  const int M = ms[0].MaxNei;
  long long NE = 0, NF = 0, NNT = 0, NG = 0;
  for (int c = 0; c < n; ++c) {
    if (ms[c].MaxNei != M) return "MaxNei differs between cases";
    NE += ms[c].NE; NF += ms[c].NF; NNT += ms[c].NNT; NG += ms[c].Nghostcell;
  }
  if (NE > (1LL << 30) || NF > (1LL << 30) || NNT > (1LL << 30) || NG > (1LL << 30)) return "batch too large";
  auto sh = [](int v, int off) { return v > 0 ? v + off : v; };
  int oc = 0, of = 0, on = 0, og = 0;
  b.case_off.assign(1, 0);
  double vt = 0.0;
  for (int c = 0; c < n; ++c) {
    const rc_mesh& m = ms[c];
    for (int i = 0; i < m.NE; ++i) {
      o.KFace.push_back(m.KFace[i]);
      o.Neigh.push_back(m.Neigh[i]);
      o.Num_ghostcell.push_back(m.Num_ghostcell[i]);
      for (int q = 0; q < 4; ++q) o.NeighF.push_back(sh(m.NeighF[4 * (size_t)i + q], of));
      for (int q = 0; q <= M; ++q) o.NeighC.push_back(sh(m.NeighC[(size_t)(M + 1) * i + q], oc));
      for (int q = 0; q < M; ++q) o.Ghostcell.push_back(sh(m.Ghostcell[(size_t)M * i + q], og));
      o.VOL.push_back(m.VOL[i]);
      for (int r = 0; r < 2; ++r) {
        o.CELLXY.push_back(m.CELLXY[2 * (size_t)i + r]);
        o.reflen.push_back(m.reflen[2 * (size_t)i + r]);
      }
      for (int q = 0; q < M; ++q) o.wdis.push_back(m.wdis[(size_t)M * i + q]);
      for (int q = 0; q < 2 * M; ++q) o.AMLS.push_back(m.AMLS[(size_t)2 * M * i + q]);
    }
    for (int f = 0; f < m.NF; ++f) {
      o.Neighbor.push_back(sh(m.Neighbor[2 * (size_t)f], oc));
      o.Neighbor.push_back(sh(m.Neighbor[2 * (size_t)f + 1], oc));
      o.FNode.push_back(sh(m.FNode[2 * (size_t)f], on));
      o.FNode.push_back(sh(m.FNode[2 * (size_t)f + 1], on));
      o.FProperty.push_back(m.FProperty[f]);
      for (int r = 0; r < 2; ++r) {
        o.VECX.push_back(m.VECX[2 * (size_t)f + r]);
        o.SideOfs.push_back(m.SideOfs[2 * (size_t)f + r]);
      }
      b.fcase.push_back(c);
    }
    for (int k = 0; k < 2 * m.NNT; ++k) o.COOR.push_back(m.COOR[k]);
    for (int j = 0; j < m.Nghostcell; ++j) {
      o.Hostcell.push_back(sh(m.Hostcell[j], oc));
      o.BCtype.push_back(m.BCtype_Ghostcell[j]);
      for (int k = 0; k < 8; ++k) o.CoorG.push_back(m.Coor_Ghostnode[8 * (size_t)j + k]);
      b.gcase.push_back(c);
    }
    oc += m.NE; of += m.NF; on += m.NNT; og += m.Nghostcell;
    b.case_off.push_back(oc);
    b.case_vol.push_back(m.total_volume);
    vt = vt + m.total_volume;
  }
  rc_mesh& r = o.m;
  r.NE = oc; r.NF = of; r.NNT = on; r.MaxNei = M; r.Nghostcell = og;
  r.KFace = o.KFace.data(); r.Neighbor = o.Neighbor.data(); r.FNode = o.FNode.data();
  r.FProperty = o.FProperty.data(); r.NeighF = o.NeighF.data(); r.Neigh = o.Neigh.data();
  r.NeighC = o.NeighC.data(); r.Ghostcell = o.Ghostcell.data(); r.Num_ghostcell = o.Num_ghostcell.data();
  r.Hostcell = o.Hostcell.data(); r.BCtype_Ghostcell = o.BCtype.data(); r.COOR = o.COOR.data();
  r.VECX = o.VECX.data(); r.SideOfs = o.SideOfs.data(); r.VOL = o.VOL.data(); r.CELLXY = o.CELLXY.data();
  r.reflen = o.reflen.data(); r.wdis = o.wdis.data(); r.AMLS = o.AMLS.data(); r.Coor_Ghostnode = o.CoorG.data();
  r.total_volume = vt;
  return "";
}

// Species, thermo, transport, diffusion and kinetics data must agree between
// the cases of a batch (one ThermoDev); inlets and exit pressure may differ.
std::string same_gas(const rc_thermo* a, const rc_thermo* b, const rc_config* ga, const rc_config* gb) {
  if (a->Nsp != b->Nsp || a->order_of_cp_polynomial != b->order_of_cp_polynomial) return "species differ";
  const int n = a->Nsp, P = a->order_of_cp_polynomial;
  auto eq = [](const double* x, const double* y, int k) {
    for (int i = 0; i < k; ++i)
      if (!(x[i] == y[i])) return false;
    return true;
  };
  bool ok = a->Rconstant == b->Rconstant && eq(a->mole_weight, b->mole_weight, n) &&
            eq(a->R_species, b->R_species, n) && a->thermo_lowest_tem == b->thermo_lowest_tem &&
            a->thermo_critical_tem == b->thermo_critical_tem && a->thermo_highest_tem == b->thermo_highest_tem &&
            eq(a->low_coef_Cp_species, b->low_coef_Cp_species, n * P) &&
            eq(a->high_coef_Cp_species, b->high_coef_Cp_species, n * P) &&
            eq(a->low_enthalpy_b1, b->low_enthalpy_b1, n) && eq(a->high_enthalpy_b1, b->high_enthalpy_b1, n) &&
            a->transport_lowest_tem == b->transport_lowest_tem &&
            a->transport_critical_tem == b->transport_critical_tem &&
            a->transport_highest_tem == b->transport_highest_tem &&
            eq(a->collision_diameter, b->collision_diameter, n) && eq(a->LJ_energy, b->LJ_energy, n) &&
            a->code_chemical_model == b->code_chemical_model && eq(a->coef_f_react, b->coef_f_react, n) &&
            eq(a->coef_r_react, b->coef_r_react, n) && a->Af_react == b->Af_react && a->E_react == b->E_react;
  for (int k = 0; k < 16 && ok; ++k) ok = eq(a->mu_K[k], b->mu_K[k], n);
  if (!ok) return "gas data differ between cases";
  if (ga->IfViscous != gb->IfViscous || ga->If_turn_on_combustion != gb->If_turn_on_combustion ||
      ga->limit_ID != gb->limit_ID || ga->cfl != gb->cfl || ga->precision != gb->precision ||
      ga->device != gb->device)
    return "solver flags differ between cases (only p_out may)";
  return "";
}

int init_impl(const rc_mesh* m, const rc_thermo* t, const rc_config* g, const BatchDesc& b, rc_ctx** out) {
  *out = nullptr;
  rc_ctx* c = new rc_ctx();
  auto bail = [&](int code, const std::string& msg) {
    std::fprintf(stderr, "rc_init: %s\n", msg.c_str());
    rc_finalize(c);
    return code;
  };
  c->NE = m->NE; c->NF = m->NF; c->NG = m->Nghostcell; c->NSP = t->Nsp; c->V = 3 + t->Nsp;
  c->visc = g->IfViscous != 0; c->comb = g->If_turn_on_combustion != 0; c->limit = g->limit_ID;
  c->precision = g->precision; c->device = g->device; c->total_volume = m->total_volume;
  if ((int)b.bctab.size() != BCS * b.ncase() || b.ncase() < 1) return bail(RC_ERR_ARG, "bad case table");
  if (c->NSP != 1 && c->NSP != 4) return bail(RC_ERR_ARG, "Nsp must be 1 or 4 in this build");
  if (c->comb && c->NSP < 2) return bail(RC_ERR_ARG, "combustion needs at least two species");
  if (t->order_of_cp_polynomial != 7) return bail(RC_ERR_ARG, "order_of_cp_polynomial must be 7");
  if (m->MaxNei > MAXF) return bail(RC_ERR_ARG, "cells with more than 4 faces");
  if (g->precision != RC_PREC_FP64 && g->precision != RC_PREC_MIXED && g->precision != RC_PREC_MIXED_DC)
    return bail(RC_ERR_ARG, "unknown precision mode");
  if (cudaSetDevice(g->device) != cudaSuccess) return bail(RC_ERR_CUDA, "cudaSetDevice failed");
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(RC_ERR_CUDA, "cudaStreamCreate failed");
  c->own_stream = true;
  const int NE = m->NE, NF = m->NF, NG = m->Nghostcell, M = m->MaxNei, V = c->V;
  const double small = 1.0e-16;
  auto C2 = [&](const double* a, int d, int i) { return a[(size_t)(d - 1) + 2 * (size_t)(i - 1)]; };

  // ---- faces
  std::vector<int> fNL(NF), fNR(NF);
  std::vector<double> fvec(2 * (size_t)NF), fsav(NF), fsn(2 * (size_t)NF), fss(NF), fs2(NF), fvL(2 * (size_t)NF),
      fvR(2 * (size_t)NF), fdxk(NF), fdxkr(2 * (size_t)NF), fysn(2 * (size_t)NF);
  for (int f = 1; f <= NF; ++f) {
    const int L = m->Neighbor[2 * (f - 1)], R = m->Neighbor[2 * (f - 1) + 1];
    if (m->FProperty[f - 1] == 100) return bail(RC_ERR_ARG, "periodic faces are not supported");
    if (L < 1 || L > NE || R > NE) return bail(RC_ERR_ARG, "Neighbor out of range");
    const int fi = f - 1;
    fNL[fi] = L - 1;
    fNR[fi] = R > 0 ? R - 1 : R;
    const double dx = C2(m->VECX, 1, f), dy = C2(m->VECX, 2, f);
    fvec[fi] = dx; fvec[NF + fi] = dy;
    const double sav = hmax(std::sqrt(dx * dx + dy * dy), small);
    fsav[fi] = sav;
    fsn[fi] = dx / sav; fsn[NF + fi] = dy / sav;
    fss[fi] = std::sqrt(dx * dx + dy * dy);
    fs2[fi] = dx * dx + dy * dy;
    const int n1 = m->FNode[2 * (f - 1)], n2 = m->FNode[2 * (f - 1) + 1];
    // Gauss point xy = Coor(n1) + wxx*(Coor(n2)-Coor(n1)), wxx = 0.5 (initParam.f90:13)
    const double x = C2(m->COOR, 1, n1) + 0.5 * (C2(m->COOR, 1, n2) - C2(m->COOR, 1, n1));
    const double y = C2(m->COOR, 2, n1) + 0.5 * (C2(m->COOR, 2, n2) - C2(m->COOR, 2, n1));
    fvL[fi] = (x - C2(m->CELLXY, 1, L)) / C2(m->reflen, 1, L);
    fvL[NF + fi] = (y - C2(m->CELLXY, 2, L)) / C2(m->reflen, 2, L);
    if (R > 0) {
      fvR[fi] = (x - (C2(m->CELLXY, 1, R) - C2(m->SideOfs, 1, f))) / C2(m->reflen, 1, R);
      fvR[NF + fi] = (y - (C2(m->CELLXY, 2, R) - C2(m->SideOfs, 2, f))) / C2(m->reflen, 2, R);
      const double dlrx = C2(m->CELLXY, 1, L) - (C2(m->CELLXY, 1, R) - C2(m->SideOfs, 1, f));
      const double dlry = C2(m->CELLXY, 2, L) - (C2(m->CELLXY, 2, R) - C2(m->SideOfs, 2, f));
      fdxk[fi] = std::fabs(dlrx * fsn[fi] + dlry * fsn[NF + fi]);
      fdxkr[fi] = 1.0 / fdxk[fi];
      fdxkr[NF + fi] = std::fma(-fdxk[fi], fdxkr[fi], 1.0) * fdxkr[fi];
    }
    const double yita = 4. / 3;
    fysn[fi] = yita * fsn[fi];
    fysn[NF + fi] = yita * fsn[NF + fi];
  }
  // ---- cells
  std::vector<unsigned char> nface(NE), cleft(NE, 0), nnei(NE), ngh(NE);
  std::vector<int> cface(4 * (size_t)NE, 0), cother(4 * (size_t)NE, -1), cnei(4 * (size_t)NE, 0), cgh(4 * (size_t)NE, 0);
  std::vector<double> vol(NE), rinv(2 * (size_t)NE), wd(4 * (size_t)NE, 0.0), am(8 * (size_t)NE, 0.0),
      lvvh(8 * (size_t)NE, 0.0);
  for (int i = 1; i <= NE; ++i) {
    const int ii = i - 1, kf = m->KFace[ii];
    if (kf < 3 || kf > 4) return bail(RC_ERR_ARG, "KFace must be 3 or 4");
    nface[ii] = (unsigned char)kf;
    vol[ii] = m->VOL[ii];
    rinv[ii] = 1. / C2(m->reflen, 1, i);
    rinv[NE + ii] = 1. / C2(m->reflen, 2, i);
    for (int q = 0; q < kf; ++q) {
      const int f = m->NeighF[4 * (size_t)ii + q];
      if (f < 1 || f > NF) return bail(RC_ERR_ARG, "NeighF out of range");
      cface[(size_t)q * NE + ii] = f - 1;
      const int L = m->Neighbor[2 * (f - 1)], R = m->Neighbor[2 * (f - 1) + 1];
      if (L == i) {
        cleft[ii] |= (unsigned char)(1u << q);
        cother[(size_t)q * NE + ii] = R > 0 ? R - 1 : -1;
      } else {
        cother[(size_t)q * NE + ii] = L - 1;
      }
      const int n1 = m->FNode[2 * (f - 1)], n2 = m->FNode[2 * (f - 1) + 1];
      const double x = 0.5 * (C2(m->COOR, 1, n1) + C2(m->COOR, 1, n2));
      const double y = 0.5 * (C2(m->COOR, 2, n1) + C2(m->COOR, 2, n2));
      lvvh[(size_t)(2 * q) * NE + ii] = (x - C2(m->CELLXY, 1, i)) / C2(m->reflen, 1, i);
      lvvh[(size_t)(2 * q + 1) * NE + ii] = (y - C2(m->CELLXY, 2, i)) / C2(m->reflen, 2, i);
    }
    const int nn = m->Neigh[ii], ng = m->Num_ghostcell[ii];
    if (nn + ng != kf) return bail(RC_ERR_ARG, "Neigh + Num_ghostcell /= KFace");
    nnei[ii] = (unsigned char)nn;
    ngh[ii] = (unsigned char)ng;
    for (int q = 0; q < nn; ++q) {
      const int j = m->NeighC[(size_t)(M + 1) * ii + q + 1];
      if (j < 1 || j > NE) return bail(RC_ERR_ARG, "NeighC out of range");
      cnei[(size_t)q * NE + ii] = j - 1;
    }
    for (int q = 0; q < ng; ++q) {
      const int gj = m->Ghostcell[(size_t)M * ii + q];
      if (gj < 1 || gj > NG || m->Hostcell[gj - 1] != i) return bail(RC_ERR_ARG, "Ghostcell/Hostcell mismatch");
      cgh[(size_t)q * NE + ii] = gj - 1;
    }
    for (int q = 0; q < kf; ++q) {
      wd[(size_t)q * NE + ii] = m->wdis[(size_t)M * ii + q];
      am[(size_t)(2 * q) * NE + ii] = m->AMLS[(size_t)2 * M * ii + 2 * q];
      am[(size_t)(2 * q + 1) * NE + ii] = m->AMLS[(size_t)2 * M * ii + 2 * q + 1];
    }
  }
  // ---- ghosts: unit normal of the ghost face (update_flow_variables.f90:114-128)
  std::vector<int> gtype(NG);
  std::vector<double> gsn(2 * (size_t)NG);
  for (int j = 0; j < NG; ++j) {
    gtype[j] = m->BCtype_Ghostcell[j];
    const double* G = &m->Coor_Ghostnode[8 * (size_t)j];
    const double sav1 = G[3] - G[1];
    const double sav2 = -(G[2] - G[0]);
    const double sav = hmax(std::sqrt(sav1 * sav1 + sav2 * sav2), small);
    gsn[j] = sav1 / sav;
    gsn[NG + j] = sav2 / sav;
  }
  // ---- LU-SGS levels over the reference cell order
  const SweepOrder so = sweep_order(NE, nface, cother);
  const std::vector<int>& fc = so.cells[0];
  const std::vector<int>& bc = so.cells[1];
  c->fwd_off = so.off[0];
  c->bwd_off = so.off[1];

  // ---- thermo tables
  if (c->NSP == 1) {
    c->thermo.resize(sizeof(ThermoDev<1>));
    fill_thermo<1>(t, g, *reinterpret_cast<ThermoDev<1>*>(c->thermo.data()));
    c->thermo32.resize(mixed_thermo<1>(nullptr, nullptr));
    mixed_thermo<1>(c->thermo.data(), c->thermo32.data());
  } else {
    c->thermo.resize(sizeof(ThermoDev<4>));
    fill_thermo<4>(t, g, *reinterpret_cast<ThermoDev<4>*>(c->thermo.data()));
    c->thermo32.resize(mixed_thermo<4>(nullptr, nullptr));
    mixed_thermo<4>(c->thermo.data(), c->thermo32.data());
  }
  c->mode = g->precision;

  // ---- upload
  Dev& d = c->d;
  d.NE = NE; d.NF = NF; d.NG = NG;
  d.bs = 128;
  d.cpw = 8;
  d.spin_limit = 1u << 24;
  if (const char* e = std::getenv("RC_LUSGS_CPW")) {
    const int v = std::atoi(e);
    if (v == 1 || v == 2 || v == 4 || v == 8) d.cpw = v;
  }
  int st = 0;
  double* p;
  unsigned char* u8;
  int* i32;
  st |= dev_upload(c, vol, &p); d.vol = p;
  st |= dev_upload(c, rinv, &p); d.rinv = p;
  st |= dev_upload(c, nface, &u8); d.nface = u8;
  st |= dev_upload(c, cleft, &u8); d.cleft = u8;
  st |= dev_upload(c, cface, &i32); d.cface = i32;
  st |= dev_upload(c, cother, &i32); d.cother = i32;
  st |= dev_upload(c, nnei, &u8); d.nnei = u8;
  st |= dev_upload(c, cnei, &i32); d.cnei = i32;
  st |= dev_upload(c, ngh, &u8); d.ngh = u8;
  st |= dev_upload(c, cgh, &i32); d.cgh = i32;
  st |= dev_upload(c, wd, &p); d.wdis = p;
  st |= dev_upload(c, am, &p); d.amls = p;
  st |= dev_upload(c, lvvh, &p); d.lvvh = p;
  st |= dev_upload(c, fNL, &i32); d.fNL = i32;
  st |= dev_upload(c, fNR, &i32); d.fNR = i32;
  st |= dev_upload(c, fvec, &p); d.fvec = p;
  st |= dev_upload(c, fsav, &p); d.fsav = p;
  st |= dev_upload(c, fsn, &p); d.fsn = p;
  st |= dev_upload(c, fss, &p); d.fss = p;
  st |= dev_upload(c, fs2, &p); d.fs2 = p;
  st |= dev_upload(c, fvL, &p); d.fvL = p;
  st |= dev_upload(c, fvR, &p); d.fvR = p;
  st |= dev_upload(c, fdxk, &p); d.fdxk = p;
  st |= dev_upload(c, fdxkr, &p); d.fdxkr = p;
  st |= dev_upload(c, fysn, &p); d.fysn = p;
  st |= dev_upload(c, gtype, &i32); d.gtype = i32;
  st |= dev_upload(c, gsn, &p); d.gsn = p;
  st |= dev_upload(c, fc, &c->fwd_cells);
  st |= dev_upload(c, bc, &c->bwd_cells);
  st |= dev_zeros(c, (size_t)V * NE, &d.PA);
  st |= dev_zeros(c, (size_t)V * NE, &d.WA);
  st |= dev_zeros(c, (size_t)V * NE, &d.hWA);
  st |= dev_zeros(c, (size_t)2 * V * NE, &d.grad);
  st |= dev_zeros(c, (size_t)V * std::max(NG, 1), &d.GPA);
  st |= dev_zeros(c, (size_t)NE, &d.step);
  st |= dev_zeros(c, (size_t)NE, &d.dd);
  st |= dev_zeros(c, (size_t)(3 + c->NSP) * NE, &d.cst);
  st |= dev_zeros(c, (size_t)6 * NE, &d.rcp);
  st |= dev_zeros(c, (size_t)std::max(c->NSP - 1, 1) * NE, &d.src);
  st |= dev_zeros(c, (size_t)NF, &d.alpa);
  st |= dev_zeros(c, (size_t)NF, &d.visL);
  st |= dev_zeros(c, (size_t)NF, &d.visR);
  st |= dev_zeros(c, (size_t)NF, &d.alpaF);
  st |= dev_zeros(c, (size_t)V * NF, &d.Finv);
  st |= dev_zeros(c, (size_t)(V - 1) * NF, &d.Fvis);
  st |= dev_zeros(c, (size_t)b.ncase() * (V + 1) * NRM_BLOCKS, &c->norm_part);
  st |= dev_zeros(c, (size_t)b.ncase() * (V + 1), &c->norm_out);
  st |= dev_zeros(c, (size_t)2 * V * std::max(std::max(NE, NF), NG), &c->staging);
  if (g->precision != RC_PREC_FP64) {  // FP32 work arrays of the mixed modes
    double* f32;
    st |= dev_zeros(c, ((size_t)2 * V * NE + 1) / 2, &f32); d.grad32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)V * std::max(NG, 1) + 1) / 2, &f32); d.GPA32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)V * NF + 1) / 2, &f32); d.Finv32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)(V - 1) * NF + 1) / 2, &f32); d.Fvis32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)V * NE + 1) / 2, &f32); d.PA32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)(3 + c->NSP) * NE + 1) / 2, &f32); d.cst32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)V * NE + 1) / 2, &f32); d.dU32 = reinterpret_cast<float*>(f32);
    st |= dev_zeros(c, ((size_t)NF + 1) / 2, &f32); d.alpaF32 = reinterpret_cast<float*>(f32);
    std::vector<float> fv32(fvec.begin(), fvec.end());
    float* fv;
    st |= dev_upload(c, fv32, &fv); d.fvec32 = fv;
  }
  double* e;
  st |= dev_zeros(c, 1, &e);
  d.err = reinterpret_cast<unsigned*>(e);
  c->nlevels = (int)(c->fwd_off.size() + c->bwd_off.size()) - 2;
  st |= dev_zeros(c, (size_t)std::max(c->nlevels, 1), &c->lvl_count);
  st |= dev_upload(c, c->fwd_off, &c->fwd_off_dev);
  st |= dev_upload(c, c->bwd_off, &c->bwd_off_dev);
  {  // sweep tables in level order
    for (int dir = 0; dir < 2; ++dir) {
      const std::vector<int>& lst = dir == 0 ? fc : bc;
      std::vector<int> ti(NE), tj(4 * (size_t)NE, -1), tf(4 * (size_t)NE, 0);
      for (int t = 0; t < NE; ++t) {
        const int i = lst[t];
        ti[t] = i;
        for (int q = 0; q < nface[i]; ++q) {
          const int j = cother[(size_t)q * NE + i];
          if (j >= 0 && (dir == 0 ? j < i : j > i)) {
            tj[(size_t)q * NE + t] = j;
            const int f = cface[(size_t)q * NE + i];
            tf[(size_t)q * NE + t] = ((cleft[i] >> q) & 1u) ? f : ~f;
          }
        }
      }
      int* p;
      st |= dev_upload(c, ti, &p); d.swi[dir] = p;
      st |= dev_upload(c, tj, &p); d.swj[dir] = p;
      st |= dev_upload(c, tf, &p); d.swf[dir] = p;
    }
  }
  {  // dataflow schedule of the sweeps (k_lusgs_flow), one block per SM
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, g->device);
    const int G = std::max(nsm, 1);
    for (int gr = 1; gr <= FLOW_GMAX + FLOWC_GMAX; ++gr) {
      // G = 1..3 groups of 8 positions, then the compact plans of 1..2 groups
      const int cg = gr > FLOW_GMAX ? gr - FLOW_GMAX : 0;
      const int cap = flowc_cells(c->V);
      FlowPlan fp = cg ? flow_plan(NE, G, nface, cother, so, cap * cg, cg, cap) : flow_plan(NE, G, nface, cother, so, 8 * gr);
      std::vector<int>& pstart = fp.pstart;
      std::vector<int>& pcount = fp.pcount;
      std::vector<int>& doff = fp.doff;
      std::vector<int>& deps = fp.deps;
      std::vector<int>* boff = fp.boff;
      std::vector<int>* blist = fp.blist;
      FlowDev& f = cg ? c->flowc[cg - 1] : c->flows[gr - 1];
      int* ip;
      if (cg) {
        st |= dev_upload(c, fp.gcell, &ip); f.gcell = ip;
        st |= dev_upload(c, fp.poff, &ip); f.poff = ip;
        if (fp.plist.empty()) fp.plist.push_back(0);
        st |= dev_upload(c, fp.plist, &ip); f.plist = ip;
      }
      st |= dev_upload(c, pstart, &ip); f.pstart = ip;
      st |= dev_upload(c, pcount, &ip); f.pcount = ip;
      for (int dir = 0; dir < 2; ++dir) {
        st |= dev_upload(c, boff[dir], &ip); f.boff[dir] = ip;
        st |= dev_upload(c, blist[dir], &ip); f.blist[dir] = ip;
      }
      st |= dev_upload(c, doff, &ip); f.doff = ip;
      if (deps.empty()) deps.push_back(0);
      st |= dev_upload(c, deps, &ip); f.deps = ip;
      st |= dev_upload(c, std::vector<unsigned>(pstart.size() + 1, 0u), &f.pflag);
      st |= dev_upload(c, std::vector<unsigned>(2, 0u), &f.ctr);
    }
    c->flow_grid = G;
  }
  {  // boundary data per case, case layout
    std::vector<float> tab32(b.bctab.begin(), b.bctab.end());
    double* tp;
    float* tp32;
    st |= dev_upload(c, b.bctab, &tp); d.bctab = tp;
    st |= dev_upload(c, tab32, &tp32); d.bctab32 = tp32;
    c->ncase = b.ncase();
    c->case_off = b.case_off;
    c->case_vol = b.case_vol;
    st |= dev_upload(c, c->case_off, &c->case_off_dev);
    st |= dev_upload(c, c->case_vol, &c->case_vol_dev);
    int* ip;
    if (!b.fcase.empty()) { st |= dev_upload(c, b.fcase, &ip); d.fcase = ip; }
    if (!b.gcase.empty()) { st |= dev_upload(c, b.gcase, &ip); d.gcase = ip; }
  }
  if (st) return bail(st, c->err);
  // LU-SGS schedule: which cooperative kernels every SM can hold a block of,
  // and the schedule RC_LUSGS_SCHEDULE names (rc_autotune may change it).
  {
    int nsm = 0, occ64 = 0, occ32 = 0, coop = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, g->device);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device);
    if (c->NSP == 1) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, k_lusgs_persistent<1>, PERS_THREADS, 0);
      occ32 = mixed_persistent_occupancy<1>();
    } else {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, k_lusgs_persistent<4>, PERS_THREADS, 0);
      occ32 = mixed_persistent_occupancy<4>();
    }
    const char* sched = std::getenv("RC_LUSGS_SCHEDULE");
    c->pers_grid = nsm;
    c->can_persistent = coop && nsm > 0 && occ64 >= 1 && occ32 >= 1;
    // default (no or another value): the dataflow launches (where they cannot
    // run: the four-warp per-level sweeps for FP64, the per-level sweeps for
    // the mixed forms)
    const std::string sc = sched ? sched : "";
    c->persistent = c->can_persistent && sc == "persistent";
    c->wide = sc == "levels" ? 0 : sc == "levels8" ? 1 : sc == "levels2w" ? 2 : sc == "levels4w" ? 3 : 4;
    c->flow_g = sc == "flow3" ? 3 : sc == "flow2" || sc == "flowc2" ? 2 : 1;
    c->flow_c = sc == "flowc" || sc == "flowc2";
    auto occ_flow = [&](auto kern, int threads, int dsmem) {
      int o = 0;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dsmem);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, threads, dsmem);
      return coop && nsm > 0 && o >= 1 && c->flow_grid == nsm;
    };
    if (c->NSP == 1) {
      c->can_flow[0] = occ_flow(k_lusgs_flow<1, 1>, flow_threads(1), flow_dsmem<1, 1>());
      c->can_flow[1] = occ_flow(k_lusgs_flow<1, 2>, flow_threads(2), flow_dsmem<1, 2>());
      c->can_flow[2] = occ_flow(k_lusgs_flow<1, 3>, flow_threads(3), flow_dsmem<1, 3>());
      c->can_flowc[0] = occ_flow(k_lusgs_flowc<1, 1>, flowc_threads(1), flowc_dsmem<1, 1>());
      c->can_flowc[1] = occ_flow(k_lusgs_flowc<1, 2>, flowc_threads(2), flowc_dsmem<1, 2>());
    } else {
      c->can_flow[0] = occ_flow(k_lusgs_flow<4, 1>, flow_threads(1), flow_dsmem<4, 1>());
      c->can_flow[1] = occ_flow(k_lusgs_flow<4, 2>, flow_threads(2), flow_dsmem<4, 2>());
      c->can_flow[2] = occ_flow(k_lusgs_flow<4, 3>, flow_threads(3), flow_dsmem<4, 3>());
      c->can_flowc[0] = occ_flow(k_lusgs_flowc<4, 1>, flowc_threads(1), flowc_dsmem<4, 1>());
      c->can_flowc[1] = occ_flow(k_lusgs_flowc<4, 2>, flowc_threads(2), flowc_dsmem<4, 2>());
    }
    cudaGetLastError();  // an attribute or occupancy query that failed leaves can_flow false
    occ32 = c->NSP == 1 ? mixed_flow_occupancy<1>() : mixed_flow_occupancy<4>();
    c->can_flow32 = coop && nsm > 0 && occ32 >= 1 && c->flow_grid == nsm;
    for (int g = 1; g <= FLOWC_GMAX; ++g) {
      const int o = c->NSP == 1 ? mixed_flowc_occupancy<1>(g) : mixed_flowc_occupancy<4>(g);
      c->can_flowc32[g - 1] = coop && nsm > 0 && o >= 1 && c->flow_grid == nsm;
    }
    cudaGetLastError();
  }
  *out = c;
  return RC_OK;
}

}  // namespace

// The plan with passes of up to `width` positions; stats as rc_flow_plan_check.
// groups > 0: the compact plan of that many groups of at most `cap` cells.
int flow_plan_check_width(int ne, int nblocks, const std::vector<int>& nf, const std::vector<int>& co,
                          const SweepOrder& so, int width, long long* stats, int groups = 0, int cap = 0) {
  const FlowPlan fp = groups > 0 ? flow_plan(ne, nblocks, nf, co, so, cap * groups, groups, cap)
                                 : flow_plan(ne, nblocks, nf, co, so, width);
  if (groups > 0) width = cap * groups;
  const int P = (int)fp.pstart.size(), C = fp.C;
  bool ok = true;
  long long npass[2] = {0, 0}, maxdep = 0;
  // compact plans: the groups of a pass split its positions in order; a
  // group holds at most `cap` cells and lists exactly their active
  // (position, slot) pairs, at most FLOWC_PAIRS, in (position, slot) order
  if (groups > 0) {
    if ((int)fp.gcell.size() != P * groups || (int)fp.poff.size() != P * groups + 1 || fp.poff[0] != 0) ok = false;
    for (int pz = 0; pz < P && ok; ++pz) {
      const int dir = fp.pdir[pz];
      int t = fp.pstart[pz], tot = 0;
      for (int g = 0; g < groups && ok; ++g) {
        const int nc = fp.gcell[pz * groups + g], e0 = fp.poff[pz * groups + g], e1 = fp.poff[pz * groups + g + 1];
        if (nc < 0 || nc > cap || e1 - e0 < 0 || e1 - e0 > FLOWC_PAIRS) { ok = false; break; }
        int e = e0;
        for (int u = t; u < t + nc && ok; ++u)
          for (int q = 0; q < 4 && ok; ++q)
            if (sweep_slot(ne, nf, co, dir, so.cells[dir][u], q)) ok = e < e1 && fp.plist[e++] == (u << 2 | q);
        if (e != e1) ok = false;
        t += nc;
        tot += nc;
      }
      if (tot != fp.pcount[pz]) ok = false;
    }
  }
  // every cell in exactly one pass per sweep; a pass is 1..8 positions of one
  // level, all owned by its block
  for (int dir = 0; dir < 2 && ok; ++dir) {
    std::vector<int> seen(ne, 0);
    for (int pz = 0; pz < P; ++pz) {
      if (fp.pdir[pz] != dir) continue;
      ++npass[dir];
      const int l = fp.plevel[pz], t0 = fp.pstart[pz], n = fp.pcount[pz];
      if (n < 1 || n > width || t0 < so.off[dir][l] || t0 + n > so.off[dir][l + 1]) ok = false;
      for (int u = t0; u < t0 + n && ok; ++u) {
        const int i = so.cells[dir][u];
        if (i / C != fp.powner[pz] || fp.cellpass[dir][i] != pz) ok = false;
        ++seen[i];
      }
    }
    for (int i = 0; i < ne && ok; ++i) ok = seen[i] == 1;
  }
  // dependencies: passes of the same sweep, other blocks, lower levels, and
  // every neighbour the pass reads from another block
  for (int pz = 0; pz < P && ok; ++pz) {
    const int dir = fp.pdir[pz];
    maxdep = std::max<long long>(maxdep, fp.doff[pz + 1] - fp.doff[pz]);
    for (int k = fp.doff[pz]; k < fp.doff[pz + 1]; ++k) {
      const int dp = fp.deps[k];
      if (dp < 0 || dp >= P || fp.pdir[dp] != dir || fp.powner[dp] == fp.powner[pz] || fp.plevel[dp] >= fp.plevel[pz])
        ok = false;
    }
    for (int u = fp.pstart[pz]; u < fp.pstart[pz] + fp.pcount[pz] && ok; ++u) {
      const int i = so.cells[dir][u];
      for (int q = 0; q < nf[i]; ++q) {
        const int j = co[(size_t)q * ne + i];
        if (j < 0 || (dir == 0 ? j >= i : j <= i)) continue;
        const int jp = fp.cellpass[dir][j];
        if (j / C == i / C) {
          if (fp.plevel[jp] >= fp.plevel[pz]) ok = false;  // done earlier by the same block
        } else if (std::find(fp.deps.begin() + fp.doff[pz], fp.deps.begin() + fp.doff[pz + 1], jp) ==
                   fp.deps.begin() + fp.doff[pz + 1]) {
          ok = false;
        }
      }
    }
  }
  // the blocks' sequences (forward then backward, each in level order); run
  // the protocol in synchronous steps: every block finishes its next pass
  // once the passes it depends on are done.  A step without progress is a
  // deadlock.
  std::vector<std::vector<int>> seq(nblocks);
  for (int b = 0; b < nblocks && ok; ++b) {
    for (int dir = 0; dir < 2; ++dir)
      for (int k = fp.boff[dir][b]; k < fp.boff[dir][b + 1]; ++k) {
        const int pz = fp.blist[dir][k];
        if (fp.powner[pz] != b || fp.pdir[pz] != dir ||
            (k > fp.boff[dir][b] && fp.plevel[fp.blist[dir][k - 1]] > fp.plevel[pz]))
          ok = false;
        seq[b].push_back(pz);
      }
  }
  long long steps = 0;
  if (ok) {
    std::vector<char> done(P, 0);
    std::vector<size_t> at(nblocks, 0);
    long long left = P;
    std::vector<int> fin;
    while (left > 0) {
      fin.clear();
      for (int b = 0; b < nblocks; ++b) {
        if (at[b] >= seq[b].size()) continue;
        const int pz = seq[b][at[b]];
        bool ready = true;
        for (int k = fp.doff[pz]; k < fp.doff[pz + 1] && ready; ++k) ready = done[fp.deps[k]] != 0;
        if (ready) fin.push_back(b);
      }
      if (fin.empty()) { ok = false; break; }
      for (int b : fin) { done[seq[b][at[b]]] = 1; ++at[b]; --left; }
      ++steps;
    }
  }
  stats[0] = npass[0];
  stats[1] = npass[1];
  stats[2] = (long long)fp.deps.size();
  stats[3] = maxdep;
  stats[4] = steps;
  stats[5] = (long long)so.off[0].size() - 1;
  stats[6] = (long long)so.off[1].size() - 1;
  stats[7] = C;
  return ok ? RC_OK : RC_ERR_SYNC;
}

extern "C" {

int rc_flow_plan_check(int ne, int nblocks, const int* nface, const int* cother, long long* stats) {
  if (ne < 1 || nblocks < 1 || !nface || !cother || !stats) return RC_ERR_ARG;
  std::vector<int> nf(nface, nface + ne);
  std::vector<int> co(cother, cother + 4 * (size_t)ne);
  for (int i = 0; i < ne; ++i) {
    if (nf[i] < 0 || nf[i] > 4) return RC_ERR_ARG;
    for (int q = 0; q < nf[i]; ++q) {
      const int j = co[(size_t)q * ne + i];
      if (j < -1 || j >= ne || j == i) return RC_ERR_ARG;
    }
  }
  const SweepOrder so = sweep_order(ne, nf, co);
  int st = RC_OK;
  for (int nv : {4, 7})  // the compact plans of the one- and four-species builds
    for (int gr = FLOWC_GMAX; gr >= 1 && st == RC_OK; --gr)
      st = flow_plan_check_width(ne, nblocks, nf, co, so, 0, stats, gr, flowc_cells(nv));
  for (int gr = FLOW_GMAX; gr >= 1 && st == RC_OK; --gr) st = flow_plan_check_width(ne, nblocks, nf, co, so, 8 * gr, stats);
  return st;
}

int rc_flow_plan_stats(int ne, int nblocks, const int* nface, const int* cother, int groups, int compact, int nvar,
                       long long* stats) {
  if (ne < 1 || nblocks < 1 || !nface || !cother || !stats) return RC_ERR_ARG;
  if (compact && (nvar < 3 || nvar > 16)) return RC_ERR_ARG;
  if (compact ? (groups < 1 || groups > FLOWC_GMAX) : (groups < 1 || groups > FLOW_GMAX)) return RC_ERR_ARG;
  std::vector<int> nf(nface, nface + ne);
  std::vector<int> co(cother, cother + 4 * (size_t)ne);
  for (int i = 0; i < ne; ++i) {
    if (nf[i] < 0 || nf[i] > 4) return RC_ERR_ARG;
    for (int q = 0; q < nf[i]; ++q) {
      const int j = co[(size_t)q * ne + i];
      if (j < -1 || j >= ne || j == i) return RC_ERR_ARG;
    }
  }
  const SweepOrder so = sweep_order(ne, nf, co);
  return compact ? flow_plan_check_width(ne, nblocks, nf, co, so, 0, stats, groups, flowc_cells(nvar))
                 : flow_plan_check_width(ne, nblocks, nf, co, so, 8 * groups, stats);
}

int rc_init(const rc_mesh* m, const rc_thermo* t, const rc_config* g, rc_ctx** out) {
  if (!m || !t || !g || !out) return RC_ERR_ARG;
  BatchDesc b;
  bc_row_of(t, g, b.bctab);
  b.case_off = {0, m->NE};
  b.case_vol = {m->total_volume};
  return init_impl(m, t, g, b, out);
}

int rc_init_batch(int ncase, const rc_mesh* meshes, const rc_thermo* thermos, const rc_config* cfgs, rc_ctx** out) {
  if (ncase < 1 || !meshes || !thermos || !cfgs || !out) return RC_ERR_ARG;
  *out = nullptr;
  for (int k = 1; k < ncase; ++k) {
    const std::string e = same_gas(&thermos[0], &thermos[k], &cfgs[0], &cfgs[k]);
    if (!e.empty()) {
      std::fprintf(stderr, "rc_init_batch: case %d: %s\n", k, e.c_str());
      return RC_ERR_ARG;
    }
  }
  MergedMesh mm;
  BatchDesc b;
  const std::string e = merge_meshes(ncase, meshes, mm, b);
  if (!e.empty()) {
    std::fprintf(stderr, "rc_init_batch: %s\n", e.c_str());
    return RC_ERR_ARG;
  }
  for (int k = 0; k < ncase; ++k) bc_row_of(&thermos[k], &cfgs[k], b.bctab);
  if (ncase == 1) { b.fcase.clear(); b.gcase.clear(); }
  return init_impl(&mm.m, &thermos[0], &cfgs[0], b, out);
}

int rc_finalize(rc_ctx* c) {
  if (!c) return RC_OK;
  for (auto& gx : c->graphs)
    if (gx) cudaGraphExecDestroy(gx);
  if (c->bdf2_graph) cudaGraphExecDestroy(c->bdf2_graph);
  for (void* p : c->allocs) cudaFree(p);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  delete c;
  return RC_OK;
}

int rc_set_stream(rc_ctx* c, void* s) {
  if (!c) return RC_ERR_ARG;
  for (auto& gx : c->graphs)
    if (gx) { cudaGraphExecDestroy(gx); gx = nullptr; }
  c->graph = nullptr;
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->stream = static_cast<cudaStream_t>(s);
  c->own_stream = false;
  return RC_OK;
}
void* rc_get_stream(rc_ctx* c) { return c ? (void*)c->stream : nullptr; }

static int put_soa(rc_ctx* c, const double* host, double* dst, int N, int V) {
  RC_CU(cudaMemcpyAsync(c->staging, host, sizeof(double) * (size_t)N * V, cudaMemcpyHostToDevice, c->stream));
  k_aos_to_soa<<<blocks((long)N * V, 256), 256, 0, c->stream>>>(c->staging, dst, N, V);
  c->launches++;
  return check_launch(c, "k_aos_to_soa");
}
static int get_soa(rc_ctx* c, const double* src, double* host, int N, int V) {
  k_soa_to_aos<<<blocks((long)N * V, 256), 256, 0, c->stream>>>(src, c->staging, N, V);
  c->launches++;
  RC_CU(cudaMemcpyAsync(host, c->staging, sizeof(double) * (size_t)N * V, cudaMemcpyDeviceToHost, c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  return check_launch(c, "k_soa_to_aos");
}

// The device address of a page-locked host buffer, which kernels can read and
// write in place (over the CPU-GPU link); null for pageable memory.
static double* mapped_host(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? static_cast<double*>(at.devicePointer) : nullptr;
}
// The state (PA, WA): a page-locked host array is converted in place by the
// layout kernel; a pageable one goes through its half of the staging buffer
// (PA the first, WA the second) with one copy.  get_state synchronizes once.
int rc_set_state(rc_ctx* c, const double* PA, const double* WA) {
  if (!c) return RC_ERR_ARG;
  const int N = c->NE, V = c->V;
  const size_t n = (size_t)N * V;
  const double* src[2] = {PA, WA};
  double* dst[2] = {c->d.PA, c->d.WA};
  for (int a = 0; a < 2; ++a) {
    if (!src[a]) continue;
    const double* m = mapped_host(src[a]);
    if (!m) {
      RC_CU(cudaMemcpyAsync(c->staging + a * n, src[a], sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
      m = c->staging + a * n;
    }
    k_aos_to_soa<<<blocks((long)n, 256), 256, 0, c->stream>>>(m, dst[a], N, V);
    c->launches++;
  }
  return check_launch(c, "k_aos_to_soa");
}
int rc_get_state(rc_ctx* c, double* PA, double* WA) {
  if (!c) return RC_ERR_ARG;
  const int N = c->NE, V = c->V;
  const size_t n = (size_t)N * V;
  const double* src[2] = {c->d.PA, c->d.WA};
  double* dst[2] = {PA, WA};
  for (int a = 0; a < 2; ++a) {
    if (!dst[a]) continue;
    double* m = mapped_host(dst[a]);
    k_soa_to_aos<<<blocks((long)n, 256), 256, 0, c->stream>>>(src[a], m ? m : c->staging + a * n, N, V);
    c->launches++;
    if (!m)
      RC_CU(cudaMemcpyAsync(dst[a], c->staging + a * n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  }
  RC_CU(cudaStreamSynchronize(c->stream));
  const int st = check_launch(c, "k_soa_to_aos");
  return st ? st : latch(c);
}

static int bdf2_setup(rc_ctx* c);
static int array_desc(rc_ctx* c, const std::string& s, double** ptr, int* N, int* V, int* grad) {
  *grad = 0;
  if (s == "PA") { *ptr = c->d.PA; *N = c->NE; *V = c->V; }
  else if (s == "WA") { *ptr = c->d.WA; *N = c->NE; *V = c->V; }
  else if (s == "hWA") { *ptr = c->d.hWA; *N = c->NE; *V = c->V; }
  else if (s == "GradC") { *ptr = c->d.grad; *N = c->NE; *V = 2 * c->V; *grad = 1; }
  else if (s == "GPA") { *ptr = c->d.GPA; *N = c->NG; *V = c->V; }
  else if (s == "alpaF") { *ptr = c->d.alpaF; *N = c->NF; *V = 1; }
  else if (s == "step") { *ptr = c->d.step; *N = c->NE; *V = 1; }
  else if (s == "WP" || s == "WP2") {
    if (int st = bdf2_setup(c)) return st;
    *ptr = s == "WP" ? c->d.WP : c->d.WP2; *N = c->NE; *V = c->V;
  } else return RC_ERR_ARG;
  return RC_OK;
}
int rc_get_array(rc_ctx* c, const char* name, double* out) {
  if (!c || !name || !out) return RC_ERR_ARG;
  double* p; int N, V, gr;
  if (array_desc(c, name, &p, &N, &V, &gr)) return RC_ERR_ARG;
  int st = get_soa(c, p, out, N, V);  // GradC(2,NVar,NE): planes (2k+r) are the fastest (V=2*NVar) index
  return st ? st : latch(c);
}
int rc_set_array(rc_ctx* c, const char* name, const double* in) {
  if (!c || !name || !in) return RC_ERR_ARG;
  double* p; int N, V, gr;
  if (array_desc(c, name, &p, &N, &V, &gr)) return RC_ERR_ARG;
  return put_soa(c, in, p, N, V);
}

#define RC_NSP_OK(c) \
  if (!(c)) return RC_ERR_ARG;

int rc_timestep(rc_ctx* c) {
  RC_NSP_OK(c);
  RC_DISPATCH(c, q_timestep_mode, c);
  return check_launch(c, "rc_timestep");
}
int rc_reconstruction(rc_ctx* c) {
  RC_NSP_OK(c);
  RC_DISPATCH(c, q_reconstruction_mode, c);
  return check_launch(c, "rc_reconstruction");
}
int rc_flux_sourceterm(rc_ctx* c) {
  RC_NSP_OK(c);
  RC_DISPATCH(c, q_flux_mode, c);
  return check_launch(c, "rc_flux_sourceterm");
}
int rc_lusgs_steady(rc_ctx* c) {
  RC_NSP_OK(c);
  RC_DISPATCH(c, q_lusgs_mode, c);
  return check_launch(c, "rc_lusgs_steady");
}
int rc_set_precision(rc_ctx* c, int precision) {
  if (!c) return RC_ERR_ARG;
  if (precision != RC_PREC_FP64 && precision != RC_PREC_MIXED && precision != RC_PREC_MIXED_DC) return RC_ERR_ARG;
  if (precision != RC_PREC_FP64 && !c->d.grad32) {
    c->err = "mixed-precision modes need a context created with RC_PREC_MIXED or RC_PREC_MIXED_DC";
    return RC_ERR_ARG;
  }
  c->mode = precision;
  c->graph = c->graphs[precision];
  c->graph_kernels = c->graph_kernels_of[precision];
  return RC_OK;
}
static void drop_graphs(rc_ctx* c) {
  for (int k = 0; k < 3; ++k)
    if (c->graphs[k]) { cudaGraphExecDestroy(c->graphs[k]); c->graphs[k] = nullptr; }
  c->graph = nullptr;
  if (c->bdf2_graph) { cudaGraphExecDestroy(c->bdf2_graph); c->bdf2_graph = nullptr; }
}
int rc_autotune(rc_ctx* c, int iters, char* report, int report_len) {
  if (!c || iters < 1) return RC_ERR_ARG;
  const size_t n = (size_t)c->V * c->NE;
  double* save = nullptr;
  RC_CU(cudaMalloc(&save, 2 * n * sizeof(double)));
  auto restore = [&]() {
    cudaMemcpyAsync(c->d.PA, save, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->d.WA, save + n, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  };
  cudaMemcpyAsync(save, c->d.PA, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(save + n, c->d.WA, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  struct Cand { bool pers; int bs; int cpw; int wide; int fg; bool fc; };
  std::vector<Cand> cands;
  for (int pers = c->can_persistent ? 1 : 0; pers >= 0; --pers)
    for (int cpw : {8, 4, 2})
      for (int bs : {128, 64}) cands.push_back({pers != 0, bs, cpw, 0, 1, false});
  for (int wide : {1, 2, 3})
    for (int bs : {128, 64}) cands.push_back({false, bs, 8, wide, 1, false});
  if (c->mode == RC_PREC_FP64) {
    for (int g = 1; g <= FLOW_GMAX; ++g)
      if (c->can_flow[g - 1]) cands.push_back({false, 128, 8, 4, g, false});
    for (int g = 1; g <= FLOWC_GMAX; ++g)
      if (c->can_flowc[g - 1]) cands.push_back({false, 128, 8, 4, g, true});
  } else {
    if (c->can_flow32) cands.push_back({false, 128, 8, 4, 1, false});
    for (int g = 1; g <= FLOWC_GMAX; ++g)
      if (c->can_flowc32[g - 1]) cands.push_back({false, 128, 8, 4, g, true});
  }
  auto name = [](const Cand& k) {
    const std::string fl = k.fc ? "flowc" : "flow";
    return std::string(k.pers ? "persistent"
                              : k.wide == 4 ? (k.fg == 1 ? fl : fl + std::to_string(k.fg))
                              : k.wide == 3 ? "levels4w" : k.wide == 2 ? "levels2w" : k.wide ? "levels8" : "levels");
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::string rep;
  double best = 1e300;
  Cand bc = {c->persistent, c->d.bs, c->d.cpw, c->wide, c->flow_g, c->flow_c};
  int st = RC_OK;
  for (const Cand& k : cands) {
    c->persistent = k.pers;
    c->d.bs = k.bs;
    c->d.cpw = k.cpw;
    c->wide = k.wide;
    c->flow_g = k.fg;
    c->flow_c = k.fc;
    drop_graphs(c);
    restore();
    for (int w = 0; w < 2 && !st; ++w) st = rc_lusgs_stage(c, 1);
    cudaEventRecord(e0, c->stream);
    for (int it = 0; it < iters && !st; ++it) st = rc_lusgs_stage(c, 1);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    if (st) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double per = ms / iters;
    rep += name(k) + " bs=" + std::to_string(k.bs) + " cpw=" + std::to_string(k.wide >= 2 ? 8 : k.wide ? 4 : k.cpw) + ": " +
           std::to_string(per) + " ms; ";
    if (per < best) { best = per; bc = k; }
  }
  c->persistent = bc.pers;
  c->d.bs = bc.bs;
  c->d.cpw = bc.cpw;
  c->wide = bc.wide;
  c->flow_g = bc.fg;
  c->flow_c = bc.fc;
  drop_graphs(c);
  restore();
  cudaStreamSynchronize(c->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(save);
  rep += std::string("chosen: ") + name(bc) + " bs=" + std::to_string(bc.bs) + " cpw=" + std::to_string(bc.wide >= 2 ? 8 : bc.wide ? 4 : bc.cpw);
  if (report && report_len > 0) {
    std::snprintf(report, (size_t)report_len, "%s", rep.c_str());
  }
  if (st) return st;
  return latch(c);
}
int rc_set_surrogate(rc_ctx* c, rc_mlp* net, double spread_tol) {
  if (!c || !net || !(spread_tol > 0.0)) return RC_ERR_ARG;
  if (c->NSP != 4) {
    c->err = "the surrogate is built for 4 species";
    return RC_ERR_ARG;
  }
  if (!c->sur_list) {
    if (int st = dev_zeros(c, (size_t)c->NE, &c->sur_list)) return st;
    if (int st = dev_zeros(c, (size_t)2, &c->sur_counts)) return st;
    if (int st = dev_zeros(c, (size_t)1, &c->sur_mode)) return st;
    if (int st = dev_zeros(c, (size_t)c->NE, &c->sur_dec)) return st;
  }
  RC_CU(surrogate_prepare());
  c->net = net;
  c->spread_tol = (float)spread_tol;
  drop_graphs(c);
  return RC_OK;
}
int rc_surrogate_freeze(rc_ctx* c, int on) {
  if (!c || !c->sur_mode) return RC_ERR_ARG;
  const int m = on ? 1 : 0;
  RC_CU(cudaMemcpyAsync(c->sur_mode, &m, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  c->sur_freeze_pending = on != 0;
  return RC_OK;
}
int rc_surrogate_stats(rc_ctx* c, unsigned* n_surrogate, unsigned* n_fallback) {
  if (!c) return RC_ERR_ARG;
  unsigned h[2] = {0, 0};
  if (c->sur_counts) {
    RC_CU(cudaMemcpyAsync(h, c->sur_counts, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    RC_CU(cudaStreamSynchronize(c->stream));
  }
  if (n_fallback) *n_fallback = h[0];
  if (n_surrogate) *n_surrogate = h[1];
  return latch(c);
}
int rc_surrogate_samples(rc_ctx* c, const double* d_P0, const double* d_P1, const double* d_dt, int n, float* d_x,
                         float* d_t) {
  if (!c || n < 0 || (n > 0 && (!d_P0 || !d_P1 || !d_dt || !d_x || !d_t))) return RC_ERR_ARG;
  if (c->NSP != 4) return RC_ERR_ARG;
  if (n == 0) return RC_OK;
  RC_CU(surrogate_samples(c->thermo.data(), d_P0, d_P1, d_dt, n, d_x, d_t, c->stream));
  c->launches++;
  return RC_OK;
}
int rc_set_wait_limit(rc_ctx* c, unsigned polls) {
  if (!c || polls < 1) return RC_ERR_ARG;
  c->d.spin_limit = polls;
  drop_graphs(c);
  return RC_OK;
}
int rc_clear_error(rc_ctx* c) {
  if (!c) return RC_ERR_ARG;
  RC_CU(cudaStreamSynchronize(c->stream));
  RC_CU(cudaMemsetAsync(c->d.err, 0, sizeof(unsigned), c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  c->latched = 0;
  c->err.clear();
  return RC_OK;
}
int rc_set_chemistry(rc_ctx* c, int mode, double tol, int max_substeps) {
  if (!c) return RC_ERR_ARG;
  if (mode != RC_CHEM_EXPLICIT && mode != RC_CHEM_INTEGRATED && mode != RC_CHEM_SURROGATE) return RC_ERR_ARG;
  if (!(tol > 0.0) || max_substeps < 1) return RC_ERR_ARG;
  if (mode != RC_CHEM_EXPLICIT && !c->comb) {
    c->err = "the integrated source needs If_turn_on_combustion";
    return RC_ERR_ARG;
  }
  if (mode == RC_CHEM_SURROGATE && !c->net) {
    c->err = "RC_CHEM_SURROGATE needs rc_set_surrogate first";
    return RC_ERR_ARG;
  }
  if (mode != RC_CHEM_EXPLICIT && !c->chem_nsub) {
    if (int st = dev_zeros(c, (size_t)c->NE, &c->chem_nsub)) return st;
    if (int st = dev_zeros(c, (size_t)c->NE, &c->chem_order)) return st;
    if (int st = dev_zeros(c, (size_t)256, &c->chem_hist)) return st;
    if (int st = dev_zeros(c, (size_t)1, &c->chem_counter)) return st;
    RC_CU(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    RC_CU(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    RC_CU(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
  }
  c->chem = mode;
  c->chem_tol = tol;
  c->chem_maxsub = max_substeps;
  drop_graphs(c);
  return RC_OK;
}
int rc_chem_substeps(rc_ctx* c, int* out) {
  if (!c || !out) return RC_ERR_ARG;
  if (!c->chem_nsub) {
    for (int i = 0; i < c->NE; ++i) out[i] = 0;
    return RC_OK;
  }
  RC_CU(cudaMemcpyAsync(out, c->chem_nsub, sizeof(int) * (size_t)c->NE, cudaMemcpyDeviceToHost, c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  return latch(c);
}
int rc_chem_integrate(rc_ctx* c, const double* d_P, const double* d_dt, int n, double* d_out, int* d_nsub,
                      double tol, int max_substeps) {
  if (!c || n < 0 || (n > 0 && (!d_P || !d_dt || !d_out || !d_nsub))) return RC_ERR_ARG;
  if (c->NSP < 2 || !(tol > 0.0) || max_substeps < 1) return RC_ERR_ARG;
  if (n == 0) return RC_OK;
  if (!c->chem_counter)
    if (int st = dev_zeros(c, (size_t)1, &c->chem_counter)) return st;
  RC_DISPATCH(c, chem_batch, c->thermo.data(), d_P, d_dt, n, d_out, d_nsub, tol, max_substeps, c->chem_counter,
              c->d.err, c->stream);
  c->launches++;
  return check_launch(c, "rc_chem_integrate");
}
int rc_lusgs_stage(rc_ctx* c, int istep) {
  (void)istep;
  RC_NSP_OK(c);
  if (!c->graph) {
    cudaGraph_t gph;
    const long long before = c->launches;
    RC_CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    RC_DISPATCH(c, q_stage, c);
    cudaError_t e = cudaStreamEndCapture(c->stream, &gph);
    if (e != cudaSuccess) return cuda_fail(c, e, "capture of lu_sgs_stage");
    c->graph_kernels = c->launches - before;
    c->launches = before;
    e = cudaGraphInstantiate(&c->graph, gph, 0);
    cudaGraphDestroy(gph);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
    c->graphs[c->mode] = c->graph;
    c->graph_kernels_of[c->mode] = c->graph_kernels;
  }
  RC_CU(cudaGraphLaunch(c->graph, c->stream));
  c->launches += c->graph_kernels;
  if (c->sur_freeze_pending) {  // this stage recorded the surrogate's decisions: keep them from now on
    static const int recorded = 2;
    RC_CU(cudaMemcpyAsync(c->sur_mode, &recorded, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    c->sur_freeze_pending = false;
  }
  return RC_OK;
}

int rc_sync(rc_ctx* c) {
  if (!c) return RC_ERR_ARG;
  RC_CU(cudaStreamSynchronize(c->stream));
  return latch(c);
}

// Norms of every case into norm_out ([case][V+1]); synchronises.
static int norms(rc_ctx* c, std::vector<double>& h) {
  const int nc = c->ncase;
  q_norms(c);
  h.resize((size_t)nc * (c->V + 1));
  RC_CU(cudaMemcpyAsync(h.data(), c->norm_out, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
  RC_CU(cudaStreamSynchronize(c->stream));
  return check_launch(c, "norms");
}
int rc_residual(rc_ctx* c, double* res, double* romax) {
  if (!c || !res || !romax) return RC_ERR_ARG;
  if (c->ncase != 1) {
    c->err = "rc_residual on a batch: use rc_residual_batch";
    return RC_ERR_ARG;
  }
  std::vector<double> h;
  if (int st = norms(c, h)) return st;
  for (int k = 0; k < c->V; ++k) res[k] = h[k];
  *romax = h[c->V];
  return latch(c);
}
int rc_residual_batch(rc_ctx* c, double* res, double* romax) {
  if (!c || !res || !romax) return RC_ERR_ARG;
  std::vector<double> h;
  if (int st = norms(c, h)) return st;
  const int V = c->V;
  for (int b = 0; b < c->ncase; ++b) {
    for (int k = 0; k < V; ++k) res[(size_t)b * V + k] = h[(size_t)b * (V + 1) + k];
    romax[b] = h[(size_t)b * (V + 1) + V];
  }
  return latch(c);
}
int rc_batch_info(rc_ctx* c, int* ncase, int* cell_offsets) {
  if (!c) return RC_ERR_ARG;
  if (ncase) *ncase = c->ncase;
  if (cell_offsets)
    for (int b = 0; b <= c->ncase; ++b) cell_offsets[b] = c->case_off[b];
  return RC_OK;
}

// ------------------------------------------- unsteady dual-time BDF2 -----
static int bdf2_setup(rc_ctx* c) {
  if (c->ncase != 1) {
    c->err = "the BDF2 stage takes one case per context";
    return RC_ERR_ARG;
  }
  if (c->mode != RC_PREC_FP64 || c->chem != RC_CHEM_EXPLICIT) {
    c->err = "the BDF2 stage runs the FP64 path with the explicit chemical source";
    return RC_ERR_ARG;
  }
  if (c->bdf2_ready) return RC_OK;
  const size_t NE = (size_t)c->NE, V = (size_t)c->V;
  int nbq = 0;
  RC_DISPATCH(c, nbq = bdf2_nbq);
  int st = dev_zeros(c, V * NE, &c->d.WP);
  st |= dev_zeros(c, V * NE, &c->d.WP2);
  st |= dev_zeros(c, V * NE, &c->d.bfix);
  st |= dev_zeros(c, NE * V * (2 * V + 4), &c->d.bmat);
  st |= dev_zeros(c, 8 * NE, &c->d.bperm);
  st |= dev_zeros(c, (size_t)nbq * NE, &c->d.bnb);
  st |= dev_zeros(c, (size_t)2, &c->bpar_dev);
  if (st) return st;
  c->d.bpar = c->bpar_dev;
  if (const char* e = std::getenv("RC_BDF2_CPW")) c->bdf2_cpw = std::atoi(e);
  {  // the dataflow sweeps: a cooperative grid of one block per SM
    int nsm = 0, coop = 0, occ = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
    RC_DISPATCH(c, occ = bdf2_flow_occupancy);
    cudaGetLastError();
    const char* e = std::getenv("RC_BDF2_SCHEDULE");
    c->bdf2_flow = coop && nsm > 0 && occ >= 1 && c->flow_grid == nsm && !(e && std::string(e) == "levels");
  }
  c->bdf2_ready = true;
  drop_graphs(c);  // the captured kernels hold the old Dev
  return RC_OK;
}
static int bdf2_params(rc_ctx* c, double dt, double phi) {
  const double par[2] = {dt, phi};
  RC_CU(cudaMemcpyAsync(c->bpar_dev, par, sizeof(par), cudaMemcpyHostToDevice, c->stream));
  return RC_OK;
}
int rc_set_p_out(rc_ctx* c, const double* p_out) {
  if (!c || !p_out) return RC_ERR_ARG;
  for (int k = 0; k < c->ncase; ++k) {
    const float p32 = (float)p_out[k];
    RC_CU(cudaMemcpyAsync(const_cast<double*>(c->d.bctab) + (size_t)k * BCS + BC_POUT, &p_out[k], sizeof(double),
                          cudaMemcpyHostToDevice, c->stream));
    RC_CU(cudaMemcpyAsync(const_cast<float*>(c->d.bctab32) + (size_t)k * BCS + BC_POUT, &p32, sizeof(float),
                          cudaMemcpyHostToDevice, c->stream));
  }
  return RC_OK;
}
static int implicit_lusgs(rc_ctx* c, int inner_rk, double phi, double dt, int euler) {
  if (!c || inner_rk < 1 || !(dt > 0.0)) return RC_ERR_ARG;
  RC_NSP_OK(c);
  if (int st = bdf2_setup(c)) return st;
  if (int st = bdf2_params(c, dt, phi)) return st;
  if (inner_rk == 1) {
    RC_DISPATCH(c, bdf2_fixed, c->d, c->d.bs, euler, c->stream);
    c->launches++;
  }
  RC_DISPATCH(c, q_bdf2_lusgs, c);
  return check_launch(c, "rc_bdf2_lusgs");
}
int rc_bdf2_lusgs(rc_ctx* c, int inner_rk, double phi, double dt) { return implicit_lusgs(c, inner_rk, phi, dt, 0); }
int rc_euler_lusgs(rc_ctx* c, int inner_rk, double dt) { return implicit_lusgs(c, inner_rk, 0.0, dt, 1); }
// BDF2_stage, or with euler backwardEuler_stage (no time levels, phi = 0)
static int implicit_stage(rc_ctx* c, int istep, double dt, int inner_loop, double rel_tol, int* inner_done,
                          int euler) {
  if (!c || istep < 1 || inner_loop < 1 || !(dt > 0.0)) return RC_ERR_ARG;
  RC_NSP_OK(c);
  if (int st = bdf2_setup(c)) return st;
  const size_t bytes = sizeof(double) * (size_t)c->V * c->NE;
  double phi = 0.;
  if (euler) {
  } else if (istep == 1) {
    RC_CU(cudaMemcpyAsync(c->d.WP, c->d.WA, bytes, cudaMemcpyDeviceToDevice, c->stream));
    RC_CU(cudaMemcpyAsync(c->d.WP2, c->d.WP, bytes, cudaMemcpyDeviceToDevice, c->stream));
    phi = 0.;
  } else {
    RC_CU(cudaMemcpyAsync(c->d.WP2, c->d.WP, bytes, cudaMemcpyDeviceToDevice, c->stream));
    RC_CU(cudaMemcpyAsync(c->d.WP, c->d.WA, bytes, cudaMemcpyDeviceToDevice, c->stream));
    phi = 0.5;
  }
  if (int st = bdf2_params(c, dt, phi)) return st;
  RC_DISPATCH(c, bdf2_fixed, c->d, c->d.bs, euler, c->stream);
  c->launches++;
  if (!c->bdf2_graph) {
    cudaGraph_t gph;
    const long long before = c->launches;
    RC_CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    RC_DISPATCH(c, q_bdf2_inner, c);
    cudaError_t e = cudaStreamEndCapture(c->stream, &gph);
    if (e != cudaSuccess) return cuda_fail(c, e, "capture of the BDF2 inner iteration");
    c->bdf2_graph_kernels = c->launches - before;
    c->launches = before;
    e = cudaGraphInstantiate(&c->bdf2_graph, gph, 0);
    cudaGraphDestroy(gph);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  }
  const int V = c->V;
  std::vector<double> h((size_t)V + 1);
  unsigned derr = 0;
  double rores_tmp = 0.0;
  int inner = 1;
  for (; inner <= inner_loop; ++inner) {
    RC_CU(cudaGraphLaunch(c->bdf2_graph, c->stream));
    c->launches += c->bdf2_graph_kernels;
    // inner_iteration_residual (residual.f90:23-59): sum of the species rows
    RC_CU(cudaMemcpyAsync(h.data(), c->norm_out, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    RC_CU(cudaMemcpyAsync(&derr, c->d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    RC_CU(cudaStreamSynchronize(c->stream));
    double rores = 0.0;
    for (int k = 4; k < V; ++k) rores = rores + h[k];
    if (inner == 1) rores_tmp = rores;
    if (rores < rores_tmp * rel_tol || inner == inner_loop) {
      RC_DISPATCH(c, q_bdf2_final, c);
      break;
    }
    if (derr) break;  // the reference stops (NaN, thermo range, singular cell system)
  }
  if (inner_done) *inner_done = inner > inner_loop ? inner_loop : inner;
  if (int st = check_launch(c, "rc_bdf2_stage")) return st;
  return latch(c);
}
int rc_bdf2_stage(rc_ctx* c, int istep, double dt, int inner_loop, double rel_tol, int* inner_done) {
  return implicit_stage(c, istep, dt, inner_loop, rel_tol, inner_done, 0);
}
int rc_euler_stage(rc_ctx* c, int istep, double dt, int inner_loop, double rel_tol, int* inner_done) {
  return implicit_stage(c, istep, dt, inner_loop, rel_tol, inner_done, 1);
}

int rc_stats(rc_ctx* c, long long* launches, int* fwd, int* bwd) {
  if (!c) return RC_ERR_ARG;
  if (launches) *launches = c->launches;
  if (fwd) *fwd = (int)c->fwd_off.size() - 1;
  if (bwd) *bwd = (int)c->bwd_off.size() - 1;
  return RC_OK;
}

const char* rc_last_error(rc_ctx* c) { return c ? c->err.c_str() : "no context"; }

int rc_last_error_buf(rc_ctx* c, char* buf, int len) {
  if (!buf || len < 1) return RC_ERR_ARG;
  const char* m = rc_last_error(c);
  const size_t n = std::min(std::strlen(m), (size_t)(len - 1));
  std::memcpy(buf, m, n);
  buf[n] = '\0';
  return RC_OK;
}

}  // extern "C"
