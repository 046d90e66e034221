// Mixed-precision form of the steady iteration (RC_PREC_MIXED / RC_PREC_MIXED_DC).
//
//   FP32: spectral radius, reconstruction (ghost states, LS gradient, Barth
//         limiter), Lax/Rusanov and viscous face fluxes, and the LU-SGS
//         off-diagonal terms;
//   FP64: the state (PA, WA), the local step and the LU-SGS diagonal with its
//         division, the chemical source, the per-cell residual after a
//         compensated (Neumaier) FP32 gather, the Newton update and the norms.
// In the defect-correction phase (RC_PREC_MIXED_DC) the residual comes from the
// FP64 kernels of rc_core.cu while the LU-SGS sweeps stay in FP32, so the fixed
// point is the FP64 one.
//
// Built with approximate FP32 division and square root and FP32 denormals
// flushed (--prec-div=false --prec-sqrt=false --ftz=true; the FP32 SFU math is
// called by name in rc_thermo32.cuh), and without FMA contraction
// (--fmad=false), so that the FP64 code here (the Newton update fused into
// k_lusgs_flow32, the chemical source) gives the bits of rc_core.cu's.
#include <cuda_runtime.h>

#include "rc_dev.cuh"
#include "rc_thermo32.cuh"

namespace rc {

// ----------------------------------------------------------- TimeStep ------
template <int NSP, bool VISC>
__global__ void __launch_bounds__(128) k_ts_face32(const Dev d, const ThermoDev32<NSP> th) {
  constexpr int V = 3 + NSP;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= d.NF) return;
  unsigned err = 0;
  const int NE = d.NE, NL = d.fNL[f], NR = d.fNR[f];
  float P[V], yy[NSP];
#pragma unroll
  for (int k = 0; k < V; ++k)
    P[k] = (NR >= 0) ? (float)(0.5 * (d.PA[k * NE + NL] + d.PA[k * NE + NR])) : (float)d.PA[k * NE + NL];
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { yy[k] = P[4 + k]; s += yy[k]; }
  yy[NSP - 1] = 1.f - s;
  float Cp, gama, Rc;
  gas32<NSP>(th, yy, P[3], Cp, gama, Rc, err);
  const float rr = P[0] / (Rc * P[3]);
  if (rr < 0.f || P[0] < 0.f || P[3] < 0.f) err |= ERR_NEG_TIMESTEP;
  const float un = P[1] * (float)d.fvec[f] + P[2] * (float)d.fvec[d.NF + f];
  const float alpa = fabsf(un) + sqrtf(gama * P[0] / rr) * (float)d.fss[f];
  d.alpa[f] = alpa;
  if (VISC) {
    float vmul, akmu;
    transport32<NSP>(th, P[3], yy, vmul, akmu, err);
    const float prl = vmul * Cp / akmu;
    const double vis = (double)(2.f * (float)d.fs2[f] * fmax2f(4.f / 3.f, gama / prl) * vmul / rr);
    const double vl = vis / d.vol[NL];
    d.visL[f] = vl;
    d.visR[f] = (NR >= 0) ? vis / d.vol[NR] : 0.0;
    d.alpaF[f] = (double)alpa + vl;
    d.alpaF32[f] = (float)((double)alpa + vl);
  } else {
    d.alpaF[f] = alpa;
    d.alpaF32[f] = alpa;
  }
  if (err) atomicOr(d.err, err);
}

// --------------------------------------------------------- cell kernel -----
template <int NSP>
__global__ void __launch_bounds__(128) k_cell32(const Dev d, const ThermoDev32<NSP> th, const ThermoDev<NSP> th64,
                                                int do_step, int limit, int comb, int visc) {
  constexpr int V = 3 + NSP;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE;
  unsigned err = 0;
  const int nf = d.nface[i];
  const double vol = d.vol[i];
  if (do_step) {  // FP64: local step and LU-SGS diagonal
    const unsigned lb = d.cleft[i];
    double acc = 0.0, dsum = 0.0;
    for (int q = 0; q < nf; ++q) {
      const int f = d.cface[q * NE + i];
      acc = visc ? acc + d.alpa[f] + (((lb >> q) & 1u) ? d.visL[f] : d.visR[f]) : acc + d.alpa[f];
      dsum += 0.5 * d.alpaF[f];
    }
    const double st = th64.cfl * vol / acc;
    d.step[i] = st;
    d.dd[i] = dsum + vol / st;
  }
  double P64[V];
  float P[V], Y[NSP];
#pragma unroll
  for (int k = 0; k < V; ++k) { P64[k] = d.PA[k * NE + i]; P[k] = (float)P64[k]; }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { Y[k] = P[4 + k]; s += Y[k]; }
  Y[NSP - 1] = 1.f - s;
  float Cp, gama, Rc, entha[NSP];
  gas32<NSP>(th, Y, P[3], Cp, gama, Rc, err);
  const float rr = P[0] / (Rc * P[3]);
  enthalpy32<NSP>(th, P[3], entha, err);
  float hh = 0.f;
#pragma unroll
  for (int k = 0; k < NSP; ++k) hh += Y[k] * entha[k];
  d.cst32[0 * NE + i] = rr;
  d.cst32[1 * NE + i] = gama;
  d.cst32[2 * NE + i] = rr * (hh + 0.5f * (P[1] * P[1] + P[2] * P[2])) - P[0];
#pragma unroll
  for (int k = 0; k < NSP; ++k) d.cst32[(3 + k) * NE + i] = entha[k];
#pragma unroll
  for (int k = 0; k < V; ++k) d.PA32[k * NE + i] = P[k];
  // gradient: differences in FP64, weights and sums in FP32
  float g0[V], g1[V], mn[V], mx[V];
#pragma unroll
  for (int k = 0; k < V; ++k) { g0[k] = 0.f; g1[k] = 0.f; mn[k] = 0.f; mx[k] = 0.f; }
  const int nn = d.nnei[i];
  for (int q = 0; q < nn; ++q) {
    const int j = d.cnei[q * NE + i];
    const float w = (float)d.wdis[q * NE + i], a0 = (float)d.amls[(2 * q) * NE + i],
                a1 = (float)d.amls[(2 * q + 1) * NE + i];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const float dlt = (float)(d.PA[k * NE + j] - P64[k]);
      const float c = w * dlt;
      g0[k] += a0 * c;
      g1[k] += a1 * c;
      mn[k] = fmin2f(mn[k], dlt);
      mx[k] = fmax2f(mx[k], dlt);
    }
  }
  const int ng = d.ngh[i];
  for (int q = 0; q < ng; ++q) {
    const int gj = d.cgh[q * NE + i];
    const float s1n = (float)d.gsn[gj], s2n = (float)d.gsn[d.NG + gj];
    const float pl = P[0], ul = P[1], vl = P[2], tl = P[3];
    const float ac = sqrtf(gama * pl / rr);
    float G[V], Yr[NSP];
    float pr = pl, ur = ul, vr = vl, tr = tl, vn;
#pragma unroll
    for (int k = 0; k < NSP; ++k) Yr[k] = Y[k];
    switch (d.gtype[gj]) {
      case 1: ur = -ul; vr = -vl; break;
      case 2:
      case 6:
        vn = ul * s1n + vl * s2n;
        ur = ul - 2.f * vn * s1n;
        vr = vl - 2.f * vn * s2n;
        break;
      case 3:
      case 4: {
        const int w = d.gtype[gj] == 3 ? 0 : 1;
        const float* bc = bc_row32(d, d.gcase, gj);
#pragma unroll
        for (int k = 0; k < NSP; ++k) Yr[k] = bc[BC_Y + w * BC_NSPMAX + k];
        tr = bc[BC_T + w];
        float Cb, gb, Rb;
        gas32<NSP>(th, Yr, tr, Cb, gb, Rb, err);
        const float rb = pr / (Rb * tr);
        ur = bc[BC_MFLOW + w] / rb;
        vr = 0.f;
        break;
      }
      case 5:
        vn = ul * s1n + vl * s2n;
        if (!(fabsf(vn) > ac)) pr = bc_row32(d, d.gcase, gj)[BC_POUT];
        break;
      default: err |= ERR_BCTYPE;
    }
    G[0] = pr; G[1] = ur; G[2] = vr; G[3] = tr;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) G[4 + k] = Yr[k];
#pragma unroll
    for (int k = 0; k < V; ++k) d.GPA32[k * d.NG + gj] = G[k];
    const int m = nn + q;
    const float w = (float)d.wdis[m * NE + i], a0 = (float)d.amls[(2 * m) * NE + i],
                a1 = (float)d.amls[(2 * m + 1) * NE + i];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const float dlt = G[k] - P[k];
      const float c = w * dlt;
      g0[k] += a0 * c;
      g1[k] += a1 * c;
      mn[k] = fmin2f(mn[k], dlt);
      mx[k] = fmax2f(mx[k], dlt);
    }
  }
  if (limit > 0) {  // Barth: phi = min over faces of min(1, (max-P)/(f-P)) or (min-P)/(f-P)
    float lv0[MAXF], lv1[MAXF];
    for (int q = 0; q < nf; ++q) { lv0[q] = (float)d.lvvh[(2 * q) * NE + i]; lv1[q] = (float)d.lvvh[(2 * q + 1) * NE + i]; }
#pragma unroll
    for (int k = 0; k < V; ++k) {
      float phi = 1.f;
      for (int q = 0; q < nf; ++q) {
        const float df = g0[k] * lv0[q] + g1[k] * lv1[q];
        float pf = 1.f;
        if (df > 0.f) pf = fmin2f(1.f, mx[k] / df);
        else if (df < 0.f) pf = fmin2f(1.f, mn[k] / df);
        phi = fmin2f(phi, pf);
      }
      g0[k] *= phi;
      g1[k] *= phi;
    }
  }
#pragma unroll
  for (int k = 0; k < V; ++k) {
    d.grad32[(2 * k) * NE + i] = g0[k];
    d.grad32[(2 * k + 1) * NE + i] = g1[k];
  }
  if (comb) {  // FP64 chemistry
    double Y64[NSP], s64 = 0.0, R64 = 0.0;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { Y64[k] = P64[4 + k]; s64 += Y64[k]; }
    Y64[NSP - 1] = 1.0 - s64;
#pragma unroll
    for (int k = 0; k < NSP; ++k) R64 += th64.R[k] * Y64[k];
    double prod[NSP];
    production<NSP>(th64, P64[3], P64[0] / (R64 * P64[3]), Y64, prod);
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) d.src[k * NE + i] = vol * prod[k];
  }
  if (err) atomicOr(d.err, err);
}

// ------------------------------------------------------------ face flux ----
template <int NSP, bool VISC>
__global__ void __launch_bounds__(128) k_face_flux32(const Dev d, const ThermoDev32<NSP> th) {
  constexpr int V = 3 + NSP;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= d.NF) return;
  unsigned err = 0;
  const int NE = d.NE, NF = d.NF;
  const int NL = d.fNL[f], NR = d.fNR[f];
  const float sav1 = (float)d.fvec[f], sav2 = (float)d.fvec[NF + f], sav = (float)d.fsav[f];
  const float sn1 = (float)d.fsn[f], sn2 = (float)d.fsn[NF + f];
  float uL[V], uR[V], YL0[NSP], YR0[NSP];
  {
    const float v0 = (float)d.fvL[f], v1 = (float)d.fvL[NF + f];
#pragma unroll
    for (int k = 0; k < V; ++k)
      uL[k] = (float)d.PA[k * NE + NL] + (d.grad32[(2 * k) * NE + NL] * v0 + d.grad32[(2 * k + 1) * NE + NL] * v1);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { YL0[k] = uL[4 + k]; s += YL0[k]; }
  YL0[NSP - 1] = 1.f - s;
  float Cl0, gl0, Rl0;
  gas32<NSP>(th, YL0, uL[3], Cl0, gl0, Rl0, err);
  const float rl0 = uL[0] / (Rl0 * uL[3]);
  float gr0 = 0.f, Rr0 = 0.f, rr0 = 0.f;
  if (NR >= 0) {
    const float v0 = (float)d.fvR[f], v1 = (float)d.fvR[NF + f];
#pragma unroll
    for (int k = 0; k < V; ++k)
      uR[k] = (float)d.PA[k * NE + NR] + (d.grad32[(2 * k) * NE + NR] * v0 + d.grad32[(2 * k + 1) * NE + NR] * v1);
    s = 0.f;
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { YR0[k] = uR[4 + k]; s += YR0[k]; }
    YR0[NSP - 1] = 1.f - s;
    float Cr0;
    gas32<NSP>(th, YR0, uR[3], Cr0, gr0, Rr0, err);
    rr0 = uR[0] / (Rr0 * uR[3]);
  } else {
#pragma unroll
    for (int k = 0; k < V; ++k) uR[k] = uL[k];
  }
  // ---- Lax/Rusanov flux
  {
    float pl = uL[0], ul = uL[1], vl = uL[2], tl = uL[3], rl = rl0, gl = gl0, Rl = Rl0;
    float pr, ur, vr, tr, rr, gr, vn;
    float Yl[NSP], Yr[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) Yl[k] = YL0[k];
    if (NR >= 0) {
      pr = uR[0]; ur = uR[1]; vr = uR[2]; tr = uR[3]; rr = rr0; gr = gr0;
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = YR0[k];
    } else if (NR == -3 || NR == -4) {
      const int w = NR == -3 ? 0 : 1;
      const float* bc = bc_row32(d, d.fcase, f);
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = bc[BC_Y + w * BC_NSPMAX + k];
      tr = bc[BC_T + w];
      float Cb, Rb;
      gas32<NSP>(th, Yr, tr, Cb, gr, Rb, err);
      pr = pl;
      rr = pr / (Rb * tr);
      ur = bc[BC_MFLOW + w] / rr;
      vr = 0.f;
      pl = pr; ul = ur; vl = vr; tl = tr; rl = rr; gl = gr; Rl = Rb;
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yl[k] = Yr[k];
    } else {
      rr = rl; pr = pl; tr = tl; ur = ul; vr = vl; gr = gl;
      if (NR == -1) { ur = -ul; vr = -vl; }
      else if (NR == -2 || NR == -6) {
        vn = ul * sn1 + vl * sn2;
        ur = ul - 2.f * vn * sn1;
        vr = vl - 2.f * vn * sn2;
      } else if (NR == -5) {
        const float ac = sqrtf(gl * pl / rl);
        vn = ul * sn1 + vl * sn2;
        if (!(fabsf(vn) > ac)) {
          pr = bc_row32(d, d.fcase, f)[BC_POUT];
          ur = ul + sn1 * (pl - pr) / (rl * ac);
          vr = vl + sn2 * (pl - pr) / (rl * ac);
          rr = rl + (pr - pl) / (ac * ac);
          tr = pr / (Rl * rr);
          pl = pr; ul = ur; vl = vr; tl = tr; rl = rr;
        }
      } else {
        err |= ERR_BCTYPE;
      }
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = Yl[k];
    }
    if (rl < 0.f || pl < 0.f || (NR >= 0 && (rr < 0.f || pr < 0.f))) err |= ERR_NEG_FACE;
    float entha[NSP];
    enthalpy32<NSP>(th, tl, entha, err);
    float hl = 0.f;
#pragma unroll
    for (int k = 0; k < NSP; ++k) hl += Yl[k] * entha[k];
    enthalpy32<NSP>(th, tr, entha, err);
    float hr = 0.f;
#pragma unroll
    for (int k = 0; k < NSP; ++k) hr += Yr[k] * entha[k];
    hl += 0.5f * (ul * ul + vl * vl);
    hr += 0.5f * (ur * ur + vr * vr);
    const float el = hl - pl / rl, er = hr - pr / rr;
    const float acl = sqrtf(gl * pl / rl), acr = sqrtf(gr * pr / rr);
    const float uln = sav1 * ul + sav2 * vl, urn = sav1 * ur + sav2 * vr;
    const float coex = fmax2f(fabsf(uln) + acl * sav, fabsf(urn) + acr * sav);
    const float rul = rl * uln, rur = rr * urn;
    d.Finv32[0 * NF + f] = 0.5f * (rul + rur - coex * (rr - rl));
    d.Finv32[1 * NF + f] = 0.5f * (rul * ul + rur * ur + sav1 * (pl + pr) - coex * (rr * ur - rl * ul));
    d.Finv32[2 * NF + f] = 0.5f * (rul * vl + rur * vr + sav2 * (pl + pr) - coex * (rr * vr - rl * vl));
    d.Finv32[3 * NF + f] = 0.5f * (rul * hl + rur * hr - coex * (rr * er - rl * el));
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k)
      d.Finv32[(4 + k) * NF + f] = 0.5f * (rul * Yl[k] + rur * Yr[k] - coex * (rr * Yr[k] - rl * Yl[k]));
  }
  // ---- viscous flux
  if (VISC) {
    float pl = uL[0], ul = uL[1], vl = uL[2], tl = uL[3];
    float pr, ur, vr, tr;
    float Yl[NSP], Yr[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) Yl[k] = YL0[k];
    if (NR >= 0) {
      pr = uR[0]; ur = uR[1]; vr = uR[2]; tr = uR[3];
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = YR0[k];
    } else if (NR == -3 || NR == -4) {
      const int w = NR == -3 ? 0 : 1;
      const float* bc = bc_row32(d, d.fcase, f);
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = bc[BC_Y + w * BC_NSPMAX + k];
      tr = bc[BC_T + w];
      float Cb, gb, Rb;
      gas32<NSP>(th, Yr, tr, Cb, gb, Rb, err);
      pr = pl;
      ur = bc[BC_MFLOW + w] / (pr / (Rb * tr));
      vr = 0.f;
      pl = pr; ul = ur; vl = vr; tl = tr;
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yl[k] = Yr[k];
    } else {
      if (NR == -1) { ul = 0.f; vl = 0.f; }
      else if (NR == -2 || NR == -6 || NR == -7) {
        const float vn = ul * sn1 + vl * sn2;
        ul -= vn * sn1;
        vl -= vn * sn2;
      }
      pr = pl; tr = tl; ur = ul; vr = vl;
      if (NR == -5) {
        const float ac = sqrtf(gl0 * pl / rl0);
        const float vn = ul * sn1 + vl * sn2;
        if (!(fabsf(vn) > ac)) {
          pr = bc_row32(d, d.fcase, f)[BC_POUT];
          ur = ul + sn1 * (pl - pr) / (rl0 * ac);
          vr = vl + sn2 * (pl - pr) / (rl0 * ac);
          tr = pr / (Rl0 * (rl0 + (pr - pl) / (ac * ac)));
          pl = pr; ul = ur; vl = vr; tl = tr;
        }
      } else if (NR == -7) {
        pr = 2.0e6f; tr = 700.f; ur = -100.f; vr = 0.f;
      }
#pragma unroll
      for (int k = 0; k < NSP; ++k) Yr[k] = Yl[k];
    }
    const float pp = 0.5f * (pl + pr), uu = 0.5f * (ul + ur), vv = 0.5f * (vl + vr), tem = 0.5f * (tl + tr);
    float YY[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) YY[k] = 0.5f * (Yl[k] + Yr[k]);
    float Cp, gama, Rc;
    gas32<NSP>(th, YY, tem, Cp, gama, Rc, err);
    const float rr = pp / (Rc * tem);
    float t0[V], t1[V];
    {
      const float dxl = (float)d.rinv[NL], dyl = (float)d.rinv[NE + NL];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        t0[k] = d.grad32[(2 * k) * NE + NL] * dxl;
        t1[k] = d.grad32[(2 * k + 1) * NE + NL] * dyl;
      }
    }
    if (NR >= 0) {
      const float rdxk = 1.f / (float)d.fdxk[f], y1 = (float)d.fysn[f], y2 = (float)d.fysn[NF + f];
      const float dxr = (float)d.rinv[NR], dyr = (float)d.rinv[NE + NR];
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const float du = (uR[k] - uL[k]) * rdxk;
        t0[k] = 0.5f * (t0[k] + d.grad32[(2 * k) * NE + NR] * dxr) + y1 * du;
        t1[k] = 0.5f * (t1[k] + d.grad32[(2 * k + 1) * NE + NR] * dyr) + y2 * du;
      }
    }
    float dudx = t0[1], dudy = t1[1], dvdx = t0[2], dvdy = t1[2], dtdx = t0[3], dtdy = t1[3];
    float dYdx[NSP], dYdy[NSP];
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) { dYdx[k] = t0[4 + k]; dYdy[k] = t1[4 + k]; }
    auto rmv = [](float& vx, float& vy, float nx, float ny) {
      const float vn = vx * nx + vy * ny;
      vx -= vn * nx;
      vy -= vn * ny;
    };
    if (NR == -1 || NR == -6) rmv(dtdx, dtdy, sn1, sn2);
    if (NR == -2) {
      const float snx = sn1, sny = sn2, stx = -sny, sty = snx;
      rmv(dtdx, dtdy, snx, sny);
#pragma unroll
      for (int k = 0; k < NSP - 1; ++k) rmv(dYdx[k], dYdy[k], snx, sny);
      float dutdx = dudx * stx + dvdx * sty, dutdy = dudy * stx + dvdy * sty;
      float dundx = dudx * snx + dvdx * sny, dundy = dudy * snx + dvdy * sny;
      rmv(dutdx, dutdy, snx, sny);
      rmv(dundx, dundy, stx, sty);
      dudx = dutdx * stx + dundx * snx;
      dudy = dutdy * stx + dundy * snx;
      dvdx = dutdx * sty + dundx * sny;
      dvdy = dutdy * sty + dundy * sny;
    }
    {
      float sx = 0.f, sy = 0.f;
#pragma unroll
      for (int k = 0; k < NSP - 1; ++k) { sx += dYdx[k]; sy += dYdy[k]; }
      dYdx[NSP - 1] = -sx;
      dYdy[NSP - 1] = -sy;
    }
    float entha[NSP], Dk[NSP], vmulc, akmu;
    enthalpy32<NSP>(th, tem, entha, err);
    transport32<NSP>(th, tem, YY, vmulc, akmu, err);
    diffusion32<NSP>(th, pp, tem, YY, Dk);
    float uicx = 0.f, uicy = 0.f;
#pragma unroll
    for (int k = 0; k < NSP; ++k) { uicx += Dk[k] * dYdx[k]; uicy += Dk[k] * dYdy[k]; }
    const float vlac = -2.f / 3.f * vmulc;
    const float div = dudx + dvdy;
    const float txx = 2.f * vmulc * dudx + vlac * div;
    const float tyy = 2.f * vmulc * dvdy + vlac * div;
    const float txy = vmulc * (dudy + dvdx);
    float sx = 0.f, sy = 0.f;
#pragma unroll
    for (int k = 0; k < NSP; ++k) {
      sx += (Dk[k] * dYdx[k] - YY[k] * uicx) * entha[k];
      sy += (Dk[k] * dYdy[k] - YY[k] * uicy) * entha[k];
    }
    const float qx = -akmu * dtdx - rr * sx;
    const float qy = -akmu * dtdy - rr * sy;
    const float btx = uu * txx + vv * txy - qx;
    const float bty = uu * txy + vv * tyy - qy;
    d.Fvis32[0 * NF + f] = -(sav1 * txx + sav2 * txy);
    d.Fvis32[1 * NF + f] = -(sav1 * txy + sav2 * tyy);
    d.Fvis32[2 * NF + f] = -(sav1 * btx + sav2 * bty);
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) {
      const float spx = rr * (Dk[k] * dYdx[k] - YY[k] * uicx);
      const float spy = rr * (Dk[k] * dYdy[k] - YY[k] * uicy);
      d.Fvis32[(3 + k) * NF + f] = -(sav1 * spx + sav2 * spy);
    }
  }
  if (err) atomicOr(d.err, err);
}

// Neumaier-compensated FP32 gather of the face fluxes into the FP64 residual.
__device__ __forceinline__ void neumaier(float& s, float& c, float x) {
  const float t = s + x;
  c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
  s = t;
}

template <int NSP>
__global__ void __launch_bounds__(128) k_gather32(const Dev d, int visc, int comb) {
  constexpr int V = 3 + NSP;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE, NF = d.NF, nf = d.nface[i];
  const unsigned lb = d.cleft[i];
  float s[V], c[V];
#pragma unroll
  for (int k = 0; k < V; ++k) { s[k] = 0.f; c[k] = 0.f; }
  for (int q = 0; q < nf; ++q) {
    const int f = d.cface[q * NE + i];
    const float sg = ((lb >> q) & 1u) ? -1.f : 1.f;
#pragma unroll
    for (int k = 0; k < V; ++k) neumaier(s[k], c[k], sg * d.Finv32[k * NF + f]);
    if (visc) {
#pragma unroll
      for (int k = 1; k < V; ++k) neumaier(s[k], c[k], sg * d.Fvis32[(k - 1) * NF + f]);
    }
  }
#pragma unroll
  for (int k = 0; k < V; ++k) {
    double R = (double)s[k] + (double)c[k];
    if (comb && k >= 4) R += d.src[(k - 4) * NE + i];
    d.hWA[k * NE + i] = R;
  }
}

// ---------------------------------------------------------------- LU-SGS ---
// Four lanes per cell as in the FP64 sweep; the off-diagonal terms in FP32,
// the diagonal division in FP64.
// The FP32 sweep step, split like the FP64 one (rc_core.cu): sweep_load32
// reads the data the sweep does not change (and forms the FP64 reciprocal of
// the diagonal), sweep_compute32 the increments and the arithmetic.
template <int NSP>
struct SweepPre32 {
  int i;
  bool valid, act;
  int j;
  float dx, dy, pp, uu, vv, tt, rr, gama, roe, aF;
  double rdd;
  float cs[NSP];
  float Yk[NSP > 1 ? NSP - 1 : 1];
};
template <int NSP, bool FWD>
__device__ __forceinline__ SweepPre32<NSP> sweep_load32(const Dev& d, int t, int tend, int q) {
  constexpr int DIR = FWD ? 0 : 1;
  SweepPre32<NSP> p;
  p.valid = t < tend;
  const int NE = d.NE, NF = d.NF;
  p.i = p.valid ? d.swi[DIR][t] : 0;
  p.j = p.valid ? d.swj[DIR][q * NE + t] : -1;
  const int fs = p.valid ? d.swf[DIR][q * NE + t] : 0;
  p.rdd = p.valid ? 1.0 / d.dd[p.i] : 0.0;
  p.act = p.j >= 0;
  if (p.act) {
    const int j = p.j, f = fs >= 0 ? fs : ~fs;
    p.dx = d.fvec32[f];
    p.dy = d.fvec32[NF + f];
    if (fs < 0) { p.dx = -p.dx; p.dy = -p.dy; }
    p.pp = d.PA32[0 * NE + j]; p.uu = d.PA32[1 * NE + j]; p.vv = d.PA32[2 * NE + j]; p.tt = d.PA32[3 * NE + j];
    p.rr = d.cst32[0 * NE + j]; p.gama = d.cst32[1 * NE + j]; p.roe = d.cst32[2 * NE + j];
    p.aF = d.alpaF32[f];
#pragma unroll
    for (int k = 0; k < NSP; ++k) p.cs[k] = d.cst32[(3 + k) * NE + j];
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) p.Yk[k] = d.PA32[(4 + k) * NE + j];
  }
  return p;
}
// The FP32 off-diagonal terms of one face slot (P: SweepPre32 or PairPre32;
// nb: the neighbour's FP32 increment dU32, V values) into c[V].
template <int NSP, class P>
__device__ __forceinline__ void terms32(const ThermoDev32<NSP>& th, const P& p, const float* nb, float* c) {
  const float dx = p.dx, dy = p.dy, pp = p.pp, uu = p.uu, vv = p.vv, tt = p.tt, rr = p.rr, gama = p.gama,
              roe = p.roe;
  const float rou = rr * uu, rov = rr * vv;
  const float drr = nb[0], dru = nb[1], drv = nb[2], dre = nb[3];
  float dry[NSP], s = 0.f;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { dry[k] = nb[4 + k]; s += dry[k]; }
  dry[NSP - 1] = drr - s;
  const float rinv = 1.f / rr;
  const float duu = (dru - uu * drr) * rinv;
  const float dvv = (drv - vv * drr) * rinv;
  float s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int k = 0; k < NSP; ++k) {
    s1 += p.cs[k] * dry[k];
    s2 += th.R[k] * dry[k];
  }
  const float gm1 = gama - 1.f;
  const float dpp = gm1 * (dre - s1 + tt * s2 * gama / gm1 - 0.5f * (dru * uu + duu * rou + drv * vv + dvv * rov));
  const float un = uu * dx + vv * dy, dun = duu * dx + dvv * dy;
  const float aF = p.aF;
  c[0] = 0.5f * (-aF * drr + dru * dx + drv * dy);
  c[1] = 0.5f * (-aF * dru + dru * un + rou * dun + dpp * dx);
  c[2] = 0.5f * (-aF * drv + drv * un + rov * dun + dpp * dy);
  c[3] = 0.5f * (-aF * dre + dun * (roe + pp) + un * (dre + dpp));
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) c[4 + k] = 0.5f * (-aF * dry[k] + dry[k] * un + rr * p.Yk[k] * dun);
}
// L2: read the sweep's values (own residual, the neighbour's FP32 increment)
// through L2, as the dataflow launch needs (other SMs write them during it)
template <int NSP, bool FWD, bool L2 = false>
__device__ __forceinline__ void sweep_compute32(const Dev& d, const ThermoDev32<NSP>& th, const SweepPre32<NSP>& p,
                                                int q, float* wsm) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
  auto ldd = [](const double* a) { return L2 ? __ldcg(a) : *a; };
  auto ldf = [](const float* a) { return L2 ? __ldcg(a) : *a; };
  double R0 = 0.0, R1 = 0.0;
  if (p.valid) {
    R0 = ldd(d.hWA + q * NE + p.i);
    if (q + 4 < V) R1 = ldd(d.hWA + (q + 4) * NE + p.i);
  }
  float c[V];
#pragma unroll
  for (int k = 0; k < V; ++k) c[k] = 0.f;
  if (p.act) {
    float nb[V];
#pragma unroll
    for (int k = 0; k < V; ++k) nb[k] = ldf(d.dU32 + k * NE + p.j);
    terms32<NSP>(th, p, nb, c);
  }
  // terms in slot order through the warp's shared scratch (see sweep_compute)
  const int lane = threadIdx.x & 31, base = lane & ~3;
  __syncwarp();
#pragma unroll
  for (int k = 0; k < V; ++k) wsm[k * 32 + lane] = c[k];
  __syncwarp();
  float df0 = 0.f, df1 = 0.f;
#pragma unroll
  for (int sl = 0; sl < 4; ++sl) {
    df0 += wsm[q * 32 + base + sl];
    if (q + 4 < V) df1 += wsm[(q + 4) * 32 + base + sl];
  }
  if (!p.valid) return;
  const double rdd = p.rdd;
  const double u0 = FWD ? (R0 - (double)df0) * rdd : R0 - (double)df0 * rdd;
  d.hWA[q * NE + p.i] = u0;
  d.dU32[q * NE + p.i] = (float)u0;
  if (q + 4 < V) {
    const double u1 = FWD ? (R1 - (double)df1) * rdd : R1 - (double)df1 * rdd;
    d.hWA[(q + 4) * NE + p.i] = u1;
    d.dU32[(q + 4) * NE + p.i] = (float)u1;
  }
}
template <int NSP, bool FWD>
__device__ __forceinline__ void sweep_step32(const Dev& d, const ThermoDev32<NSP>& th, int t, int tend, int q,
                                             float* wsm) {
  const SweepPre32<NSP> p = sweep_load32<NSP, FWD>(d, t, tend, q);
  sweep_compute32<NSP, FWD>(d, th, p, q, wsm);
}

// FP32 copies for the FP32 sweeps when the residual comes from the FP64
// kernels (defect-correction phase).
template <int NSP>
__global__ void __launch_bounds__(128) k_pack32(const Dev d) {
  constexpr int V = 3 + NSP;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE;
#pragma unroll
  for (int k = 0; k < V; ++k) d.PA32[k * NE + i] = (float)d.PA[k * NE + i];
#pragma unroll
  for (int k = 0; k < 3 + NSP; ++k) d.cst32[k * NE + i] = (float)d.cst[k * NE + i];
}

// one level, launched as a programmatic dependent of the previous one (see k_sweep4)
template <int NSP, bool FWD>
__global__ void __launch_bounds__(32) k_sweep32(const Dev d, const ThermoDev32<NSP> th, int t0, int t1) {
  pdl_launch_dependents();
  const int lt = threadIdx.x >> 2;
  __shared__ float wsm[32 * (3 + NSP)];
  const SweepPre32<NSP> p =
      sweep_load32<NSP, FWD>(d, lt < d.cpw ? t0 + blockIdx.x * d.cpw + lt : t1, t1, threadIdx.x & 3);
  pdl_wait();
  sweep_compute32<NSP, FWD>(d, th, p, threadIdx.x & 3, wsm);
}

// Both FP32 sweeps in one cooperative launch (chunks of d.cpw cells), ordered by per-level completion
// counters (the schedule of k_lusgs_persistent in rc_core.cu); the FP64
// update runs afterwards as its own kernel.
constexpr int PERS32_THREADS = 256;
template <int NSP>
__global__ void __launch_bounds__(PERS32_THREADS) k_lusgs_persistent32(const Dev d, const ThermoDev32<NSP> th,
                                                                       const int* __restrict__ foff, int nf,
                                                                       const int* __restrict__ boff, int nb,
                                                                       unsigned* cnt) {
  const int G = gridDim.x, wpb = PERS32_THREADS / 32, w = threadIdx.x >> 5;
  const int gw = blockIdx.x + w * G, nw = G * wpb;
  const int lt = (threadIdx.x & 31) >> 2, q = threadIdx.x & 3;
  __shared__ float wsm_all[PERS32_THREADS / 32][32 * (3 + NSP)];
  float* wsm = wsm_all[w];
  const int nl = nf + nb, cpw = d.cpw;
  auto nchunks = [&](int L) {
    const int a = L < nf ? foff[L] : boff[L - nf], b = L < nf ? foff[L + 1] : boff[L - nf + 1];
    return (unsigned)((b - a + cpw - 1) / cpw);
  };
  for (int L = 0; L < nl; ++L) {
    const bool fwd = L < nf;
    const int t0 = fwd ? foff[L] : boff[L - nf], t1 = fwd ? foff[L + 1] : boff[L - nf + 1];
    const int nch = (t1 - t0 + cpw - 1) / cpw;
    if (gw >= nch) continue;
    bool waited = L == 0;
    for (int c = gw; c < nch; c += nw) {
      const int t = lt < cpw ? t0 + c * cpw + lt : t1;
      if (fwd) {
        const SweepPre32<NSP> p = sweep_load32<NSP, true>(d, t, t1, q);
        if (!waited) {
          if (!wait_count(cnt + L - 1, nchunks(L - 1), d.err, d.spin_limit)) return;
          waited = true;
        }
        sweep_compute32<NSP, true>(d, th, p, q, wsm);
      } else {
        const SweepPre32<NSP> p = sweep_load32<NSP, false>(d, t, t1, q);
        if (!waited) {
          if (!wait_count(cnt + L - 1, nchunks(L - 1), d.err, d.spin_limit)) return;
          waited = true;
        }
        sweep_compute32<NSP, false>(d, th, p, q, wsm);
      }
      count_done(cnt + L);
    }
  }
}

// Both FP32 sweeps as a dataflow on the pass tables of k_lusgs_flow (one block
// per SM, its cells' passes in level order, each pass waiting only for the
// passes of other blocks that hold its neighbours).  An FP32 pass is short, so
// the work around it is split over two warps: warp 1 stages the passes'
// sweep_load32 data up to NBUF passes ahead into a ring of shared buffers
// (s_staged counts the staged passes, s_consumed the passes warp 0 has taken);
// warp 2 looks at the next pass's flags, hands each pass to warp 0 (barrier 3)
// once it is staged and its flags are set, and publishes each finished pass
// (barrier 4 from warp 0, then the flag = this launch's epoch), before any
// blocking wait, so that no block waits while holding a finished pass.  Warp 0
// runs the step of k_sweep32 (8 cells, 4 lanes each) with the sweep's values
// read through L2.  Every wait is bounded (ERR_SYNC).
// The FP64 Newton update (update_primitve_variables) of a cell needs only
// its own final increment, which its backward pass writes; the sweeps read
// neither WA nor PA (their FP32 copies PA32, cst32 stay as the iteration
// began), so warps 3 and 6 update the cells of each finished backward pass
// during the sweep, on the FP64 units of sub-partitions 3 and 2 that the
// FP32 passes leave idle (warps 4 and 5 only keep them there).  Warp 0
// counts its finished passes in s_done; update warp u takes the backward
// passes nf + u, nf + u + 2, ..., as many finished ones at a time as fill
// its 32 lanes with one cell each.  The update is the function k_update
// runs, compiled with the same flags, so the bits are the same.
constexpr int FLOW32_THREADS = 224, FLOW32_NBUF = 4;
template <int NSP>
__global__ void __launch_bounds__(FLOW32_THREADS, 1) k_lusgs_flow32(const Dev d, const ThermoDev32<NSP> th,
                                                                 const ThermoDev<NSP> th64, const FlowDev f) {
  __shared__ SweepPre32<NSP> s_pre[FLOW32_NBUF][32];
  __shared__ float wsm[32 * (3 + NSP)];
  __shared__ int s_cells[2][32];
  __shared__ unsigned s_epoch;
  __shared__ volatile int s_bad, s_staged, s_consumed, s_done;
  if (threadIdx.x == 0) {
    s_epoch = ld_acquire(f.ctr) + 1u;
    s_bad = 0;
    s_staged = 0;
    s_consumed = 0;
    s_done = 0;
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
  if (warp == 1) {
    for (int k = 0; k < n && !s_bad; ++k) {
      // pass k reuses the buffer of pass k - NBUF once warp 0 has taken it
      for (unsigned spin = 0; s_consumed < k - FLOW32_NBUF + 1 && !s_bad; ++spin)
        if (spin >= d.spin_limit) give_up();
      if (s_bad) break;
      const int pz = pass_of(k), t0 = f.pstart[pz], t1 = t0 + f.pcount[pz];
      if (k < nf) s_pre[k % FLOW32_NBUF][lane] = sweep_load32<NSP, true>(d, t0 + (lane >> 2), t1, lane & 3);
      else s_pre[k % FLOW32_NBUF][lane] = sweep_load32<NSP, false>(d, t0 + (lane >> 2), t1, lane & 3);
      __syncwarp();
      __threadfence_block();
      if (lane == 0) s_staged = k + 1;
      __syncwarp();
    }
  } else if (warp == 2) {
    auto staged = [&](int k) {  // wait (bounded) until pass k is staged
      for (unsigned spin = 0; s_staged <= k && !s_bad; ++spin)
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
      if (s_staged <= k) return false;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && ld_acquire(f.pflag + f.deps[d0 + u]) >= epoch;
      return __all_sync(0xffffffffu, ok) != 0;
    };
    if (n > 0) {
      staged(0);
      poll(0);
      bar_arrive(3, 64);
    }
    for (int k = 0; k < n; ++k) {
      const bool more = k + 1 < n;
      const bool go = more && ready(k + 1);
      if (go) __threadfence_block();
      bar_named(4, 64);
      if (go) bar_arrive(3, 64);
      if (lane == 0 && !s_bad) st_release(f.pflag + pass_of(k), epoch);
      if (more && !go) {
        poll(k + 1);
        staged(k + 1);
        bar_arrive(3, 64);
      }
    }
  } else if (warp == 0) {
    for (int k = 0; k < n; ++k) {
      bar_named(3, 64);
      // after a give-up warp 2 still hands every pass over (the barrier
      // counts must match) but warp 1 has stopped staging: the buffer may
      // hold no pass at all, so nothing of it is read
      if (s_bad) {
        bar_arrive(4, 64);
        continue;
      }
      const SweepPre32<NSP> p = s_pre[k % FLOW32_NBUF][lane];
      __syncwarp();
      __threadfence_block();
      if (lane == 0) s_consumed = k + 1;
      if (k < nf) sweep_compute32<NSP, true, true>(d, th, p, lane & 3, wsm);
      else sweep_compute32<NSP, false, true>(d, th, p, lane & 3, wsm);
      __syncwarp();
      __threadfence_block();
      if (lane == 0) s_done = k + 1;
      bar_arrive(4, 64);
    }
  } else if (warp == 3 || warp == 6) {
    const int u = warp == 3 ? 0 : 1;
    int* cells = s_cells[u];
    unsigned err = 0;
    for (int k = nf + u; k < n;) {
      // bounded wait for pass k; the polls are spaced out, as these warps
      // wait through the whole forward sweep and must not take issue slots
      // from warp 2 on their sub-partition
      for (unsigned spin = 0; s_done <= k && !s_bad; ++spin) {
        if (spin >= d.spin_limit) give_up();
        __nanosleep(256);
      }
      if (s_bad) break;
      __threadfence_block();
      const int avail = s_done;
      // lane l looks at this warp's pass k + 2l; the finished ones whose
      // cells fit in 32 lanes (a prefix of the lanes: at least pass k) are
      // taken, their sweep positions listed in order in cells[]
      const int kl = k + 2 * lane;
      int cnt = 0, t0 = 0;
      if (kl < avail) {
        const int pz = pass_of(kl);
        cnt = f.pcount[pz];
        t0 = f.pstart[pz];
      }
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
      }
      const bool take = kl < avail && incl <= 32;
      const int ntake = __popc(__ballot_sync(0xffffffffu, take));
      if (take)
        for (int c = 0; c < cnt; ++c) cells[incl - cnt + c] = t0 + c;
      const int ncell = __shfl_sync(0xffffffffu, incl, ntake - 1);
      __syncwarp();
      if (lane < ncell) update_cell<NSP>(d, th64, d.swi[1][cells[lane]], err);
      __syncwarp();
      k += 2 * ntake;
    }
    flag(d, err);
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

// Both FP32 sweeps as a dataflow on the compact pass tables of k_lusgs_flowc
// (rc_core.cu): a pass is split into G groups of at most flowc_cells(V)
// cells and 32 active (cell, slot) pairs.  Group g is two warps (2g, 2g+1):
// warp 2g forms the FP32 terms of its 32 pairs (terms32, one pair per lane)
// into the group's [cell][variable][slot] scratch, then both warps finish the
// group's cells in two rounds, thread x = 64 round + 32 h + lane taking
// variable x % V of cell x / V:
// the terms of the active slots added in slot order from +0 (the inactive
// slots' +0 terms of k_lusgs_flow32 leave such a sum unchanged: with FP32
// denormals flushed every partial sum is normal or +0), then the FP64
// division by the diagonal and the FP32 copy.  The work around a pass is
// k_lusgs_flowc's: two staging warps fill a ring of FLOWC32_NBUF shared
// slots ahead of the compute warps, and a coordinator warp looks at the next
// pass's flags, hands it over (barrier 3) once it is staged and the current
// pass is done (barrier 4), then publishes the finished pass; s_go[slot]
// (0 after a give-up) keeps both warps of a group on the same path.
// FLOWC32_UPD more warps run the FP64 Newton update of each finished
// backward pass during the sweep, as in k_lusgs_flow32 (the sweeps read only
// the FP32 copies PA32, cst32 of the state).  The update is FP64 work of
// about a quarter of a plain FP64 iteration's face flux: two warps per SM
// (k_lusgs_flow32) fall behind the compact sweep on a large mesh and finish
// long after its last pass, so there are enough update warps to keep each
// sub-partition's FP64 unit busy.  Seven keep the block at 12 warps, three
// per SM sub-partition, so a thread may hold the 149 registers the kernel
// uses; a fourth warp on a sub-partition caps it at 128 (on the 2,000,000-cell
// nozzle: 6 update warps 8.77 ms per mixed iteration, 7 warps 7.95, 8 warps
// 8.38 with 168 bytes of spills, 10 warps 8.99).  Every wait is bounded
// (ERR_SYNC).
constexpr int FLOWC32_NBUF = 4, FLOWC32_UPD = 7;
__host__ __device__ constexpr int flowc32_threads(int G) { return 32 * (2 * G + 3 + FLOWC32_UPD); }
template <int NSP>
struct PairPre32 {
  int j;   // the neighbour (-1: no pair in this lane)
  int cq;  // the pair's cell within its group << 2 | its slot
  float dx, dy, pp, uu, vv, tt, rr, gama, roe, aF;
  float cs[NSP];  // h_k of the neighbour
  float Yk[NSP > 1 ? NSP - 1 : 1];
};
// sweep_load32's reads for one active pair (position t, slot q)
template <int NSP, bool FWD>
__device__ __forceinline__ PairPre32<NSP> pair_load32(const Dev& d, int t, int q, int tg) {
  constexpr int DIR = FWD ? 0 : 1;
  const int NE = d.NE, NF = d.NF;
  PairPre32<NSP> p;
  const int j = d.swj[DIR][q * NE + t], fs = d.swf[DIR][q * NE + t], f = fs >= 0 ? fs : ~fs;
  p.j = j;
  p.cq = ((t - tg) << 2) | q;
  p.dx = d.fvec32[f];
  p.dy = d.fvec32[NF + f];
  if (fs < 0) { p.dx = -p.dx; p.dy = -p.dy; }
  p.pp = d.PA32[0 * NE + j]; p.uu = d.PA32[1 * NE + j]; p.vv = d.PA32[2 * NE + j]; p.tt = d.PA32[3 * NE + j];
  p.rr = d.cst32[0 * NE + j]; p.gama = d.cst32[1 * NE + j]; p.roe = d.cst32[2 * NE + j];
  p.aF = d.alpaF32[f];
#pragma unroll
  for (int k = 0; k < NSP; ++k) p.cs[k] = d.cst32[(3 + k) * NE + j];
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) p.Yk[k] = d.PA32[(4 + k) * NE + j];
  return p;
}
struct FinC32 {
  int i, mask;
  double rdd;  // 1 / dd of the cell
};
template <bool FWD>
__device__ __forceinline__ FinC32 finc_load32(const Dev& d, int t) {
  constexpr int DIR = FWD ? 0 : 1;
  FinC32 f;
  const int NE = d.NE;
  f.i = d.swi[DIR][t];
  f.rdd = 1.0 / d.dd[f.i];
  f.mask = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) f.mask |= (d.swj[DIR][q * NE + t] >= 0 ? 1 : 0) << q;
  return f;
}
template <int NSP, int G>
__global__ void __launch_bounds__(flowc32_threads(G), 1) k_lusgs_flowc32(const Dev d, const ThermoDev32<NSP> th,
                                                                        const ThermoDev<NSP> th64, const FlowDev f) {
  constexpr int V = 3 + NSP, T34 = 64 * G + 32, CW = 2 * G;  // compute warps 0 .. CW-1
  constexpr int CAP = flowc_cells(V);
  __shared__ PairPre32<NSP> s_pre[FLOWC32_NBUF][32 * G];
  __shared__ FinC32 s_fin[FLOWC32_NBUF][CAP * G];
  __shared__ float wsc[G][CAP * V * 4];
  __shared__ int s_cells[FLOWC32_UPD][32];
  __shared__ unsigned s_epoch;
  __shared__ volatile int s_bad, s_consumed, s_done;
  __shared__ volatile int s_slot[FLOWC32_NBUF], s_go[FLOWC32_NBUF];
  if (threadIdx.x == 0) {
    s_epoch = ld_acquire(f.ctr) + 1u;
    s_bad = 0;
    s_consumed = 0;
    s_done = 0;
    for (int s = 0; s < FLOWC32_NBUF; ++s) { s_slot[s] = 0; s_go[s] = 0; }
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
  if (warp == CW + 1 || warp == CW + 2) {
    // staging warp s: its passes s, s + 2, ... into the ring
    const int s = warp - CW - 1;
    for (int k = s; k < n && !s_bad; k += 2) {
      for (unsigned spin = 0; s_consumed < k - FLOWC32_NBUF + 1 && !s_bad; ++spin)
        if (spin >= d.spin_limit) give_up();
      if (s_bad) break;
      const int pz = pass_of(k), sl = k % FLOWC32_NBUF;
      int tg = f.pstart[pz];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int nc = f.gcell[pz * G + g], e0 = f.poff[pz * G + g], np = f.poff[pz * G + g + 1] - e0;
        PairPre32<NSP> pl;
        pl.j = -1;
        pl.cq = 0;
        if (lane < np) {
          const int e = f.plist[e0 + lane];
          pl = k < nf ? pair_load32<NSP, true>(d, e >> 2, e & 3, tg) : pair_load32<NSP, false>(d, e >> 2, e & 3, tg);
        }
        s_pre[sl][32 * g + lane] = pl;
        if (lane < CAP) {
          FinC32 fc = {-1, 0, 0.0};
          if (lane < nc) fc = k < nf ? finc_load32<true>(d, tg + lane) : finc_load32<false>(d, tg + lane);
          s_fin[sl][CAP * g + lane] = fc;
        }
        tg += nc;
      }
      __syncwarp();
      __threadfence_block();
      if (lane == 0) s_slot[sl] = k + 1;
      __syncwarp();
    }
  } else if (warp == CW) {
    // the coordinator
    auto staged = [&](int k) {
      for (unsigned spin = 0; s_slot[k % FLOWC32_NBUF] != k + 1 && !s_bad; ++spin)
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
      if (s_slot[k % FLOWC32_NBUF] != k + 1) return false;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && ld_acquire(f.pflag + f.deps[d0 + u]) >= epoch;
      return __all_sync(0xffffffffu, ok) != 0;
    };
    auto hand_over = [&](int k) {
      if (lane == 0) s_go[k % FLOWC32_NBUF] = s_bad ? 0 : 1;
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
      if (lane == 0) {
        s_consumed = k + 1;  // pass k's slot is free
        s_done = k + 1;      // and its increments are final
      }
      if (go) hand_over(k + 1);
      if (lane == 0 && !s_bad) st_release(f.pflag + pass_of(k), epoch);
      if (more && !go) {
        poll(k + 1);
        staged(k + 1);
        hand_over(k + 1);
      }
    }
  } else if (warp < CW) {
    const int gi = warp >> 1, h = warp & 1;
    float* wsm = wsc[gi];
    for (int k = 0; k < n; ++k) {
      bar_named(3, T34);
      const int sl = k % FLOWC32_NBUF;
      if (s_go[sl] && s_fin[sl][CAP * gi].i >= 0) {
        const bool fwd = k < nf;
        // the own residuals of this warp's two rounds of (cell, variable)
        int fc[2], r[2];
        FinC32 fn[2];
        double R[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int x = 64 * u + 32 * h + lane;
          fc[u] = x / V;
          r[u] = x - fc[u] * V;
          fn[u] = s_fin[sl][CAP * gi + min(fc[u], CAP - 1)];
          if (fc[u] >= CAP) fn[u].i = -1;
          R[u] = fn[u].i >= 0 ? __ldcg(d.hWA + r[u] * d.NE + fn[u].i) : 0.0;
        }
        if (h == 0) {
          const PairPre32<NSP> p = s_pre[sl][32 * gi + lane];
          if (p.j >= 0) {
            float nb[V], c[V];
#pragma unroll
            for (int v = 0; v < V; ++v) nb[v] = __ldcg(d.dU32 + v * d.NE + p.j);
            terms32<NSP>(th, p, nb, c);
            float* w = wsm + min(p.cq >> 2, CAP - 1) * V * 4 + (p.cq & 3);
#pragma unroll
            for (int v = 0; v < V; ++v) w[v * 4] = c[v];
          }
        }
        bar_named(5 + gi, 64);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (fn[u].i < 0) continue;
          const float* wf = wsm + fc[u] * V * 4 + r[u] * 4;
          float df = 0.f;
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if ((fn[u].mask >> q) & 1) df += wf[q];
          const double rdd = fn[u].rdd;
          const double uo = fwd ? (R[u] - (double)df) * rdd : R[u] - (double)df * rdd;
          d.hWA[r[u] * d.NE + fn[u].i] = uo;
          d.dU32[r[u] * d.NE + fn[u].i] = (float)uo;
        }
        // the scratch is written again by the next pass only after barrier 3,
        // which follows every warp's barrier 4 below
      }
      bar_arrive(4, T34);
    }
  } else {
    // the Newton update warps (CW + 3 ..): update warp u takes the cells of
    // the backward passes nf + u, nf + u + UPD, ... once finished, 32 at a
    // time, one per lane: a batch runs on from pass to pass and may end inside
    // one (off: the cells of pass k already taken)
    constexpr int UPD = FLOWC32_UPD;
    const int u = warp - CW - 3;
    int* cells = s_cells[u];
    unsigned err = 0;
    for (int k = nf + u, off = 0; k < n;) {
      for (unsigned spin = 0; s_done <= k && !s_bad; ++spin) {
        if (spin >= d.spin_limit) give_up();
        __nanosleep(256);
      }
      if (s_bad) break;
      __threadfence_block();
      const int avail = s_done;
      const int kl = k + UPD * lane;
      int cnt = 0, t0 = 0;
      if (kl < avail) {
        const int pz = pass_of(kl);
        cnt = f.pcount[pz];
        t0 = f.pstart[pz];
        if (lane == 0) {
          cnt -= off;
          t0 += off;
        }
      }
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
      }
      const int excl = incl - cnt;
      for (int c = 0; c < cnt && excl + c < 32; ++c) cells[excl + c] = t0 + c;
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      const int ncell = total < 32 ? total : 32;
      __syncwarp();
      if (lane < ncell) update_cell<NSP>(d, th64, d.swi[1][cells[lane]], err);
      __syncwarp();
      if (total <= 32) {
        // every finished pass of this warp taken whole
        k += UPD * __popc(__ballot_sync(0xffffffffu, kl < avail));
        off = 0;
      } else {
        // the batch ends inside candidate j (the first whose cells pass 32)
        const int j = __ffs(__ballot_sync(0xffffffffu, incl > 32)) - 1;
        const int ex = __shfl_sync(0xffffffffu, excl, j);
        off = (j == 0 ? off : 0) + (32 - ex);
        k += UPD * j;
      }
    }
    flag(d, err);
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

// ------------------------------------------------------- host launchers ----
inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

template <int NSP>
void mixed_ts_face(const Dev& d, const void* th32, int visc, cudaStream_t s) {
  const auto& th = *static_cast<const ThermoDev32<NSP>*>(th32);
  if (visc) k_ts_face32<NSP, true><<<nblk(d.NF, d.bs), d.bs, 0, s>>>(d, th);
  else k_ts_face32<NSP, false><<<nblk(d.NF, d.bs), d.bs, 0, s>>>(d, th);
}
template <int NSP>
void mixed_cell(const Dev& d, const void* th32, const ThermoDev<NSP>& th64, int do_step, int limit, int comb,
                int visc, cudaStream_t s) {
  k_cell32<NSP><<<nblk(d.NE, d.bs), d.bs, 0, s>>>(d, *static_cast<const ThermoDev32<NSP>*>(th32), th64, do_step,
                                                 limit, comb, visc);
}
template <int NSP>
void mixed_face_flux(const Dev& d, const void* th32, int visc, cudaStream_t s) {
  const auto& th = *static_cast<const ThermoDev32<NSP>*>(th32);
  if (visc) k_face_flux32<NSP, true><<<nblk(d.NF, d.bs), d.bs, 0, s>>>(d, th);
  else k_face_flux32<NSP, false><<<nblk(d.NF, d.bs), d.bs, 0, s>>>(d, th);
}
template <int NSP>
void mixed_pack(const Dev& d, cudaStream_t s) {
  k_pack32<NSP><<<nblk(d.NE, d.bs), d.bs, 0, s>>>(d);
}
template <int NSP>
void mixed_gather(const Dev& d, int visc, int comb, cudaStream_t s) {
  k_gather32<NSP><<<nblk(d.NE, d.bs), d.bs, 0, s>>>(d, visc, comb);
}
template <int NSP>
void mixed_sweep(const Dev& d, const void* th32, bool fwd, int t0, int t1, cudaStream_t s) {
  const auto& th = *static_cast<const ThermoDev32<NSP>*>(th32);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblk(t1 - t0, d.cpw));
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (fwd) cudaLaunchKernelEx(&cfg, k_sweep32<NSP, true>, d, th, t0, t1);
  else cudaLaunchKernelEx(&cfg, k_sweep32<NSP, false>, d, th, t0, t1);
}
// Cooperative launch of the persistent FP32 sweeps (level counters zeroed by the caller).
template <int NSP>
cudaError_t mixed_lusgs_persistent(const Dev& d, const void* th32, const int* foff, int nf, const int* boff, int nb,
                                   unsigned* count, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(PERS32_THREADS);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_lusgs_persistent32<NSP>, d, *static_cast<const ThermoDev32<NSP>*>(th32), foff, nf,
                            boff, nb, count);
}
// Cooperative launch of the dataflow FP32 sweeps with the fused FP64 Newton
// update, one block per SM (th32, th64: ThermoDev32<NSP>, ThermoDev<NSP>).
template <int NSP>
cudaError_t mixed_lusgs_flow(const Dev& d, const void* th32, const void* th64, const FlowDev& f, int grid,
                             cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(FLOW32_THREADS);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_lusgs_flow32<NSP>, d, *static_cast<const ThermoDev32<NSP>*>(th32),
                            *static_cast<const ThermoDev<NSP>*>(th64), f);
}
// Cooperative launch of the compact dataflow FP32 sweeps (G groups) with the
// fused FP64 Newton update, one block per SM.
template <int NSP>
cudaError_t mixed_lusgs_flowc(const Dev& d, const void* th32, const void* th64, const FlowDev& f, int G, int grid,
                              cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(flowc32_threads(G));
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const auto& t32 = *static_cast<const ThermoDev32<NSP>*>(th32);
  const auto& t64 = *static_cast<const ThermoDev<NSP>*>(th64);
  if (G == 2) return cudaLaunchKernelEx(&cfg, k_lusgs_flowc32<NSP, 2>, d, t32, t64, f);
  return cudaLaunchKernelEx(&cfg, k_lusgs_flowc32<NSP, 1>, d, t32, t64, f);
}
template <int NSP>
int mixed_flowc_occupancy(int G) {
  int nb = 0;
  if (G == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lusgs_flowc32<NSP, 2>, flowc32_threads(2), 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lusgs_flowc32<NSP, 1>, flowc32_threads(1), 0);
  return nb;
}
template <int NSP>
int mixed_flow_occupancy() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lusgs_flow32<NSP>, FLOW32_THREADS, 0);
  return nb;
}
template <int NSP>
int mixed_persistent_occupancy() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lusgs_persistent32<NSP>, PERS32_THREADS, 0);
  return nb;
}
template <int NSP>
size_t mixed_thermo(const void* th64, void* out) {
  if (out) make_thermo32<NSP>(*static_cast<const ThermoDev<NSP>*>(th64), *static_cast<ThermoDev32<NSP>*>(out));
  return sizeof(ThermoDev32<NSP>);
}

#define RC_MIXED_INST(N)                                                                                        \
  template void mixed_ts_face<N>(const Dev&, const void*, int, cudaStream_t);                                   \
  template void mixed_cell<N>(const Dev&, const void*, const ThermoDev<N>&, int, int, int, int, cudaStream_t);  \
  template void mixed_face_flux<N>(const Dev&, const void*, int, cudaStream_t);                                 \
  template void mixed_gather<N>(const Dev&, int, int, cudaStream_t);                                            \
  template void mixed_pack<N>(const Dev&, cudaStream_t);                                                        \
  template void mixed_sweep<N>(const Dev&, const void*, bool, int, int, cudaStream_t);                          \
  template size_t mixed_thermo<N>(const void*, void*);                                                       \
  template cudaError_t mixed_lusgs_persistent<N>(const Dev&, const void*, const int*, int, const int*, int,       \
                                                 unsigned*, int, cudaStream_t);                                 \
  template int mixed_persistent_occupancy<N>();                                                                 \
  template cudaError_t mixed_lusgs_flow<N>(const Dev&, const void*, const void*, const FlowDev&, int,           \
                                           cudaStream_t);                                                       \
  template int mixed_flow_occupancy<N>();                                                                       \
  template cudaError_t mixed_lusgs_flowc<N>(const Dev&, const void*, const void*, const FlowDev&, int, int,      \
                                            cudaStream_t);                                                      \
  template int mixed_flowc_occupancy<N>(int);
RC_MIXED_INST(1)
RC_MIXED_INST(4)

}  // namespace rc
