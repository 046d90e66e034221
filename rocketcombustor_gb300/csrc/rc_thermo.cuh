// Thermochemistry point functions of RocketCombustor on the device (FP64).
//
// Each function keeps the operation order of the reference routine it cites,
// so that with FMA contraction disabled (--fmad=false) +,-,*,/ and sqrt give
// the reference's IEEE results; exp/log/pow come from include/rc_math.h, the
// same code the CPU oracle runs, so the results are bit-identical.  Constants
// that depend on species data only (pair terms of the Wilke and Chapman-Enskog
// sums) are evaluated once on the host with the reference's expressions and
// passed in ThermoDev, with reciprocal pairs of the fixed divisors; divisions
// by those, and the transport fits' divisions by T and T^2, use the correctly
// rounded division of rc_div.cuh (the IEEE quotient bit for bit, four FP64
// operations instead of a division sequence).
#pragma once
#include <cstdint>

#include "rc_div.cuh"
#include "rc_math.h"

namespace rc {

enum : unsigned {
  ERR_THERMO_T = 1u, ERR_TRANSPORT_T = 2u, ERR_NEG_TIMESTEP = 4u, ERR_NEG_FACE = 8u,
  ERR_NAN = 16u, ERR_BCTYPE = 32u, ERR_SYNC = 64u, ERR_LINSOLVE = 128u
};

template <int NSP>
struct ThermoDev {
  double R[NSP];                 // R_species
  double mw[NSP];                // mole_weight
  double Rconstant;
  double tlo, tcrit, thi;        // thermo_{lowest,critical,highest}_tem
  double cl[7][NSP], ch[7][NSP]; // low/high_coef_Cp_species(j,i) -> [j][i]
  double b1l[NSP], b1h[NSP];     // low/high_enthalpy_b1
  double trlo, trcrit, trhi;     // transport_{lowest,critical,highest}_tem
  double mu[2][4][NSP];          // [low/high][A..D][species]
  double kk[2][4][NSP];
  double wc[NSP][NSP];           // (mole_weight(j)/mole_weight(i))**0.25
  double wd[NSP][NSP];           // sqrt(1. + mole_weight(i)/mole_weight(j))
  double dlj[NSP][NSP];          // sqrt(LJ_energy(i)*LJ_energy(j))
  double dmw[NSP][NSP];          // sqrt(2./(1./mw(i)+1./mw(j))*1000)
  double dcd[NSP][NSP];          // (0.5*(sigma(i)+sigma(j)))**2
  int model;                     // code_chemical_model
  double Af, E;                  // Af_react(1), E_react(1)
  double prodc[NSP];             // 1000*mole_weight(ks)*(coef_r-coef_f)
  double mw1000[2];              // mole_weight(1..2)*1000
  double cfl;
  // reciprocal pairs {RN(1/x), RN((1 - x RN(1/x)) RN(1/x))} of fixed divisors
  double mwr[NSP][2];            // of mw
  double wdr[NSP][NSP][2];       // of wd
  double dljr[NSP][NSP][2];      // of dlj
  double mw1000r[2][2];          // of mw1000
};

__device__ __forceinline__ double fmin2(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double fmax2(double a, double b) { return (b > a) ? b : a; }

// ComputeGasParameter (thermo_property.f90:78-112)
template <int NSP>
__device__ __forceinline__ void gas(const ThermoDev<NSP>& th, const double* Y, double tem, double& Cp,
                                    double& gama, double& Rcpcv, unsigned& err) {
  const double t2 = tem * tem;
  const double b[7] = {1.0 / t2, 1.0 / tem, 1.0, tem, t2, tem * t2, t2 * t2};
  const bool low = (th.tlo <= tem && tem <= th.tcrit);
  if (!low && !(th.tcrit < tem && tem <= th.thi)) err |= ERR_THERMO_T;
  double cps[NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 7; ++j) s = s + (low ? th.cl[j][i] : th.ch[j][i]) * b[j];
    cps[i] = s * th.R[i];
  }
  double c = 0.0, r = 0.0;
#pragma unroll
  for (int i = 0; i < NSP; ++i) c = c + cps[i] * Y[i];
#pragma unroll
  for (int i = 0; i < NSP; ++i) r = r + th.R[i] * Y[i];
  Cp = c;
  Rcpcv = r;
  gama = c / (c - r);
}

// compute_enthalpy (thermo_property.f90:114-144)
template <int NSP>
__device__ __forceinline__ void enthalpy(const ThermoDev<NSP>& th, double tem, double* entha, unsigned& err) {
  const double t2 = tem * tem;
  const double e[7] = {-(1.0 / t2), rcm::log(tem) / tem, 1.0, tem / 2.0, t2 / 3.0, (tem * t2) / 4.0, (t2 * t2) / 5.0};
  const bool low = (th.tlo <= tem && tem <= th.tcrit);
  if (!low && !(th.tcrit < tem && tem <= th.thi)) err |= ERR_THERMO_T;
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 7; ++j) s = s + (low ? th.cl[j][i] : th.ch[j][i]) * e[j];
    entha[i] = th.R[i] * (tem * s + (low ? th.b1l[i] : th.b1h[i]));
  }
}

// Newton_temperature (thermo_property.f90:146-180); returns T, sets Rcpcv.
template <int NSP>
__device__ __forceinline__ double newton_T(const ThermoDev<NSP>& th, double et, const double* Y, double t0,
                                           double& Rcpcv, unsigned& err) {
  double t = t0, Cp, gama;
  double entha[NSP];
  for (int it = 0; it < 200; ++it) {
    enthalpy<NSP>(th, t, entha, err);
    gas<NSP>(th, Y, t, Cp, gama, Rcpcv, err);
    double h = 0.0;
#pragma unroll
    for (int i = 0; i < NSP; ++i) h = h + Y[i] * entha[i];
    const double ft = h - Rcpcv * t - et;
    const double dft = Cp - Rcpcv;
    const double dtt = -ft / dft;
    t = t + dtt;
    t = fmax2(t, th.tlo);
    t = fmin2(t, th.thi);
    if (fabs(dtt) < 1.0e-5) break;
  }
  return t;
}

// compute_transport_property (transport_property.f90:78-125)
template <int NSP>
__device__ __forceinline__ void transport(const ThermoDev<NSP>& th, double tem2, const double* yy, double& vmul,
                                          double& akmu, unsigned& err) {
  const double tem = fmax2(th.trlo, tem2);
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NSP; ++i) s = s + div_rn(yy[i], th.mw[i], th.mwr[i]);
  const double ww = 1.0 / s;
  double xx[NSP], mul[NSP], Kl[NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i) xx[i] = div_rn(ww * yy[i], th.mw[i], th.mwr[i]);
  const bool low = (th.trlo <= tem && tem <= th.trcrit);
  if (!low && !(th.trcrit < tem && tem <= th.trhi)) err |= ERR_TRANSPORT_T;
  const int rg = low ? 0 : 1;
  const double lt = rcm::log(tem);
  const double t2 = tem * tem;
  const Recip rt = recip_of(tem), rt2 = recip_of(t2);
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    mul[i] = rcm::exp(th.mu[rg][0][i] * lt + div_rn(th.mu[rg][1][i], tem, rt.h, rt.l) +
                      div_rn(th.mu[rg][2][i], t2, rt2.h, rt2.l) + th.mu[rg][3][i]);
    Kl[i] = rcm::exp(th.kk[rg][0][i] * lt + div_rn(th.kk[rg][1][i], tem, rt.h, rt.l) +
                     div_rn(th.kk[rg][2][i], t2, rt2.h, rt2.l) + th.kk[rg][3][i]);
  }
#pragma unroll
  for (int i = 0; i < NSP; ++i) { mul[i] = mul[i] * 1.0e-7; Kl[i] = Kl[i] * 1.0e-4; }
  double v = 0.0;
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    double phil = 0.0;
#pragma unroll
    for (int j = 0; j < NSP; ++j) {
      // sqrt(mul(i)/mul(i)) is exactly 1
      const double sq = (i == j) ? 1.0 : sqrt(mul[i] / mul[j]);
      const double q = 1.0 + sq * th.wc[i][j];
      phil = phil + div_rn(xx[j] * (q * q), th.wd[i][j], th.wdr[i][j]);
    }
    phil = (0.25 * sqrt(2.0)) * phil;
    v = v + xx[i] * mul[i] / phil;
  }
  double s1 = 0.0, s2 = 0.0;
#pragma unroll
  for (int i = 0; i < NSP; ++i) s1 = s1 + xx[i] * Kl[i];
#pragma unroll
  for (int i = 0; i < NSP; ++i) s2 = s2 + xx[i] / Kl[i];
  vmul = v;
  akmu = 0.5 * (s1 + 1.0 / s2);
}

// compute_diffusion_velocity (diffusion_velocity.f90:55-118).  D_ij is
// symmetric bit for bit (every pair term is), so each pair is evaluated once;
// the diagonal D_ii is never used.
template <int NSP>
__device__ __forceinline__ void diffusion(const ThermoDev<NSP>& th, double pp, double tem, const double* YY,
                                          double* Dk) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NSP; ++i) s = s + div_rn(YY[i], th.mw[i], th.mwr[i]);
  const double ww = 1.0 / s;
  double XX[NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i) XX[i] = div_rn(ww * YY[i], th.mw[i], th.mwr[i]);
  const double num = 0.0266 * sqrt(tem * (tem * tem));
  double D[NSP][NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i)
#pragma unroll
    for (int j = i + 1; j < NSP; ++j) {
      const double tstar = div_rn(tem, th.dlj[i][j], th.dljr[i][j]);
      const double om = 1.06036 * rcm::pow(tstar, -0.15610) + 0.19300 * rcm::exp(-0.47635 * tstar) +
                        1.03587 * rcm::exp(-1.52996 * tstar) + 1.76474 * rcm::exp(-3.89411 * tstar);
      const double d = num / (pp * th.dmw[i][j] * th.dcd[i][j] * om);
      D[i][j] = d;
      D[j][i] = d;
    }
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    double xd = 0.0;
#pragma unroll
    for (int j = 0; j < NSP; ++j)
      if (j != i) xd = xd + XX[j] / D[i][j];
    Dk[i] = (1.0 - XX[i]) / (xd + 1.0e-16);
  }
}

// compute_production_rate (chemical_kinetics.f90:109-165)
template <int NSP>
__device__ __forceinline__ void production(const ThermoDev<NSP>& th, double T, double rho, const double* Y2,
                                           double* prod) {
  double kf;
  const double y0 = fmin2(1.0, fmax2(0.0, Y2[0]));
  if (th.model == 0) {
    const double y1 = fmin2(1.0, fmax2(0.0, Y2[NSP > 1 ? 1 : 0]));
    kf = th.Af * rcm::exp(-th.E / (th.Rconstant * T));
    kf = kf * rcm::pow(div_rn(y0 * rho, th.mw1000[0], th.mw1000r[0]), 0.2);
    kf = kf * rcm::pow(div_rn(y1 * rho, th.mw1000[1], th.mw1000r[1]), 1.3);
  } else {
    kf = (T > 710.0) ? 1e4 : 0.0;
    kf = kf * div_rn(y0 * rho, th.mw1000[0], th.mw1000r[0]);
  }
#pragma unroll
  for (int k = 0; k < NSP; ++k) prod[k] = th.prodc[k] * kf;
}

}  // namespace rc
