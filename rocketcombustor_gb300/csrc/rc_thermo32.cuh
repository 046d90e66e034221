// Single-precision thermochemistry for the mixed-precision form: the same
// point functions as rc_thermo.cuh (ComputeGasParameter, compute_enthalpy,
// compute_transport_property, compute_diffusion_velocity of the reference's
// src/combustion_modeling) evaluated in FP32 with the fast SFU math
// (__logf, __expf, __powf; the unit is built with approximate FP32 division
// and square root).  Used for the spectral radius, reconstruction, limiter and
// face fluxes; chemistry, the LU-SGS diagonal, Newton and norms stay FP64.
#pragma once
#include "rc_thermo.cuh"

namespace rc {

template <int NSP>
struct ThermoDev32 {
  float R[NSP], mw[NSP];
  float tlo, tcrit, thi;
  float cl[7][NSP], ch[7][NSP];
  float b1l[NSP], b1h[NSP];
  float trlo, trcrit, trhi;
  float mu[2][4][NSP], kk[2][4][NSP];
  float wc[NSP][NSP], wd[NSP][NSP];
  float dlj[NSP][NSP], dmw[NSP][NSP], dcd[NSP][NSP];
  float cfl;
};

template <int NSP>
void make_thermo32(const ThermoDev<NSP>& a, ThermoDev32<NSP>& b) {
  for (int i = 0; i < NSP; ++i) {
    b.R[i] = (float)a.R[i];
    b.mw[i] = (float)a.mw[i];
    b.b1l[i] = (float)a.b1l[i];
    b.b1h[i] = (float)a.b1h[i];
    for (int j = 0; j < 7; ++j) { b.cl[j][i] = (float)a.cl[j][i]; b.ch[j][i] = (float)a.ch[j][i]; }
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 4; ++c) { b.mu[r][c][i] = (float)a.mu[r][c][i]; b.kk[r][c][i] = (float)a.kk[r][c][i]; }
    for (int j = 0; j < NSP; ++j) {
      b.wc[i][j] = (float)a.wc[i][j]; b.wd[i][j] = (float)a.wd[i][j];
      b.dlj[i][j] = (float)a.dlj[i][j]; b.dmw[i][j] = (float)a.dmw[i][j]; b.dcd[i][j] = (float)a.dcd[i][j];
    }
  }
  b.tlo = (float)a.tlo; b.tcrit = (float)a.tcrit; b.thi = (float)a.thi;
  b.trlo = (float)a.trlo; b.trcrit = (float)a.trcrit; b.trhi = (float)a.trhi;
  b.cfl = (float)a.cfl;
}

__device__ __forceinline__ float fmin2f(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float fmax2f(float a, float b) { return (b > a) ? b : a; }

template <int NSP>
__device__ __forceinline__ void gas32(const ThermoDev32<NSP>& th, const float* Y, float tem, float& Cp, float& gama,
                                      float& Rcpcv, unsigned& err) {
  const float t2 = tem * tem, r1 = 1.0f / tem;
  const float b[7] = {r1 * r1, r1, 1.0f, tem, t2, tem * t2, t2 * t2};
  const bool low = (th.tlo <= tem && tem <= th.tcrit);
  if (!low && !(th.tcrit < tem && tem <= th.thi)) err |= ERR_THERMO_T;
  float c = 0.f, r = 0.f;
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 7; ++j) s += (low ? th.cl[j][i] : th.ch[j][i]) * b[j];
    c += s * th.R[i] * Y[i];
    r += th.R[i] * Y[i];
  }
  Cp = c;
  Rcpcv = r;
  gama = c / (c - r);
}

template <int NSP>
__device__ __forceinline__ void enthalpy32(const ThermoDev32<NSP>& th, float tem, float* entha, unsigned& err) {
  const float t2 = tem * tem, r1 = 1.0f / tem;
  const float e[7] = {-(r1 * r1), __logf(tem) * r1, 1.0f, 0.5f * tem, t2 * (1.f / 3.f), 0.25f * tem * t2, 0.2f * t2 * t2};
  const bool low = (th.tlo <= tem && tem <= th.tcrit);
  if (!low && !(th.tcrit < tem && tem <= th.thi)) err |= ERR_THERMO_T;
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 7; ++j) s += (low ? th.cl[j][i] : th.ch[j][i]) * e[j];
    entha[i] = th.R[i] * (tem * s + (low ? th.b1l[i] : th.b1h[i]));
  }
}

template <int NSP>
__device__ __forceinline__ void transport32(const ThermoDev32<NSP>& th, float tem2, const float* yy, float& vmul,
                                            float& akmu, unsigned& err) {
  const float tem = fmax2f(th.trlo, tem2);
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < NSP; ++i) s += yy[i] / th.mw[i];
  const float ww = 1.f / s;
  float xx[NSP], mul[NSP], Kl[NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i) xx[i] = ww * yy[i] / th.mw[i];
  const bool low = (th.trlo <= tem && tem <= th.trcrit);
  if (!low && !(th.trcrit < tem && tem <= th.trhi)) err |= ERR_TRANSPORT_T;
  const int rg = low ? 0 : 1;
  const float lt = __logf(tem), r1 = 1.f / tem, r2 = r1 * r1;
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    mul[i] = 1.0e-7f * __expf(th.mu[rg][0][i] * lt + th.mu[rg][1][i] * r1 + th.mu[rg][2][i] * r2 + th.mu[rg][3][i]);
    Kl[i] = 1.0e-4f * __expf(th.kk[rg][0][i] * lt + th.kk[rg][1][i] * r1 + th.kk[rg][2][i] * r2 + th.kk[rg][3][i]);
  }
  float v = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    float phil = 0.f;
#pragma unroll
    for (int j = 0; j < NSP; ++j) {
      const float sq = (i == j) ? 1.f : sqrtf(mul[i] / mul[j]);
      const float q = 1.f + sq * th.wc[i][j];
      phil += xx[j] * (q * q) / th.wd[i][j];
    }
    phil *= 0.35355339f;
    v += xx[i] * mul[i] / phil;
    s1 += xx[i] * Kl[i];
    s2 += xx[i] / Kl[i];
  }
  vmul = v;
  akmu = 0.5f * (s1 + 1.f / s2);
}

template <int NSP>
__device__ __forceinline__ void diffusion32(const ThermoDev32<NSP>& th, float pp, float tem, const float* YY,
                                            float* Dk) {
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < NSP; ++i) s += YY[i] / th.mw[i];
  const float ww = 1.f / s;
  float XX[NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i) XX[i] = ww * YY[i] / th.mw[i];
  const float num = 0.0266f * sqrtf(tem * tem * tem);
  float D[NSP][NSP];
#pragma unroll
  for (int i = 0; i < NSP; ++i)
#pragma unroll
    for (int j = i + 1; j < NSP; ++j) {
      const float tstar = tem / th.dlj[i][j];
      const float om = 1.06036f * __powf(tstar, -0.15610f) + 0.19300f * __expf(-0.47635f * tstar) +
                       1.03587f * __expf(-1.52996f * tstar) + 1.76474f * __expf(-3.89411f * tstar);
      const float dv = num / (pp * th.dmw[i][j] * th.dcd[i][j] * om);
      D[i][j] = dv;
      D[j][i] = dv;
    }
#pragma unroll
  for (int i = 0; i < NSP; ++i) {
    float xd = 0.f;
#pragma unroll
    for (int j = 0; j < NSP; ++j)
      if (j != i) xd += XX[j] / D[i][j];
    Dk[i] = (1.f - XX[i]) / (xd + 1.0e-16f);
  }
}

}  // namespace rc
