// Per-cell chemistry integrator on the device (FP64, built with --fmad=false).
//
// The reference has no chemistry ODE integrator; its explicit source adds
// vol*omega to the residual (sourceterm.f90:43-51).  This integrator is new.
// It is built on the reference's own Jacobians:
//   con_to_pri_jaco   Compute_Con_to_Pri_Jaco (Con_to_Pri_Jacobian.f90:1-87)
//   dwdp              compute_derivative_production_rate (chemical_kinetics.f90:167-265)
// and it keeps the operation order of the CPU oracle's restatement, so that
// the device result is bit-identical to the oracle's.
//
// chem_integrate: the isolated constant-volume adiabatic reactor of one cell
// over dt.  rho, u, v and e = h - R_mix T stay fixed and
// dY_k/dt = omega_k(T, rho, Y)/rho.  A substep of length hs is one linearly
// implicit (Rosenbrock-Euler) step in primitive variables:
//   (dU/dP - hs d omega/dP) dP = hs (0, 0, 0, 0, omega_1 .. omega_{Nsp-1}),
// solved by Gaussian elimination with partial pivoting.  Its flow rows keep
// rho, rho u, rho v and rho E.  Then Y += dP_Y, T comes from Newton_temperature
// at the fixed e (guess T + dP_T clamped to the thermo range), and
// p = rho R_mix T.
//
// Step control: d = max(max_k |dY_k| / (tol (|Y_k| + 1e-3)), |dT| / (0.1 tol T)).
// A substep with d > 1 is rejected and shortened to hs max(0.2, 0.9/d).  An
// accepted substep lets the next one grow to hs min(2, 0.9/d).  Substep
// number maxsub, and any attempt after 2 maxsub attempts, takes the remaining
// time unconditionally (implicit Euler is L-stable).
#pragma once
#include "rc_thermo.cuh"

namespace rc {

// dU/dP, row-major [V][V]; U = (rho, rho u, rho v, rho E, rho Y_1..), P = (p, u, v, T, Y_1..).
template <int NSP>
__device__ __forceinline__ void con_to_pri_jaco(const ThermoDev<NSP>& th, const double* pri, double* J,
                                                unsigned& err) {
  constexpr int V = 3 + NSP, NS1 = NSP - 1;
  const double p = pri[0], u = pri[1], v = pri[2], t = pri[3];
  double y2[NSP], entha[NSP], dhdy[NSP], drdy[NSP], Cp, gama, Rcpcv;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NS1; ++i) { y2[i] = pri[4 + i]; s = s + pri[4 + i]; }
  y2[NSP - 1] = 1. - s;
  gas<NSP>(th, y2, t, Cp, gama, Rcpcv, err);
  const double r = p / (Rcpcv * t);
  enthalpy<NSP>(th, t, entha, err);
  double h = entha[NSP - 1];
#pragma unroll
  for (int i = 0; i < NS1; ++i) {
    h = h + pri[4 + i] * (entha[i] - entha[NSP - 1]);
    dhdy[i] = entha[i] - entha[NSP - 1];
  }
  const double drdp = 1. / (Rcpcv * t), drdt = -p / (Rcpcv * t * t);
#pragma unroll
  for (int i = 0; i < NS1; ++i) drdy[i] = -(th.R[i] - th.R[NSP - 1]) * p / (t * Rcpcv * Rcpcv);
  const double ke = h + 0.5 * (u * u + v * v);
#pragma unroll
  for (int k = 0; k < V * V; ++k) J[k] = 0.0;
  J[0] = drdp; J[3] = drdt;
  J[V + 0] = u * drdp; J[V + 1] = r; J[V + 3] = u * drdt;
  J[2 * V + 0] = v * drdp; J[2 * V + 2] = r; J[2 * V + 3] = v * drdt;
  J[3 * V + 0] = ke * drdp - 1.; J[3 * V + 1] = r * u; J[3 * V + 2] = r * v; J[3 * V + 3] = r * Cp + ke * drdt;
#pragma unroll
  for (int i = 0; i < NS1; ++i) {
    const double yi = pri[4 + i];
    J[4 + i] = drdy[i];
    J[V + 4 + i] = u * drdy[i];
    J[2 * V + 4 + i] = v * drdy[i];
    J[3 * V + 4 + i] = ke * drdy[i] + r * dhdy[i];
    J[(4 + i) * V + 0] = drdp * yi;
    J[(4 + i) * V + 3] = drdt * yi;
#pragma unroll
    for (int j = 0; j < NS1; ++j) J[(4 + i) * V + 4 + j] = (j == i) ? r + yi * drdy[i] : yi * drdy[j];
  }
}

// d omega_i / dP, row-major [NSP-1][V].  Model 1 leaves dkfdy(3:) unset in
// the reference (chemical_kinetics.f90:228-243); it is taken as dkfdr*drdy(3:).
template <int NSP>
__device__ __forceinline__ void dwdp(const ThermoDev<NSP>& th, const double* pri, double* D, unsigned& err) {
  constexpr int V = 3 + NSP, NS1 = NSP - 1;
  const double p = pri[0], T = pri[3];
  double y[NSP], y2[NSP], drdy[NSP], dkf[V], Cp, gama, Rcpcv;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NS1; ++i) { y[i] = pri[4 + i]; y2[i] = y[i]; s = s + y[i]; }
  y2[NSP - 1] = 1. - s;
  gas<NSP>(th, y2, T, Cp, gama, Rcpcv, err);
  const double rho = p / (Rcpcv * T);
#pragma unroll
  for (int i = 0; i < NS1; ++i) y[i] = fmin2(1., fmax2(0., y[i]));
  if (y[0] < 1.0e-12) {
#pragma unroll
    for (int c = 0; c < V; ++c) dkf[c] = 0.;
  } else {
    double af = th.Af * rcm::exp(-th.E / (th.Rconstant * T));
    const double r1 = div_rn(y[0] * rho, th.mw1000[0], th.mw1000r[0]);
    const double dr1dr = div_rn(y[0], th.mw1000[0], th.mw1000r[0]);
    const double dr1dy1 = div_rn(rho, th.mw1000[0], th.mw1000r[0]);
    const double y1 = NS1 > 1 ? y[NS1 > 1 ? 1 : 0] : 0.0;
    const double r2 = div_rn(y1 * rho, th.mw1000[1], th.mw1000r[1]);
    const double dr2dr = div_rn(y1, th.mw1000[1], th.mw1000r[1]);
    const double dr2dy2 = div_rn(rho, th.mw1000[1], th.mw1000r[1]);
    const double drdp = rho / p, drdT = -rho / T;
#pragma unroll
    for (int i = 0; i < NS1; ++i) drdy[i] = -(th.R[i] - th.R[NSP - 1]) * rho / Rcpcv;
    double dkfdr, dkfdT, dkfdy[NSP];
    if (th.model == 0) {
      const double dter1_dr = 0.2 * rcm::pow(rho, -0.8) * rcm::pow(dr1dr, 0.2);
      dkfdr = af * (rcm::pow(r1, 0.2) * 1.3 * rcm::pow(r2, 0.3) * dr2dr + dter1_dr * rcm::pow(r2, 1.3));
      dkfdT = af * rcm::pow(r1, 0.2) * rcm::pow(r2, 1.3) * th.E / (th.Rconstant * T * T) + dkfdr * drdT;
      dkfdy[0] = af * 0.2 * rcm::pow(r1, -0.8) * dr1dy1 * rcm::pow(r2, 1.3) + dkfdr * drdy[0];
      if (NS1 > 1) dkfdy[1] = af * rcm::pow(r1, 0.2) * 1.3 * rcm::pow(r2, 0.3) * dr2dy2 + dkfdr * drdy[1];
    } else {
      af = 0.0;
      if (T > 710.0) af = 1e4;
      const double dter1_dr = dr1dr;
      dkfdr = af * (r1 * 0 * dr2dr + dter1_dr);
      dkfdT = 0.;
      dkfdy[0] = af * dr1dy1 + dkfdr * drdy[0];
      if (NS1 > 1) dkfdy[1] = af * r1 * 0 * dr2dy2 + dkfdr * drdy[1];
    }
#pragma unroll
    for (int i = 2; i < NS1; ++i) dkfdy[i] = dkfdr * drdy[i];
    dkf[0] = dkfdr * drdp; dkf[1] = 0.; dkf[2] = 0.; dkf[3] = dkfdT;
#pragma unroll
    for (int i = 0; i < NS1; ++i) dkf[4 + i] = dkfdy[i];
  }
#pragma unroll
  for (int i = 0; i < NS1; ++i)
#pragma unroll
    for (int k = 0; k < V; ++k) D[i * V + k] = th.prodc[i] * dkf[k];
}

// Gaussian elimination with partial pivoting, in place; b gets the solution.
// Returns false for a singular matrix.
template <int N>
__device__ __forceinline__ bool gepp_solve(double* A, double* b) {
#pragma unroll
  for (int k = 0; k < N; ++k) {
    int piv = k;
    double best = fabs(A[k * N + k]);
#pragma unroll
    for (int r = k + 1; r < N; ++r) {
      const double a = fabs(A[r * N + k]);
      if (a > best) { best = a; piv = r; }
    }
    if (!(best > 0.0)) return false;
    if (piv != k) {
#pragma unroll
      for (int r = k + 1; r < N; ++r)
        if (r == piv) {
#pragma unroll
          for (int c = 0; c < N; ++c) { const double tmp = A[k * N + c]; A[k * N + c] = A[r * N + c]; A[r * N + c] = tmp; }
          const double tb = b[k]; b[k] = b[r]; b[r] = tb;
        }
    }
    const double dk = A[k * N + k];
#pragma unroll
    for (int r = k + 1; r < N; ++r) {
      const double f = A[r * N + k] / dk;
#pragma unroll
      for (int c = k + 1; c < N; ++c) A[r * N + c] = A[r * N + c] - f * A[k * N + c];
      b[r] = b[r] - f * b[k];
    }
  }
#pragma unroll
  for (int k = N - 1; k >= 0; --k) {
    double s = b[k];
#pragma unroll
    for (int c = k + 1; c < N; ++c) s = s - A[k * N + c] * b[c];
    b[k] = s / A[k * N + k];
  }
  return true;
}

// Integrates primitive state P (in place) over dt; returns the accepted substeps.
template <int NSP>
__device__ __noinline__ int chem_integrate(const ThermoDev<NSP>& th, double* P, double dt, double tol, int maxsub,
                                           unsigned& err) {
  constexpr int V = 3 + NSP, NS1 = NSP - 1;
  double Y2[NSP], entha[NSP], A[V * V], J[V * V], D[(NS1 > 0 ? NS1 : 1) * V], b[V], prod[NSP], Cp, gama, Rcpcv;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NS1; ++i) { Y2[i] = P[4 + i]; s = s + Y2[i]; }
  Y2[NSP - 1] = 1. - s;
  gas<NSP>(th, Y2, P[3], Cp, gama, Rcpcv, err);
  const double rho = P[0] / (Rcpcv * P[3]);
  enthalpy<NSP>(th, P[3], entha, err);
  double h = 0.0;
#pragma unroll
  for (int i = 0; i < NSP; ++i) h = h + Y2[i] * entha[i];
  const double e = h - Rcpcv * P[3];
  double rem = dt, hs = dt;
  int nacc = 0, natt = 0;
  while (rem > 0.0) {
    const bool last = nacc + 1 >= maxsub || natt >= 2 * maxsub;
    if (last || hs > rem) hs = rem;
    con_to_pri_jaco<NSP>(th, P, J, err);
    dwdp<NSP>(th, P, D, err);
    double yc[NSP], sc = 0.0;
#pragma unroll
    for (int i = 0; i < NS1; ++i) { yc[i] = P[4 + i]; sc = sc + yc[i]; }
    yc[NSP - 1] = 1. - sc;
    production<NSP>(th, P[3], rho, yc, prod);
#pragma unroll
    for (int k = 0; k < V * V; ++k) A[k] = J[k];
#pragma unroll
    for (int i = 0; i < NS1; ++i)
#pragma unroll
      for (int c = 0; c < V; ++c) A[(4 + i) * V + c] = A[(4 + i) * V + c] - hs * D[i * V + c];
#pragma unroll
    for (int k = 0; k < 4; ++k) b[k] = 0.0;
#pragma unroll
    for (int i = 0; i < NS1; ++i) b[4 + i] = hs * prod[i];
    if (!gepp_solve<V>(A, b)) { err |= ERR_NAN; break; }
    ++natt;
    double d = fabs(b[3]) / (0.1 * tol * P[3]);
#pragma unroll
    for (int i = 0; i < NS1; ++i) d = fmax2(d, fabs(b[4 + i]) / (tol * (fabs(P[4 + i]) + 1.0e-3)));
    if (d > 1.0 && !last) {
      hs = hs * fmax2(0.2, 0.9 / d);
      continue;
    }
#pragma unroll
    for (int i = 0; i < NS1; ++i) P[4 + i] = P[4 + i] + b[4 + i];
    s = 0.0;
#pragma unroll
    for (int i = 0; i < NS1; ++i) { Y2[i] = P[4 + i]; s = s + Y2[i]; }
    Y2[NSP - 1] = 1. - s;
    const double tg = fmin2(fmax2(P[3] + b[3], th.tlo), th.thi);
    const double t = newton_T<NSP>(th, e, Y2, tg, Rcpcv, err);
    P[3] = t;
    P[0] = rho * Rcpcv * t;
    rem = rem - hs;
    ++nacc;
    if (d > 0.0) hs = hs * fmin2(2.0, 0.9 / d);
    else hs = 2.0 * hs;
    if (rem - hs < 0.01 * hs) hs = rem;
  }
  return nacc;
}

}  // namespace rc
