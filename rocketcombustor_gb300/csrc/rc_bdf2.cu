// Unsteady dual-time BDF2 stage of RocketCombustor on the device (FP64, built
// with --fmad=false): the implicit_time_method 5 branch of the main loop,
// BDF2_stage / BDF2_LU_SGS (Time_BDF2.f90:4-337).  The backward Euler stage
// (implicit_time_method 3, Time_BackwardEuler.f90:4-324) runs the same
// kernels: its source term is vol/dt WA, its diagonal and right-hand side
// those of phi = 0.
//
// Per inner iteration, after the residual assembly that the steady path
// shares (timestep, reconstruction, flux_sourceterm):
//   k_bdf2_prep    every cell at once: the diagonal dd, the BDF2 right-hand
//                  side hWA - (1+phi) vol/dt WA + fixed, the cell's system
//                  matrix dU/dP dd - vol d omega/dP (Time_BDF2.f90:121-129),
//                  its equilibration, LU factors and condition estimate (the
//                  LAPACK dgesvx steps below), and the gas state the
//                  neighbours' sweeps read;
//   k_bdf2_sweep   one level of the forward or backward sweep: eight lanes
//                  per cell, each face slot's flux difference of the
//                  neighbour's increment split over two lanes, the terms added
//                  in NeighF order, then the cell's 7x7 solve with one lane per
//                  row (interchanges, triangular solves and the iterative
//                  refinement of dgerfs through warp shuffles);
//   k_bdf2_update  PA += dP, then primitve_to_conserved_variables.
// The system matrix depends on PA, dd and vol only, so both sweeps share one
// factorisation; the reference recomputes the same matrix in each sweep and
// factors it the same way, so the results are the same bits.
//
// The per-cell solve restates reference LAPACK 3.12's dgesvx('E', 'N') as
// called by advanced_linear_solve_lapack (la_math.f90:120-213): dgeequ +
// dlaqge, dgetrf with partial pivoting, dgecon (dlacn2 over triangular
// solves; only its comparison with eps matters: the reference stops there),
// dgetrs and the refinement loop of dgerfs, in the operation order of the
// netlib routines, which the CPU oracle restates too.
#include "rc_chem.cuh"
#include "rc_dev.cuh"
#include "rc_div.cuh"

namespace rc {

namespace bdf2 {
constexpr double EPS = 1.1102230246251565e-16;     // dlamch('E') = 2^-53
constexpr double SFMIN = 2.2250738585072014e-308;  // dlamch('S') = 2^-1022
constexpr double PREC = 2.220446049250313e-16;     // dlamch('P') = 2^-52
constexpr unsigned FULL = 0xffffffffu;

// gas state of a cell as a neighbour (bnb planes)
enum : int { NB_RR = 0, NB_RRC, NB_RT, NB_RCT, NB_RCP, NB_HH, NB_EK, NB_ROU, NB_ROV, NB_ROEPP, NB_H };
template <int NSP>
__host__ __device__ constexpr int nb_ry() { return NB_H + NSP; }
template <int NSP>
__host__ __device__ constexpr int nb_rct() { return NB_H + NSP + (NSP - 1); }  // recip_of(Rcpcv T): 2 planes
template <int NSP>
__host__ __device__ constexpr int nbq() { return nb_rct<NSP>() + 2; }

__device__ __forceinline__ double mx(double a, double b) { return (b > a) ? b : a; }
__device__ __forceinline__ double mn(double a, double b) { return (b < a) ? b : a; }

// ---- dgesvx steps on one row-major N x N matrix, a[r*N + c] = A(r, c)
template <int N>
__device__ __forceinline__ int dgeequ(const double* a, double* r, double* c, double& rowcnd, double& colcnd,
                                      double& amax) {
  const double smlnum = SFMIN, bignum = 1.0 / smlnum;
#pragma unroll
  for (int i = 0; i < N; ++i) r[i] = 0.0;
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int i = 0; i < N; ++i) r[i] = mx(r[i], fabs(a[i * N + j]));
  double rcmin = bignum, rcmax = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) { rcmax = mx(rcmax, r[i]); rcmin = mn(rcmin, r[i]); }
  amax = rcmax;
  if (rcmin == 0.0) return 1;
#pragma unroll
  for (int i = 0; i < N; ++i) r[i] = 1.0 / mn(mx(r[i], smlnum), bignum);
  rowcnd = mx(rcmin, smlnum) / mn(rcmax, bignum);
#pragma unroll
  for (int j = 0; j < N; ++j) c[j] = 0.0;
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int i = 0; i < N; ++i) c[j] = mx(c[j], fabs(a[i * N + j]) * r[i]);
  rcmin = bignum; rcmax = 0.0;
#pragma unroll
  for (int j = 0; j < N; ++j) { rcmin = mn(rcmin, c[j]); rcmax = mx(rcmax, c[j]); }
  if (rcmin == 0.0) return 2;
#pragma unroll
  for (int j = 0; j < N; ++j) c[j] = 1.0 / mn(mx(c[j], smlnum), bignum);
  colcnd = mx(rcmin, smlnum) / mn(rcmax, bignum);
  return 0;
}
// dlaqge; returns bit 0 = rows scaled, bit 1 = columns scaled
template <int N>
__device__ __forceinline__ int dlaqge(double* a, const double* r, const double* c, double rowcnd, double colcnd,
                                      double amax) {
  const double thresh = 0.1, small = SFMIN / PREC, large = 1.0 / small;
  if (rowcnd >= thresh && amax >= small && amax <= large) {
    if (colcnd >= thresh) return 0;
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int i = 0; i < N; ++i) a[i * N + j] = c[j] * a[i * N + j];
    return 2;
  }
  if (colcnd >= thresh) {
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int i = 0; i < N; ++i) a[i * N + j] = r[i] * a[i * N + j];
    return 1;
  }
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int i = 0; i < N; ++i) a[i * N + j] = c[j] * r[i] * a[i * N + j];
  return 3;
}
// dgetrf (partial pivoting, unit L below the diagonal); returns 0 or the
// 1-based column of the first zero pivot
template <int N>
__device__ __forceinline__ int dgetrf(double* a, int* ipiv) {
  int info = 0;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    int jp = j;
    double m = fabs(a[j * N + j]);
#pragma unroll
    for (int i = j + 1; i < N; ++i)
      if (fabs(a[i * N + j]) > m) { jp = i; m = fabs(a[i * N + j]); }
    ipiv[j] = jp;
    if (a[jp * N + j] != 0.0) {
      if (jp != j) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const double t = a[j * N + k];
          a[j * N + k] = a[jp * N + k];
          a[jp * N + k] = t;
        }
      }
      if (j < N - 1) {
        if (fabs(a[j * N + j]) >= SFMIN) {
          const double rp = 1.0 / a[j * N + j];
#pragma unroll
          for (int i = j + 1; i < N; ++i) a[i * N + j] = rp * a[i * N + j];
        } else {
#pragma unroll
          for (int i = j + 1; i < N; ++i) a[i * N + j] = a[i * N + j] / a[j * N + j];
        }
      }
    } else if (info == 0) {
      info = j + 1;
    }
#pragma unroll
    for (int jj = j + 1; jj < N; ++jj) {
      if (a[j * N + jj] != 0.0) {
        const double temp = -1.0 * a[j * N + jj];
#pragma unroll
        for (int i = j + 1; i < N; ++i) a[i * N + jj] = a[i * N + jj] + a[i * N + j] * temp;
      }
    }
  }
  return info;
}
// the triangular solves of dgecon: kase 1 inv(L) then inv(U), kase 2 inv(U^T) then inv(L^T)
template <int N>
__device__ __forceinline__ void trs_kase(const double* af, int kase, double* x) {
  if (kase == 1) {
#pragma unroll
    for (int j = 0; j < N; ++j)
      if (x[j] != 0.0) {
        const double temp = x[j];
#pragma unroll
        for (int i = j + 1; i < N; ++i) x[i] = x[i] - temp * af[i * N + j];
      }
#pragma unroll
    for (int j = N - 1; j >= 0; --j)
      if (x[j] != 0.0) {
        x[j] = x[j] / af[j * N + j];
        const double temp = x[j];
#pragma unroll
        for (int i = j - 1; i >= 0; --i) x[i] = x[i] - temp * af[i * N + j];
      }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      double temp = x[j];
#pragma unroll
      for (int i = 0; i < j; ++i) temp = temp - af[i * N + j] * x[i];
      x[j] = temp / af[j * N + j];
    }
#pragma unroll
    for (int j = N - 1; j >= 0; --j) {
      double temp = x[j];
#pragma unroll
      for (int i = N - 1; i > j; --i) temp = temp - af[i * N + j] * x[i];
      x[j] = temp;
    }
  }
}
template <int N>
__device__ __forceinline__ double dasum(const double* x) {
  double t = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) t = t + fabs(x[i]);
  return t;
}
template <int N>
__device__ __forceinline__ int idamax(const double* x) {
  int k = 0;
  double m = fabs(x[0]);
#pragma unroll
  for (int i = 1; i < N; ++i)
    if (fabs(x[i]) > m) { k = i; m = fabs(x[i]); }
  return k;
}
// dgecon('1') with dlacn2 (at most 5 iterations) unrolled
template <int N>
__device__ double dgecon(const double* af, double anorm) {
  if (anorm == 0.0) return 0.0;
  if (isnan(anorm)) return anorm;
  double x[N], est, estold;
  int isgn[N];
#pragma unroll
  for (int i = 0; i < N; ++i) x[i] = 1.0 / (double)N;
  trs_kase<N>(af, 1, x);
  if (N == 1) {
    est = fabs(x[0]);
  } else {
    est = dasum<N>(x);
#pragma unroll
    for (int i = 0; i < N; ++i) { x[i] = (x[i] >= 0.0) ? 1.0 : -1.0; isgn[i] = x[i] >= 0.0 ? 1 : -1; }
    trs_kase<N>(af, 2, x);
    int j = idamax<N>(x), iter = 2;
    for (int guard = 0; guard < 8; ++guard) {
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = (i == j) ? 1.0 : 0.0;
      trs_kase<N>(af, 1, x);
      estold = est;
      est = dasum<N>(x);
      bool same = true;
#pragma unroll
      for (int i = 0; i < N; ++i)
        if ((x[i] >= 0.0 ? 1 : -1) != isgn[i]) same = false;
      if (same || est <= estold) break;
#pragma unroll
      for (int i = 0; i < N; ++i) { x[i] = (x[i] >= 0.0) ? 1.0 : -1.0; isgn[i] = x[i] >= 0.0 ? 1 : -1; }
      trs_kase<N>(af, 2, x);
      const int jlast = j;
      j = idamax<N>(x);
      double xl = 0.0;
#pragma unroll
      for (int i = 0; i < N; ++i)
        if (i == jlast) xl = x[i];
      double xj = 0.0;
#pragma unroll
      for (int i = 0; i < N; ++i)
        if (i == j) xj = x[i];
      if (xl != fabs(xj) && iter < 5) { iter = iter + 1; continue; }
      break;
    }
    double altsgn = 1.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      x[i] = altsgn * (1.0 + (double)i / (double)(N - 1));
      altsgn = -altsgn;
    }
    trs_kase<N>(af, 1, x);
    const double temp = 2.0 * (dasum<N>(x) / (double)(3 * N));
    if (temp > est) est = temp;
  }
  if (est != 0.0) return (1.0 / est) / anorm;
  return 0.0;
}

// ---- the per-row solve of one cell's system by its eight lanes
// x: this row's right-hand side (already row-scaled); returns A^-1 x for this
// row (dgetrs('N')): the composed interchanges, then the column-oriented unit
// lower and upper solves of dtrsm, skipping zero entries as dtrsm does.  The
// divisions by the diagonal of U use its reciprocal pairs urh, url (div_rn:
// the same bits as the IEEE division).
template <int N>
__device__ __forceinline__ double getrs_rows(double x, int src, const double* lu, const double* ukk,
                                             const double* urh, const double* url, int r, int base) {
  x = __shfl_sync(FULL, x, base + src);
#pragma unroll
  for (int k = 0; k < N - 1; ++k) {
    const double xk = __shfl_sync(FULL, x, base + k);
    if (r > k && r < N && nonzero(xk)) x = x - xk * lu[k];
  }
#pragma unroll
  for (int k = N - 1; k >= 0; --k) {
    double xk = __shfl_sync(FULL, x, base + k);
    if (nonzero(xk)) {
      xk = div_rn(xk, ukk[k], urh[k], url[k]);
      if (r == k) x = xk;
      else if (r < k) x = x - xk * lu[k];
    }
  }
  return x;
}
}  // namespace bdf2

// fixed = vol/dt ((1+2 phi) WP - phi WP2) (Time_BDF2.f90:88-92), or for
// backward Euler vol/dt WA (Time_BackwardEuler.f90:75-79)
template <int NSP>
__global__ void __launch_bounds__(128) k_bdf2_fixed(const Dev d, int euler) {
  constexpr int V = 3 + NSP;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE;
  const double dt = d.bpar[0], phi = d.bpar[1];
  const double vd = d.vol[i] / dt;
#pragma unroll
  for (int k = 0; k < V; ++k)
    d.bfix[k * NE + i] = euler ? vd * d.WA[k * NE + i]
                               : vd * ((1 + 2 * phi) * d.WP[k * NE + i] - phi * d.WP2[k * NE + i]);
}

// Everything of BDF2_LU_SGS that the sweeps do not change, one thread per cell.
template <int NSP>
__global__ void __launch_bounds__(128) k_bdf2_prep(const Dev d, const ThermoDev<NSP> th) {
  using namespace bdf2;
  constexpr int V = 3 + NSP, RW = 2 * V + 4;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE;
  const double dt = d.bpar[0], phi = d.bpar[1], vol = d.vol[i];
  unsigned err = 0;
  // diagonal (Time_BDF2.f90:94-102) and right-hand side (:104-111)
  double s = 0.0;
  const int nf = d.nface[i];
  for (int q = 0; q < nf; ++q) s = s + 0.5 * d.alpaF[d.cface[q * NE + i]];
  const double ddi = s + vol * (1. / d.step[i] + (1 + phi) / dt);
#pragma unroll
  for (int k = 0; k < V; ++k)
    d.hWA[k * NE + i] = d.hWA[k * NE + i] - (1 + phi) * vol / dt * d.WA[k * NE + i] + d.bfix[k * NE + i];
  // system matrix (:121-129)
  double pri[V];
#pragma unroll
  for (int k = 0; k < V; ++k) pri[k] = d.PA[k * NE + i];
  double a[V * V];
  con_to_pri_jaco<NSP>(th, pri, a, err);
#pragma unroll
  for (int k = 0; k < V * V; ++k) a[k] = a[k] * ddi;
  if (NSP > 1) {
    double dw[(NSP > 1 ? NSP - 1 : 1) * V];
    dwdp<NSP>(th, pri, dw, err);
#pragma unroll
    for (int j = 0; j < NSP - 1; ++j)
#pragma unroll
      for (int c = 0; c < V; ++c) a[(4 + j) * V + c] = a[(4 + j) * V + c] - vol * dw[j * V + c];
  }
  // dgesvx('E'): equilibrate, factor, condition estimate.  The equilibrated
  // matrix goes to the cell's record and gives its 1-norm (dlange('1')) before
  // the factorisation overwrites it in registers, so one V x V array is live
  // instead of two (the same operations as factoring a copy).
  double rs[V], cs[V], rowcnd = 0, colcnd = 0, amax = 0;
  int equ = 0;
  if (dgeequ<V>(a, rs, cs, rowcnd, colcnd, amax) == 0) equ = dlaqge<V>(a, rs, cs, rowcnd, colcnd, amax);
  double* m = d.bmat + (size_t)i * V * RW;
  double anorm = 0.0;
#pragma unroll
  for (int j = 0; j < V; ++j) {
    double sum = 0.0;
#pragma unroll
    for (int r = 0; r < V; ++r) sum = sum + fabs(a[r * V + j]);
    if (anorm < sum || isnan(sum)) anorm = sum;
  }
#pragma unroll
  for (int r = 0; r < V; ++r)
#pragma unroll
    for (int c = 0; c < V; ++c) m[r * RW + c] = a[r * V + c];
  double* af = a;
  int ipiv[V];
  const int info = dgetrf<V>(af, ipiv);
  if (info > 0) {
    err |= ERR_LINSOLVE;
  } else {
    if (dgecon<V>(af, anorm) < EPS) err |= ERR_LINSOLVE;
  }
  int src[V];
#pragma unroll
  for (int k = 0; k < V; ++k) src[k] = k;
#pragma unroll
  for (int k = 0; k < V; ++k) {
    const int p = ipiv[k], t = src[k];
    src[k] = src[p];
    src[p] = t;
  }
#pragma unroll
  for (int r = 0; r < V; ++r) {
#pragma unroll
    for (int c = 0; c < V; ++c) m[r * RW + V + c] = af[r * V + c];
    m[r * RW + 2 * V] = rs[r];
    m[r * RW + 2 * V + 1] = cs[r];
    const Recip ru = recip_of(af[r * V + r]);
    m[r * RW + 2 * V + 2] = ru.h;
    m[r * RW + 2 * V + 3] = ru.l;
    d.bperm[i * 8 + r] = src[r];
  }
  d.bperm[i * 8 + 7] = equ;
  // this cell's gas state for its neighbours' sweeps (Time_BDF2.f90:145-166)
  double yy[NSP], entha[NSP], Cp, gama, Rcpcv;
  double sy = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { yy[k] = pri[4 + k]; sy = sy + yy[k]; }
  yy[NSP - 1] = 1. - sy;
  const double pp = pri[0], uu = pri[1], vv = pri[2], tt = pri[3];
  gas<NSP>(th, yy, tt, Cp, gama, Rcpcv, err);
  enthalpy<NSP>(th, tt, entha, err);
  double hh = 0.0;
#pragma unroll
  for (int k = 0; k < NSP; ++k) hh = hh + yy[k] * entha[k];
  const double rct = Rcpcv * tt, rr = pp / rct, ek = 0.5 * (uu * uu + vv * vv);
  double* nb = d.bnb;
  nb[NB_RR * NE + i] = rr;
  nb[NB_RRC * NE + i] = rr * Rcpcv;
  nb[NB_RT * NE + i] = rr * tt;
  nb[NB_RCT * NE + i] = rct;
  nb[NB_RCP * NE + i] = rr * Cp;
  nb[NB_HH * NE + i] = hh;
  nb[NB_EK * NE + i] = ek;
  nb[NB_ROU * NE + i] = rr * uu;
  nb[NB_ROV * NE + i] = rr * vv;
  nb[NB_ROEPP * NE + i] = (rr * (hh + ek) - pp) + pp;
#pragma unroll
  for (int k = 0; k < NSP; ++k) nb[(NB_H + k) * NE + i] = entha[k];
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) nb[(nb_ry<NSP>() + k) * NE + i] = rr * yy[k];
  const Recip rc = recip_of(rct);
  nb[nb_rct<NSP>() * NE + i] = rc.h;
  nb[(nb_rct<NSP>() + 1) * NE + i] = rc.l;
  flag(d, err);
}

// What a sweep does not change, loaded before the wait for the previous level:
// the face of slot q of the cell at level position t and its neighbour's gas
// state (BSlot), and row r of the cell's factorised system (BRow).
template <int NSP>
struct BSlot {
  int j;
  bool act;
  double dx, dy, aF, uu, vv, rr, rrc, rt, rct, rcth, rctl, unormal, rou, rov, rcp, hh, ek, roepp;
  double ent[NSP], yy[NSP], ry[NSP];
};
template <int NSP, bool FWD>
__device__ __forceinline__ BSlot<NSP> bslot_load(const Dev& d, int t, bool valid, int q) {
  using namespace bdf2;
  constexpr int DIR = FWD ? 0 : 1;
  const int NE = d.NE, NF = d.NF;
  BSlot<NSP> b;
  b.j = valid ? d.swj[DIR][q * NE + t] : -1;
  b.act = b.j >= 0;
  b.dx = b.dy = b.aF = b.uu = b.vv = b.rr = b.rrc = b.rt = b.rct = b.rctl = b.unormal = 0.0;
  b.rou = b.rov = b.rcp = b.hh = b.ek = b.roepp = 0.0;
  b.rcth = 1.0;
#pragma unroll
  for (int k = 0; k < NSP; ++k) { b.ent[k] = 0.0; b.yy[k] = 0.0; b.ry[k] = 0.0; }
  if (b.act) {
    const int j = b.j, fs = d.swf[DIR][q * NE + t], f = fs >= 0 ? fs : ~fs;
    b.dx = d.fvec[f];
    b.dy = d.fvec[NF + f];
    if (fs < 0) { b.dx = -b.dx; b.dy = -b.dy; }
    b.aF = d.alpaF[f];
    b.uu = d.PA[1 * NE + j];
    b.vv = d.PA[2 * NE + j];
    const double* nb = d.bnb;
    b.rr = nb[NB_RR * NE + j]; b.rrc = nb[NB_RRC * NE + j]; b.rt = nb[NB_RT * NE + j]; b.rct = nb[NB_RCT * NE + j];
    b.rcth = nb[nb_rct<NSP>() * NE + j]; b.rctl = nb[(nb_rct<NSP>() + 1) * NE + j];
    b.unormal = b.uu * b.dx + b.vv * b.dy;
    b.rou = nb[NB_ROU * NE + j];
    b.rov = nb[NB_ROV * NE + j];
    b.rcp = nb[NB_RCP * NE + j]; b.hh = nb[NB_HH * NE + j]; b.ek = nb[NB_EK * NE + j];
    b.roepp = nb[NB_ROEPP * NE + j];
#pragma unroll
    for (int k = 0; k < NSP; ++k) b.ent[k] = nb[(NB_H + k) * NE + j];
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) {
      b.yy[k] = d.PA[(4 + k) * NE + j];
      b.ry[k] = nb[(nb_ry<NSP>() + k) * NE + j];
    }
  }
  return b;
}
template <int NSP>
struct BRow {
  double arow[3 + NSP], lrow[3 + NSP], ukk[3 + NSP], urh[3 + NSP], url[3 + NSP], rsc, csc;
  int src, equ;
};
template <int NSP>
__device__ __forceinline__ BRow<NSP> brow_load(const Dev& d, int i, bool valid, int r) {
  constexpr int V = 3 + NSP, RW = 2 * V + 4;
  BRow<NSP> w;
  w.rsc = 1.0; w.csc = 1.0; w.src = 0; w.equ = 0;
#pragma unroll
  for (int k = 0; k < V; ++k) { w.arow[k] = 0.0; w.lrow[k] = 0.0; w.ukk[k] = 1.0; w.urh[k] = 1.0; w.url[k] = 0.0; }
  if (valid) {
    const double* m = d.bmat + (size_t)i * V * RW;
    if (r < V) {
#pragma unroll
      for (int k = 0; k < V; ++k) { w.arow[k] = m[r * RW + k]; w.lrow[k] = m[r * RW + V + k]; }
      w.rsc = m[r * RW + 2 * V];
      w.csc = m[r * RW + 2 * V + 1];
      w.src = d.bperm[i * 8 + r];
    }
#pragma unroll
    for (int k = 0; k < V; ++k) {
      w.ukk[k] = m[k * RW + V + k];
      w.urh[k] = m[k * RW + 2 * V + 2];
      w.url[k] = m[k * RW + 2 * V + 3];
    }
    w.equ = d.bperm[i * 8 + 7];
  }
  return w;
}
// The flux difference of slot b's neighbour increment dP (Time_BDF2.f90:168-197),
// rows 1-3 (lo) or rows 4.. (energy and species) of the slot's terms.
// L2: the neighbour's increment read through L2 (ld.global.cg), as the
// dataflow launch needs (other SMs write it during the launch).
template <int NSP, bool L2 = false>
__device__ __forceinline__ void bslot_terms(const Dev& d, const ThermoDev<NSP>& th, const BSlot<NSP>& b, bool lo,
                                            double* c) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
  auto ld = [](const double* p) { return L2 ? __ldcg(p) : *p; };
#pragma unroll
  for (int k = 0; k < V; ++k) c[k] = 0.0;
  if (!b.act) return;
  const int j = b.j;
  const double dpp = ld(d.hWA + 0 * NE + j), duu = ld(d.hWA + 1 * NE + j), dvv = ld(d.hWA + 2 * NE + j),
               dtt = ld(d.hWA + 3 * NE + j);
  double dyy[NSP], s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { dyy[k] = ld(d.hWA + (4 + k) * NE + j); s = s + dyy[k]; }
  dyy[NSP - 1] = -s;
  double s1 = 0.0;
#pragma unroll
  for (int k = 0; k < NSP; ++k) s1 = s1 + th.R[k] * dyy[k];
  const double drr = div_rn(dpp - b.rrc * dtt - b.rt * s1, b.rct, b.rcth, b.rctl);
  const double dunormal = duu * b.dx + dvv * b.dy;
  const double aF = b.aF, unormal = b.unormal, rr = b.rr;
  if (lo) {
    const double dru = rr * duu + b.uu * drr;
    const double drv = rr * dvv + b.vv * drr;
    c[0] = 0.5 * (-aF * drr + dru * b.dx + drv * b.dy);
    c[1] = 0.5 * (-aF * dru + dru * unormal + b.rou * dunormal + dpp * b.dx);
    c[2] = 0.5 * (-aF * drv + drv * unormal + b.rov * dunormal + dpp * b.dy);
  } else {
    double s2 = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; ++k) s2 = s2 + b.ent[k] * dyy[k];
    const double dre = b.rcp * dtt + rr * s2 + b.hh * drr + rr * (b.uu * duu + b.vv * dvv) + b.ek * drr - dpp;
    c[3] = 0.5 * (-aF * dre + dunormal * b.roepp + unormal * (dre + dpp));
#pragma unroll
    for (int k = 0; k < NSP - 1; ++k) {
      const double dry = rr * dyy[k] + b.yy[k] * drr;
      c[4 + k] = 0.5 * (-aF * dry + dry * unormal + b.ry[k] * dunormal);
    }
  }
}
template <int NSP>
__device__ __forceinline__ void bslot_put(double* w, bool lo, int q, const double* c) {
  constexpr int V = 3 + NSP;
  if (lo) {
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k * 4 + q] = c[k];
  } else {
#pragma unroll
    for (int k = 3; k < V; ++k) w[k * 4 + q] = c[k];
  }
}
// the backward error of one refinement pass over a cell's rows (8 lanes):
// max over the rows of |y| / w (or the guarded form), as a bit pattern
template <int V>
__device__ __forceinline__ long long berr_bits(double y, double wk, int r) {
  using namespace bdf2;
  const double safe1 = (V + 1) * SFMIN, safe2 = safe1 / EPS;
  long long vb = 0;
  if (r < V) vb = dbits((dbits(wk) > dbits(safe2)) ? fabs(y) / wk : (fabs(y) + safe1) / (wk + safe1));
  vb = max(vb, (long long)__shfl_xor_sync(FULL, (unsigned long long)vb, 1));
  vb = max(vb, (long long)__shfl_xor_sync(FULL, (unsigned long long)vb, 2));
  vb = max(vb, (long long)__shfl_xor_sync(FULL, (unsigned long long)vb, 4));
  return vb;
}

// The sweep step of up to four cells on one warp, eight lanes per cell (lane
// = 8 cell + r; lanes of cell slots >= CPW only join the shuffles): the flux
// differences of the neighbours' increments (sp: this lane's slot, q = r % 4,
// rows 1-3 on lanes r < 4, rows 4.. on the others), added in NeighF order
// through w (this warp's [cell][row][slot] scratch), then the cell's system
// (rw: row r of its factorisation) solved with one lane per row and refined
// as dgerfs does; hown is the cell's own increment (row r), i its index.
// PART 0: the whole step on this warp.  PART 1 and 2: two warps (warp 0 and
// warp 1 of the block) on the same cells, PART 1 forming rows 1-3 of every
// slot's terms, PART 2 rows 4..; they meet at named barrier 6 (64 threads),
// after which PART 1 solves and PART 2 returns.  The terms, their places in w
// and the sums are the same in every PART.
template <int NSP, bool FWD, int CPW, bool L2, int PART = 0>
__device__ __forceinline__ void bdf2_cell_step(const Dev& d, const ThermoDev<NSP>& th, const BSlot<NSP>& sp,
                                               const BRow<NSP>& rw, double hown, int i, bool valid, double* wsm) {
  using namespace bdf2;
  constexpr int V = 3 + NSP;
  const int lane = threadIdx.x & 31, cell = lane >> 3, r = lane & 7, base = cell * 8;
  const int q = r & 3;
  // PART 0: lanes 0-3 keep flux rows 1-3 of their slot, lanes 4-7 rows 4..
  // (energy, species); PART 1 / 2: all lanes the one half, lanes 0-3 store it
  const bool lo = PART == 0 ? r < 4 : PART == 1;
  const int NE = d.NE;
  double c[V];
  bslot_terms<NSP, L2>(d, th, sp, lo, c);
  double* w = wsm + (cell < CPW ? cell : 0) * V * 4;  // [row][slot]
  if (cell < CPW && (PART == 0 || r < 4)) bslot_put<NSP>(w, lo, q, c);
  __syncwarp();
  if (PART == 2) {
    bar_arrive(6, 64);
    return;
  }
  if (PART == 1) bar_named(6, 64);
  double dflux = 0.0;
  if (r < V) {
#pragma unroll
    for (int sl = 0; sl < 4; ++sl) dflux = dflux + w[r * 4 + sl];
  }
  // --- the cell's system, one row per lane (dgesvx after the factorisation)
  const bool rowequ = rw.equ & 1, colequ = rw.equ & 2;
  double b = FWD ? hown - dflux : dflux;
  if (rowequ) b = rw.rsc * b;
  if (!(valid && r < V)) b = 0.0;
  double x = getrs_rows<V>(b, rw.src, rw.lrow, rw.ukk, rw.urh, rw.url, r, base);
  // dgerfs refinement: residual, componentwise backward error, correction.
  // The backward error is non-negative: its maximum and the loop tests
  // compare bit patterns; 2 berr <= lstres is berr <= lstres/2 (both exact).
  long long lstres_half = dbits(1.5);  // lstres = 3
  int count = 1;
  bool go = valid;
  for (int it = 0; it < 6; ++it) {
    double xs[V];
#pragma unroll
    for (int k = 0; k < V; ++k) xs[k] = __shfl_sync(FULL, x, base + k);
    double y = b;
#pragma unroll
    for (int k = 0; k < V; ++k) y = y + (-1.0 * xs[k]) * rw.arow[k];
    double wk = fabs(b);
#pragma unroll
    for (int k = 0; k < V; ++k) wk = wk + fabs(rw.arow[k]) * fabs(xs[k]);
    const long long vb = berr_bits<V>(y, wk, r);
    const bool cont = go && vb > dbits(EPS) && vb <= lstres_half && count <= 5;
    if (!__any_sync(FULL, cont)) break;
    const double corr = getrs_rows<V>(y, rw.src, rw.lrow, rw.ukk, rw.urh, rw.url, r, base);
    if (cont) {
      x = x + corr;
      lstres_half = vb - (1LL << 52);  // berr / 2: berr > eps is a normal number
      count = count + 1;
    }
    go = cont;
  }
  if (colequ) x = rw.csc * x;
  if (valid && r < V) d.hWA[r * NE + i] = FWD ? x : hown - x;
}

// One level of the forward (FWD) or backward sweep, cells t0..t1-1 of the
// level order; eight lanes per cell, CPW cells per warp (one warp per block;
// lanes of cell slots >= CPW only join the shuffles).
template <int NSP, bool FWD, int CPW>
__global__ void __launch_bounds__(32) k_bdf2_sweep(const Dev d, const ThermoDev<NSP> th, int t0, int t1) {
  using namespace bdf2;
  constexpr int V = 3 + NSP, DIR = FWD ? 0 : 1;
  static_assert(V <= 7, "one lane per row and the flags in slot 7");
  pdl_launch_dependents();
  const int lane = threadIdx.x & 31, cell = lane >> 3, r = lane & 7;
  const int q = r & 3;
  const int NE = d.NE;
  const int t = t0 + blockIdx.x * CPW + cell;
  const bool valid = cell < CPW && t < t1;
  const int i = valid ? d.swi[DIR][t] : 0;
  const BSlot<NSP> sp = bslot_load<NSP, FWD>(d, t, valid, q);
  const BRow<NSP> rw = brow_load<NSP>(d, i, valid, r);
  double hown = 0.0;
  if (FWD && valid && r < V) hown = d.hWA[r * NE + i];  // written by k_bdf2_prep, complete before this grid
  pdl_wait();
  if (!FWD && valid && r < V) hown = d.hWA[r * NE + i];
  __shared__ double wsm[CPW * V * 4];
  bdf2_cell_step<NSP, FWD, CPW, false>(d, th, sp, rw, hown, i, valid, wsm);
}

// Both BDF2 sweeps as one cooperative dataflow launch on the pass tables of
// k_lusgs_flow (FlowDev with passes of up to 8 consecutive positions of one
// level owned by one block; one block per SM).  A cell's step is long (two
// 7 x 7 solves and up to five refinement passes, about 12 us of dependent
// FP64) and uneven: with one launch per level every level lasts as long as
// its slowest cell, here a slow cell holds up only the passes that read it.
// Warps 0 and 1 take four cells of each pass each.  Warps 3 and 4 stage one
// pass ahead what the sweep does not change (the slot data, the cell's
// factorised rows, its index and, forward, its right-hand side) in a double
// buffer of shared memory, for warp 0 and warp 1 respectively, and arrive on
// barrier 5.  Warp 2 looks at the flags of the next pass; once the current
// pass is done (barrier 4) and the next one is staged (barrier 5) it hands
// the next one over (barrier 3, which the staging warps also wait on before
// they refill the other buffer), and it publishes the finished pass (flag =
// this launch's epoch) before any blocking wait.  s_go[k % 2] = 0 after a
// bounded wait gave up (ERR_SYNC): the compute warps then skip the pass.  The
// last block to finish advances the epoch counter; the primitive update
// follows as its own launch.
template <int NSP>
struct BStage {
  BSlot<NSP> sp;
  BRow<NSP> rw;
  double hown;
  int i, valid;
};
// A pass of at most four cells runs on both compute warps split by rows
// (bdf2_cell_step PART 1 and 2), otherwise four cells on each (PART 0).
constexpr int BFLOW_THREADS = 160, BFLOW_NB = 96;  // all five warps; a role pair and the coordinator
template <int NSP>
constexpr int bflow_smem() { return (int)(2 * 2 * 32 * sizeof(BStage<NSP>)); }
template <int NSP>
__global__ void __launch_bounds__(BFLOW_THREADS, 1) k_bdf2_flow(const Dev d, const ThermoDev<NSP> th, const FlowDev f) {
  using namespace bdf2;
  constexpr int V = 3 + NSP;
  static_assert(V <= 7, "one lane per row and the flags in slot 7");
  extern __shared__ __align__(16) uint8_t bflow_smem_raw[];
  BStage<NSP>* s_st = reinterpret_cast<BStage<NSP>*>(bflow_smem_raw);  // [buffer][warp][lane]
  __shared__ double wsm[2][4 * V * 4];
  __shared__ unsigned s_epoch;
  __shared__ volatile int s_bad, s_go[2], s_split[2];
  if (threadIdx.x == 0) {
    s_epoch = ld_acquire(f.ctr) + 1u;
    s_bad = 0;
    s_go[0] = 0;
    s_go[1] = 0;
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  const int b = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int f0 = f.boff[0][b], b0 = f.boff[1][b];
  const int nf = f.boff[0][b + 1] - f0, n = nf + (f.boff[1][b + 1] - b0);
  auto pass_of = [&](int k) { return k < nf ? f.blist[0][f0 + k] : f.blist[1][b0 + k - nf]; };
  const int cell = lane >> 3, r = lane & 7, q = r & 3;
  if (warp == 2) {
    auto poll = [&](int k) {
      if (s_bad) return;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && wait_flag(f.pflag + f.deps[d0 + u], epoch, d.err, d.spin_limit);
      if (__any_sync(FULL, !ok) && lane == 0) s_bad = 1;
      __syncwarp();
    };
    auto ready = [&](int k) -> bool {
      if (s_bad) return true;
      const int pz = pass_of(k), d0 = f.doff[pz], nd = f.doff[pz + 1] - d0;
      bool ok = true;
      for (int u = lane; u < nd; u += 32) ok = ok && ld_acquire(f.pflag + f.deps[d0 + u]) >= epoch;
      return __all_sync(FULL, ok) != 0;
    };
    // pass k is staged (barrier 5), then handed over (barrier 3)
    auto hand_over = [&](int k) {
      bar_named(5, BFLOW_NB);
      if (lane == 0) s_go[k & 1] = s_bad ? 0 : 1;
      __syncwarp();
      __threadfence_block();
      bar_arrive(3, BFLOW_THREADS);
    };
    if (n > 0) {
      poll(0);
      hand_over(0);
    }
    for (int k = 0; k < n; ++k) {
      const bool more = k + 1 < n;
      const bool go = more && ready(k + 1);
      bar_named(4, BFLOW_NB);
      if (go) hand_over(k + 1);
      if (lane == 0 && !s_bad) st_release(f.pflag + pass_of(k), epoch);
      if (more && !go) {
        poll(k + 1);
        hand_over(k + 1);
      }
    }
  } else if (warp >= 3) {
    const int w = warp - 3;  // stages for compute warp w
    auto stage = [&](int k) {
      const bool fwd = k < nf;
      const int pz = pass_of(k), t0 = f.pstart[pz], t1 = t0 + f.pcount[pz];
      const bool split = t1 - t0 <= 4;  // both compute warps on cells t0 .. t0 + 3
      const int t = t0 + (split ? 0 : 4 * w) + cell;
      const bool valid = t < t1;
      if (w == 0 && lane == 0) s_split[k & 1] = split ? 1 : 0;
      const int i = valid ? d.swi[fwd ? 0 : 1][t] : 0;
      BStage<NSP>& e = s_st[((k & 1) * 2 + w) * 32 + lane];
      e.sp = fwd ? bslot_load<NSP, true>(d, t, valid, q) : bslot_load<NSP, false>(d, t, valid, q);
      e.rw = brow_load<NSP>(d, i, valid, r);
      // forward: the set-up's right-hand side, which only this cell's own
      // forward step changes
      e.hown = fwd && valid && r < V ? __ldcg(d.hWA + r * d.NE + i) : 0.0;
      e.i = i;
      e.valid = valid ? 1 : 0;
      __syncwarp();
      __threadfence_block();
      bar_arrive(5, BFLOW_NB);
    };
    if (n > 0) stage(0);
    for (int k = 0; k < n; ++k) {
      bar_named(3, BFLOW_THREADS);  // pass k handed over: the other buffer is free
      if (k + 1 < n) stage(k + 1);
    }
  } else {
    for (int k = 0; k < n; ++k) {
      const bool fwd = k < nf;
      bar_named(3, BFLOW_THREADS);
      const BStage<NSP>& e = s_st[((k & 1) * 2 + warp) * 32 + lane];
      const BSlot<NSP> sp = e.sp;
      const BRow<NSP> rw = e.rw;
      const int i = e.i;
      const bool valid = e.valid != 0;
      // backward: the cell's own increment, as this block's forward pass of
      // the cell wrote it (read after the hand-over: the other warp may have
      // been finishing the forward pass that holds the same cell)
      const double hown = fwd ? e.hown : valid && r < V ? __ldcg(d.hWA + r * d.NE + i) : 0.0;
      if (s_go[k & 1]) {
        if (s_split[k & 1]) {
          if (warp == 0) {
            if (fwd) bdf2_cell_step<NSP, true, 4, true, 1>(d, th, sp, rw, hown, i, valid, wsm[0]);
            else bdf2_cell_step<NSP, false, 4, true, 1>(d, th, sp, rw, hown, i, valid, wsm[0]);
          } else {
            if (fwd) bdf2_cell_step<NSP, true, 4, true, 2>(d, th, sp, rw, hown, i, valid, wsm[0]);
            else bdf2_cell_step<NSP, false, 4, true, 2>(d, th, sp, rw, hown, i, valid, wsm[0]);
          }
        } else {
          if (fwd) bdf2_cell_step<NSP, true, 4, true>(d, th, sp, rw, hown, i, valid, wsm[warp]);
          else bdf2_cell_step<NSP, false, 4, true>(d, th, sp, rw, hown, i, valid, wsm[warp]);
        }
      }
      __syncwarp();
      bar_arrive(4, BFLOW_NB);
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

// PA += dP, then primitve_to_conserved_variables (update_flow_variables.f90:50-84)
template <int NSP>
__global__ void __launch_bounds__(128) k_bdf2_update(const Dev d, const ThermoDev<NSP> th) {
  constexpr int V = 3 + NSP;
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NE) return;
  const int NE = d.NE;
  unsigned err = 0;
  double P[V];
#pragma unroll
  for (int k = 0; k < V; ++k) {
    P[k] = d.PA[k * NE + i] + d.hWA[k * NE + i];
    d.PA[k * NE + i] = P[k];
  }
  double yy[NSP], entha[NSP], Cp, gama, Rcpcv, s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { yy[k] = P[4 + k]; s = s + yy[k]; }
  yy[NSP - 1] = 1.0 - s;
  const double pp = P[0], uu = P[1], vv = P[2], tt = P[3];
  gas<NSP>(th, yy, tt, Cp, gama, Rcpcv, err);
  const double rr = pp / (Rcpcv * tt);
  enthalpy<NSP>(th, tt, entha, err);
  double hh = 0.0;
#pragma unroll
  for (int k = 0; k < NSP; ++k) hh = hh + yy[k] * entha[k];
  d.WA[0 * NE + i] = rr;
  d.WA[1 * NE + i] = rr * uu;
  d.WA[2 * NE + i] = rr * vv;
  d.WA[3 * NE + i] = rr * (hh + 0.5 * (uu * uu + vv * vv)) - pp;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) d.WA[(4 + k) * NE + i] = rr * yy[k];
  if (i == 0 && isnan(rr)) err |= ERR_NAN;
  flag(d, err);
}

inline unsigned nblk(long n, int t) { return (unsigned)((n + t - 1) / t); }

template <int NSP>
void bdf2_fixed(const Dev& d, int bs, int euler, cudaStream_t s) {
  k_bdf2_fixed<NSP><<<nblk(d.NE, bs), bs, 0, s>>>(d, euler);
}
template <int NSP>
void bdf2_prep(const Dev& d, const void* th, int bs, cudaStream_t s) {
  k_bdf2_prep<NSP><<<nblk(d.NE, bs), bs, 0, s>>>(d, *static_cast<const ThermoDev<NSP>*>(th));
}
template <int NSP, int CPW>
void bdf2_sweep_cpw(const Dev& d, const ThermoDev<NSP>& T, bool fwd, int t0, int t1, cudaStream_t s) {
  if (fwd) launch_pdl(k_bdf2_sweep<NSP, true, CPW>, nblk(t1 - t0, CPW), 32, s, d, T, t0, t1);
  else launch_pdl(k_bdf2_sweep<NSP, false, CPW>, nblk(t1 - t0, CPW), 32, s, d, T, t0, t1);
}
template <int NSP>
void bdf2_sweep(const Dev& d, const void* th, bool fwd, int t0, int t1, int cpw, cudaStream_t s) {
  const auto& T = *static_cast<const ThermoDev<NSP>*>(th);
  if (cpw >= 4) bdf2_sweep_cpw<NSP, 4>(d, T, fwd, t0, t1, s);
  else if (cpw == 2) bdf2_sweep_cpw<NSP, 2>(d, T, fwd, t0, t1, s);
  else bdf2_sweep_cpw<NSP, 1>(d, T, fwd, t0, t1, s);
}
// the cooperative dataflow launch of both sweeps (grid: one block per SM)
template <int NSP>
cudaError_t bdf2_flow(const Dev& d, const void* th, const FlowDev& f, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(BFLOW_THREADS);
  cfg.dynamicSmemBytes = (size_t)bflow_smem<NSP>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_bdf2_flow<NSP>, d, *static_cast<const ThermoDev<NSP>*>(th), f);
}
template <int NSP>
int bdf2_flow_occupancy() {
  int nb = 0;
  if (cudaFuncSetAttribute(k_bdf2_flow<NSP>, cudaFuncAttributeMaxDynamicSharedMemorySize, bflow_smem<NSP>()) !=
      cudaSuccess)
    return 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bdf2_flow<NSP>, BFLOW_THREADS, bflow_smem<NSP>());
  return nb;
}
template <int NSP>
void bdf2_update(const Dev& d, const void* th, int bs, cudaStream_t s) {
  launch_pdl(k_bdf2_update<NSP>, nblk(d.NE, bs), bs, s, d, *static_cast<const ThermoDev<NSP>*>(th));
}
template <int NSP>
int bdf2_nbq() { return bdf2::nbq<NSP>(); }

#define RC_BDF2_INST(N)                                                             \
  template void bdf2_fixed<N>(const Dev&, int, int, cudaStream_t);                  \
  template void bdf2_prep<N>(const Dev&, const void*, int, cudaStream_t);           \
  template void bdf2_sweep<N>(const Dev&, const void*, bool, int, int, int, cudaStream_t); \
  template void bdf2_update<N>(const Dev&, const void*, int, cudaStream_t);         \
  template cudaError_t bdf2_flow<N>(const Dev&, const void*, const FlowDev&, int, cudaStream_t); \
  template int bdf2_flow_occupancy<N>();                                           \
  template int bdf2_nbq<N>();
RC_BDF2_INST(1)
RC_BDF2_INST(4)

}  // namespace rc
