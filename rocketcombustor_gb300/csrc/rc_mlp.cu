// The learned chemistry surrogate (new; the reference has no counterpart).
//
// Network: 7 raw inputs (T, p, Y_1..Y_4, dt) -> features (1000/T, log10 p,
// log10(Y + 1e-10), log10 dt) normalised -> layer 0 (7 -> 128, GELU) -> three 128 -> 128 GELU layers -> 4
// outputs.  GELU is the tanh form of Hendrycks & Gimpel on the hardware tanh.
// Training keeps FP32 master weights and BF16 operands: the three 128 x 128
// layers on the tcgen05 tensor cores (operands staged in shared memory with
// the 128-byte swizzle, FP32 accumulators in TMEM), layer 0 and the output
// layer on the CUDA cores in FP32.  Inference runs all five layers on tcgen05
// with F16 operands.
//
// Kernels:
//   k_mlp_fwd16<Io>   inference, persistent over tiles of 128 samples: all
//                     weights stay in shared memory, activations never leave
//                     the SM (inputs and outputs through Io);
//   k_gemm<EPI, BN>   training GEMMs, one 128 x BN output tile per CTA, K in
//                     chunks of 128, optional split-K: forward layers (bias +
//                     GELU epilogue), backward data (x GELU' epilogue) and
//                     weight gradients (FP32 partials);
//   k_layer0, k_head, k_small_part, k_reduce_grads, k_adam, k_pack, k_pack16: the thin
//                     layers, the loss, the small reductions, Adam and the
//                     BF16 / F16 weight copies.
// Every reduction has a fixed order, so gradients are reproducible run to run.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "rc_dev.cuh"
#include "rc_gpu.h"
#include "rc_mlp.h"
#include "rc_umma.cuh"

namespace rc {
namespace mlp {

constexpr int H = 128, NIN = 7, NOUT = 4;
constexpr int OFF_W0 = 0, OFF_B0 = H * NIN;
__host__ __device__ constexpr int off_w(int l) { return H * NIN + H + (l - 1) * (H * H + H); }  // l = 1..3
__host__ __device__ constexpr int off_b(int l) { return off_w(l) + H * H; }
constexpr int OFF_W4 = off_w(4), OFF_B4 = OFF_W4 + NOUT * H, NPARAM = OFF_B4 + NOUT;
static_assert(NPARAM == RC_MLP_NPARAM, "parameter layout");
constexpr int TILE_BYTES = 128 * 128 * 2;

struct Norm {
  float mean[NIN], stdv[NIN];
  float dom[6];  // T_lo, T_hi, p_lo, p_hi, dt_lo, dt_hi
};

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float GK0 = 0.7978845608f, GK1 = 0.044715f;  // sqrt(2/pi), cubic coefficient
__device__ __forceinline__ float gelu(float h) {
  const float t = tanh_fast(GK0 * (h + GK1 * h * h * h));
  return 0.5f * h * (1.f + t);
}
__device__ __forceinline__ float gelu_d(float h) {
  const float t = tanh_fast(GK0 * (h + GK1 * h * h * h));
  return 0.5f * (1.f + t) + 0.5f * h * (1.f - t * t) * GK0 * (1.f + 3.f * GK1 * h * h);
}
__device__ __forceinline__ uint32_t bf2(float a, float b) {
  __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&p);
}
__device__ __forceinline__ uint4 pack8(const float* v) {
  return make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
}
// raw (T, p, Y1..Y4, dt) -> normalised features (1000/T, log10 p,
// log10(Y_k + 1e-10), log10 dt): in these the log of the Damkoehler number of
// the global reaction is linear, so the mean-rate ratio is a smooth function
// of one linear combination of the features.
constexpr float YFLOOR = 1e-10f;
__device__ __forceinline__ void features(const float* raw, const Norm& nr, float* xn) {
#pragma unroll
  for (int i = 0; i < NIN; ++i) {
    float f;
    if (i == 0) f = 1000.f / fmaxf(raw[0], 1.f);
    else if (i == 1 || i == 6) f = log10f(fmaxf(raw[i], 1e-30f));
    else f = log10f(fmaxf(raw[i], 0.f) + YFLOOR);
    xn[i] = (f - nr.mean[i]) / nr.stdv[i];
  }
}

// FG warp groups of 4 warps per CTA in the fused forward (k_mlp_fwd16), each
// with its own activation tile, TMEM accumulator (128 columns) and mbarrier.
constexpr int FG = 3;
constexpr uint32_t FUSED_TMEM_COLS = 512;

// barrier of the 128 threads of group g (named barrier 1 + g; 0 is __syncthreads)
__device__ __forceinline__ void group_sync(int g) {
  asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory");
}

// ------------------------------------------------ fused forward, all tcgen05
// Every layer on the tensor cores with F16 operands: layer 0 as one K = 16
// step (the 7 features, a constant 1 in column 7 that takes b0 from column 7
// of the layer-0 weights, zeros), the three hidden layers as 8 K-steps, the
// output layer as N = 16 (4 outputs padded).  Layers 0-3 accumulate in F16
// in TMEM, read back two columns per register (tcgen05.ld .pack::16b), so
// the epilogue needs no conversion; the output layer accumulates in FP32.
// F16 keeps 11 significant bits where BF16 keeps 8, so the activations are
// closer to FP32 than the training forward's BF16 ones.  The epilogue loads
// the whole 128-column row of its accumulator (four tcgen05.ld, one wait),
// then forms 2 GELU(h) = h (1 + tanh(h (k0 + k0 k1 h^2))), h = acc + bias, in
// six packed-half operations per pair, the hardware tanh on f16x2; the F16
// weights of layers 1-4 carry the factor 1/2 (halving an F16 is exact above
// the subnormal range, |w| >= 2^-13), so the products are those of GELU(h)
// with the trained weights.  The weights come pre-scaled and pre-swizzled in
// F16 (k_pack16), in the shared-memory order of the kernel: hidden tiles
// 1..3, the layer-0 tile (128 rows, K columns 0-15 used), the output tile (16
// rows); the CTA copies them once.  FG groups of four warps, each with its
// activation tile, 128 TMEM columns and mbarrier, work on different tiles of
// 128 samples, so one group's epilogue overlaps another's MMAs (a tile's
// layers depend on one another, so the overlap is between tiles).  Issuing a
// layer's K-steps as the previous epilogue writes each 32 columns, with a
// group barrier per 32 columns, measured slower (5.0e9 against 5.4e9 samples/s
// on 4M samples), and so did two groups with two accumulators each (4.0e9).
constexpr int W0_TILE_BYTES = 128 * 128, W4_TILE_BYTES = 16 * 128 * 2;
constexpr int WH_BYTES = 3 * TILE_BYTES + W0_TILE_BYTES + W4_TILE_BYTES;  // 118784
constexpr int F2_W0 = 3 * TILE_BYTES, F2_W4 = F2_W0 + W0_TILE_BYTES, F2_ACT = F2_W4 + W4_TILE_BYTES;
constexpr int F2_BIAS = F2_ACT + FG * TILE_BYTES;  // b1..b3 as f16x2 pairs (3 x 64), then b4 (16 floats)
constexpr int F2_BAR = F2_BIAS + (3 * H / 2 + 16) * 4;
constexpr int F2_SLOT = F2_BAR + 8 * FG, F2_OK = F2_SLOT + 4;
constexpr int F2_SMEM = F2_OK + 4 * FG + 1024;
// layers 0-3 accumulate in F16, the output layer in FP32
constexpr uint32_t IDESC_H = umma::idesc_f16_acc16(128, 128), IDESC_H16 = umma::idesc_f16(128, 16);
static_assert(F2_ACT % 1024 == 0 && F2_W0 % 1024 == 0 && F2_W4 % 1024 == 0, "tile alignment");
static_assert(F2_BAR % 8 == 0, "mbarrier alignment");
static_assert(F2_SMEM <= 227 * 1024, "shared memory");

__device__ __forceinline__ uint32_t h2_bits(float v) {
  const __half2 h = __float2half2_rn(v);
  return *reinterpret_cast<const uint32_t*>(&h);
}
// pack (a, b) to f16x2, a in the low half
__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
  uint32_t x;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(x) : "f"(b), "f"(a));
  return x;
}
// twice the GELU (tanh form) of a packed pair of pre-activations acc + bias:
// h (1 + tanh(h (k0 + k0 k1 h^2)))
__device__ __forceinline__ uint32_t gelu2_h2(uint32_t acc, uint32_t bias) {
  const uint32_t c0 = h2_bits(GK0), c1 = h2_bits(GK0 * GK1);
  uint32_t h, h2, p, u, t, g;
  asm("add.rn.f16x2 %0, %1, %2;" : "=r"(h) : "r"(acc), "r"(bias));
  asm("mul.rn.f16x2 %0, %1, %1;" : "=r"(h2) : "r"(h));
  asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(p) : "r"(h2), "r"(c1), "r"(c0));
  asm("mul.rn.f16x2 %0, %1, %2;" : "=r"(u) : "r"(h), "r"(p));
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(u));
  asm("fma.rn.f16x2 %0, %1, %2, %2;" : "=r"(g) : "r"(t), "r"(h));
  return g;
}
// the same without a bias (layer 0 has it in the accumulator)
__device__ __forceinline__ uint32_t gelu2_h2(uint32_t h) {
  const uint32_t c0 = h2_bits(GK0), c1 = h2_bits(GK0 * GK1);
  uint32_t h2, p, u, t, g;
  asm("mul.rn.f16x2 %0, %1, %1;" : "=r"(h2) : "r"(h));
  asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(p) : "r"(h2), "r"(c1), "r"(c0));
  asm("mul.rn.f16x2 %0, %1, %2;" : "=r"(u) : "r"(h), "r"(p));
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(u));
  asm("fma.rn.f16x2 %0, %1, %2, %2;" : "=r"(g) : "r"(t), "r"(h));
  return g;
}

template <class Io>
__global__ void __launch_bounds__(128 * FG, 1) k_mlp_fwd16(const uint4* __restrict__ Wh, const float* __restrict__ params,
                                                           Norm nr, Io io, int n, unsigned* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = smem_raw + ((1024u - (umma::smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = umma::smem_u32(base);
  uint32_t* bias2 = reinterpret_cast<uint32_t*>(base + F2_BIAS);  // [3][64] f16x2, layers 1..3
  float* bias4 = reinterpret_cast<float*>(base + F2_BIAS) + 3 * H / 2;
  uint32_t* slot = reinterpret_cast<uint32_t*>(base + F2_SLOT);
  const int g = threadIdx.x >> 7, t = threadIdx.x & 127, warp = t >> 5;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + F2_BAR) + g;
  int* s_ok = reinterpret_cast<int*>(base + F2_OK) + g;
  for (int q = threadIdx.x; q < WH_BYTES / 16; q += 128 * FG) reinterpret_cast<uint4*>(base)[q] = Wh[q];
  for (int q = threadIdx.x; q < H / 2; q += 128 * FG)
    for (int l = 1; l <= 3; ++l) bias2[(l - 1) * H / 2 + q] = pack_h2(params[off_b(l) + 2 * q], params[off_b(l) + 2 * q + 1]);
  if (threadIdx.x < 16) bias4[threadIdx.x] = threadIdx.x < NOUT ? params[OFF_B4 + threadIdx.x] : 0.f;
  if (t == 0) umma::mbar_init(bar, 1);
  if (threadIdx.x < 32) {
    umma::tmem_alloc(slot, FUSED_TMEM_COLS);
    umma::tmem_relinquish();
  }
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = *slot, tmem_g = tmem + (uint32_t)(g * 128);
  const uint32_t act = sbase + F2_ACT + g * TILE_BYTES;
  uint8_t* actp = base + F2_ACT + g * TILE_BYTES;
  const uint32_t trow = tmem_g + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true;
  // issue nk K-steps of A (this group's tile) x B (tile at bsh, rb rows) into
  // the group's accumulator and wait for them (bounded)
  auto mma = [&](int nk, uint32_t bsh, int rb, uint32_t idesc) {
    umma::fence_async_smem();
    umma::tc_fence_before();
    group_sync(g);
    if (t == 0) {
      umma::tc_fence_after();
      for (int kk = 0; kk < nk; ++kk)
        umma::mma_bf16(tmem_g, umma::sdesc_k(act, 128, kk), umma::sdesc_k(bsh, rb, kk), idesc, kk > 0 ? 1u : 0u);
      umma::mma_commit(bar);
      *s_ok = umma::mbar_wait(bar, phase) ? 1 : 0;
    }
    group_sync(g);
    phase ^= 1u;
    umma::tc_fence_after();
    return *s_ok != 0;
  };
  // (bias +) 2 GELU of the accumulator row t -> row t of the activation tile
  auto epilogue = [&](const uint32_t* bl) {
    uint32_t v[64];
#pragma unroll
    for (int c = 0; c < 4; ++c) umma::tmem_ld32_pack16_nowait(trow + (uint32_t)(c * 32), v + 16 * c);
    umma::tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      uint32_t h[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) h[e] = bl ? gelu2_h2(v[4 * c + e], bl[4 * c + e]) : gelu2_h2(v[4 * c + e]);
      *reinterpret_cast<uint4*>(actp + umma::sw128_offset(t, c * 8, 128)) = make_uint4(h[0], h[1], h[2], h[3]);
    }
  };
  const int ntiles = (n + 127) / 128;
  for (int tile = blockIdx.x * FG + g; tile < ntiles && ok; tile += gridDim.x * FG) {
    const int s = tile * 128 + t;
    float xn[NIN];
    typename Io::Local loc;
    io.load(s, s < n, nr, xn, loc);
    // the features as K columns 0-6 of row t, 1 in column 7 (the bias), zeros to 15
    *reinterpret_cast<uint4*>(actp + umma::sw128_offset(t, 0, 128)) =
        make_uint4(pack_h2(xn[0], xn[1]), pack_h2(xn[2], xn[3]), pack_h2(xn[4], xn[5]), pack_h2(xn[6], 1.f));
    *reinterpret_cast<uint4*>(actp + umma::sw128_offset(t, 8, 128)) = make_uint4(0u, 0u, 0u, 0u);
    if (!(ok = mma(1, sbase + F2_W0, 128, IDESC_H))) break;
    epilogue(nullptr);
    for (int l = 1; l <= 3 && ok; ++l) {
      if (!(ok = mma(8, sbase + (l - 1) * TILE_BYTES, 128, IDESC_H))) break;
      epilogue(bias2 + (l - 1) * H / 2);
    }
    if (!ok || !(ok = mma(8, sbase + F2_W4, 16, IDESC_H16))) break;
    float v[32], out[NOUT];
    umma::tmem_ld32(trow, v);
#pragma unroll
    for (int m = 0; m < NOUT; ++m) out[m] = v[m] + bias4[m];
    io.store(s, s < n, out, loc);
  }
  if (!ok && t == 0) atomicOr(err, ERR_SYNC);
  umma::tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    umma::tc_fence_after();
    umma::tmem_dealloc(tmem, FUSED_TMEM_COLS);
  }
}

// raw features in, outputs out (row-major n x 7 / n x 4)
struct IoRaw {
  const float* x;
  float* y;
  struct Local {};
  __device__ void load(int s, bool valid, const Norm& nr, float* xn, Local&) const {
    float raw[NIN];
#pragma unroll
    for (int i = 0; i < NIN; ++i) raw[i] = valid ? x[(size_t)s * NIN + i] : nr.mean[i];
    if (!valid) { raw[1] = 1.f; raw[6] = 1.f; }
    features(raw, nr, xn);
  }
  __device__ void store(int s, bool valid, const float* out, const Local&) const {
    if (valid)
#pragma unroll
      for (int m = 0; m < NOUT; ++m) y[(size_t)s * NOUT + m] = out[m];
  }
};

// Progress scale of the one global reaction over dt: omega_k = c_k kf with
// c_k = 1000 M_k (nu''_k - nu'_k) (production, chemical_kinetics.f90:109-165),
// so dY_k = c_k xi for a progress xi.  The scale is the smaller of the
// explicit progress dt kf / rho and the progress that exhausts the limiting
// reactant, min_k(Y_k / -c_k) over c_k < 0; 0 when nothing reacts.  The
// network's outputs are z_k = dY_k / (c_k xi_s): near 1 while the explicit
// rate holds, the consumed fraction of the limiting reactant once it runs
// out, so both ends stay O(1) and bounded.
__device__ __forceinline__ double progress_scale(const ThermoDev<4>& th, const double* Y, const double* om,
                                                 double dt, double rho) {
  double kf = 0.0, xmax = 1e300;
  bool react = false;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (th.prodc[k] < 0.0) {
      react = true;
      kf = om[k] / th.prodc[k];
      xmax = fmin(xmax, fmax(Y[k], 0.0) / -th.prodc[k]);
    }
  if (!react) return 0.0;
  return fmin(dt * kf / rho, xmax);
}

// The surrogate source of the steady iteration: cell s of the solver.  The
// explicit rate and rho come from the FP64 state (sourceterm.f90:2-70); the
// network gives z_k, dY_k = z_k c_k xi_s (progress_scale) and
// src_k = vol * rho * dY_k / step.  A cell is handed to the FP64 integrator
// instead (appended to `list`) when its state lies outside the training
// domain, when the z_k of the reacting species disagree by more than
// spread_tol (one global reaction: they are equal for the exact integrator),
// when their mean is outside [-0.01, 3], or when Y + dY leaves [0, 1] by more
// than 1e-6.  Once the decisions are frozen (rc_surrogate_freeze: one call
// records them, later calls reuse them) a cell keeps its side, the network
// unless its source is not finite, so that the source is a smooth function of
// the state and a steady iteration can converge.
struct IoSolver {
  Dev d;
  ThermoDev<4> th;
  float spread_tol;
  int* list;
  unsigned* nlist;
  unsigned* nsurr;
  const int* mode;     // 0 decide per call, 1 decide and record in dec, 2 use dec
  unsigned char* dec;  // per cell: 1 = integrator
  struct Local {
    double Y[4], dt, rho, vol, xs;
    bool dom;
  };
  __device__ void load(int i, bool valid, const Norm& nr, float* xn, Local& L) const {
    const int NE = d.NE;
    float raw[NIN];
    if (!valid) {
      for (int k = 0; k < NIN; ++k) raw[k] = nr.mean[k];
      raw[1] = 1.f; raw[6] = 1.f;
      features(raw, nr, xn);
      L.dom = false;
      return;
    }
    unsigned e = 0;
    const double p = d.PA[i], T = d.PA[3 * NE + i];
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) { L.Y[k] = d.PA[(4 + k) * NE + i]; s = s + L.Y[k]; }
    L.Y[3] = 1.0 - s;
    double Cp, gama, R, om[4];
    gas<4>(th, L.Y, T, Cp, gama, R, e);
    L.rho = p / (T * R);
    production<4>(th, T, L.rho, L.Y, om);
    L.dt = d.step[i];
    L.xs = progress_scale(th, L.Y, om, L.dt, L.rho);
    L.vol = d.vol[i];
    L.dom = e == 0 && T >= nr.dom[0] && T <= nr.dom[1] && p >= nr.dom[2] && p <= nr.dom[3] && L.dt >= nr.dom[4] &&
            L.dt <= nr.dom[5];
    raw[0] = (float)T; raw[1] = (float)p;
#pragma unroll
    for (int k = 0; k < 4; ++k) raw[2 + k] = (float)L.Y[k];
    raw[6] = (float)L.dt;
    features(raw, nr, xn);
  }
  __device__ void store(int i, bool valid, const float* r, const Local& L) const {
    if (!valid) return;
    const int NE = d.NE;
    if (!(L.xs != 0.0)) {  // nothing reacts (or a reactant is exhausted)
#pragma unroll
      for (int k = 0; k < 3; ++k) d.src[k * NE + i] = 0.0;
      atomicAdd(nsurr, 1u);
      return;
    }
    const float rbar = (r[0] + r[1] + r[2]) * (1.f / 3.f);
    float spread = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) spread = fmaxf(spread, fabsf(r[k] - rbar));
    bool fall = !L.dom || !(spread <= spread_tol) || !(rbar >= -0.01f && rbar <= 3.f);
    double src[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double dY = (double)r[k] * th.prodc[k] * L.xs;
      const double Yn = L.Y[k] + dY;
      fall = fall || !(Yn >= -1e-6 && Yn <= 1.0 + 1e-6);
      src[k] = L.vol * (L.rho * (dY / L.dt));
    }
    const int md = *mode;
    if (md == 2) {
      fall = dec[i] != 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) fall = fall || !isfinite(src[k]);
    } else if (md == 1) {
      dec[i] = fall ? 1 : 0;
    }
    if (fall) {
      const unsigned slot = atomicAdd(nlist, 1u);
      list[slot] = i;
      return;
    }
    atomicAdd(nsurr, 1u);
#pragma unroll
    for (int k = 0; k < 3; ++k) d.src[k * NE + i] = src[k];
  }
};

// -------------------------------------------------------- training kernels --
struct GemmArgs {
  const __nv_bfloat16* A; int lda;   // M x K, K contiguous
  const __nv_bfloat16* B; int ldb;   // N x K, K contiguous
  int M, N, K;                       // multiples of 128; K split evenly over gridDim.z
  const float* bias;                 // EPI_FWD [N]
  const float* Hin;                  // EPI_BWD pre-activation [M][N]
  float* Hout;                       // EPI_FWD pre-activation [M][N]
  __nv_bfloat16* Orow;               // [M][N]
  __nv_bfloat16* Ocol;               // [N][M]
  float* C;                          // EPI_F32 [gridDim.z][M][N]
  unsigned* err;
};
enum { EPI_FWD = 0, EPI_BWD = 1, EPI_F32 = 2 };
constexpr int GS_BAR = 2 * TILE_BYTES, GS_SLOT = GS_BAR + 8, GS_OK = GS_SLOT + 4, GEMM_SMEM = GS_OK + 4 + 1024;

// 16-byte copy global -> shared (cp.async, L2 only); cp_async_wait_all: this
// thread's copies are complete
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// BN: output columns per CTA (128 or 64; the B tile holds BN rows); grid
// (N / BN, M / 128, split-K)
template <int EPI, int BN>
__global__ void __launch_bounds__(128) k_gemm(GemmArgs g) {
  static_assert(BN == 128 || BN == 64, "the tile widths of the epilogue and the TMEM allocation");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = smem_raw + ((1024u - (umma::smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sA = umma::smem_u32(base), sB = sA + TILE_BYTES;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + GS_BAR);
  uint32_t* slot = reinterpret_cast<uint32_t*>(base + GS_SLOT);
  int* s_ok = reinterpret_cast<int*>(base + GS_OK);
  const int t = threadIdx.x, warp = t >> 5;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * BN;
  const int kper = g.K / gridDim.z, kb = blockIdx.z * kper;
  if (t == 0) umma::mbar_init(bar, 1);
  if (warp == 0) {
    umma::tmem_alloc(slot, BN);
    umma::tmem_relinquish();
  }
  umma::tc_fence_before();
  __syncthreads();
  umma::tc_fence_after();
  const uint32_t tmem = *slot;
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = kb; k0 < kb + kper; k0 += 128) {
    // both 128 x 128 operand tiles as 16-byte asynchronous copies, all in
    // flight at once, into the swizzled layout
    for (int q = t; q < 2048; q += 128) {
      const int r = q >> 4, c = q & 15;
      cp_async16(sA + umma::sw128_offset(r, c * 8, 128), g.A + (size_t)(m0 + r) * g.lda + k0 + c * 8);
      if (r < BN) cp_async16(sB + umma::sw128_offset(r, c * 8, BN), g.B + (size_t)(n0 + r) * g.ldb + k0 + c * 8);
    }
    cp_async_wait_all();
    umma::fence_async_smem();
    umma::tc_fence_before();
    __syncthreads();
    if (t == 0) {
      umma::tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < 8; ++kk)
        umma::mma_bf16(tmem, umma::sdesc_k(sA, 128, kk), umma::sdesc_k(sB, BN, kk), umma::idesc_bf16(128, BN),
                       (k0 > kb || kk > 0) ? 1u : 0u);
      umma::mma_commit(bar);
      *s_ok = umma::mbar_wait(bar, phase) ? 1 : 0;
    }
    __syncthreads();
    phase ^= 1u;
    umma::tc_fence_after();
    if (!*s_ok) { ok = false; break; }
  }
  if (ok) {
    const int m = m0 + warp * 32 + (t & 31);
    for (int c = 0; c < BN / 32; ++c) {
      float v[32];
      umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
      const int nc = n0 + c * 32;
      if (EPI == EPI_F32) {
        float* dst = g.C + (size_t)blockIdx.z * g.M * g.N + (size_t)m * g.N + nc;
#pragma unroll
        for (int j = 0; j < 32; j += 4) *reinterpret_cast<float4*>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      } else {
        float o[32];
        if (EPI == EPI_FWD) {
          float4* hd = reinterpret_cast<float4*>(g.Hout + (size_t)m * g.N + nc);
          const float4* bz = reinterpret_cast<const float4*>(g.bias + nc);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float4 b4 = bz[j];
            const float4 h = make_float4(v[4 * j] + b4.x, v[4 * j + 1] + b4.y, v[4 * j + 2] + b4.z,
                                         v[4 * j + 3] + b4.w);
            hd[j] = h;
            o[4 * j] = gelu(h.x);
            o[4 * j + 1] = gelu(h.y);
            o[4 * j + 2] = gelu(h.z);
            o[4 * j + 3] = gelu(h.w);
          }
        } else {
          const float4* hs = reinterpret_cast<const float4*>(g.Hin + (size_t)m * g.N + nc);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float4 h = hs[j];
            o[4 * j] = v[4 * j] * gelu_d(h.x);
            o[4 * j + 1] = v[4 * j + 1] * gelu_d(h.y);
            o[4 * j + 2] = v[4 * j + 2] * gelu_d(h.z);
            o[4 * j + 3] = v[4 * j + 3] * gelu_d(h.w);
          }
        }
        uint4* rd = reinterpret_cast<uint4*>(g.Orow + (size_t)m * g.N + nc);
#pragma unroll
        for (int j = 0; j < 4; ++j) rd[j] = pack8(o + 8 * j);
#pragma unroll
        for (int j = 0; j < 32; ++j) g.Ocol[(size_t)(nc + j) * g.M + m] = __float2bfloat16_rn(o[j]);
      }
    }
  } else if (t == 0) {
    atomicOr(g.err, ERR_SYNC);
  }
  umma::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    umma::tc_fence_after();
    umma::tmem_dealloc(tmem, BN);
  }
}

// layer 0 for a training batch: xn (n x 7), H0 (n x 128 FP32), A0 row / column
// (BF16).  A block takes 32 samples (the lanes) and its 16 warps 8 outputs each;
// warp 0 forms the samples' features.
constexpr int L0_THREADS = 512;
__global__ void __launch_bounds__(L0_THREADS) k_layer0(const float* __restrict__ x, Norm nr,
                                                       const float* __restrict__ P, int n, float* xn, float* H0,
                                                       __nv_bfloat16* Arow, __nv_bfloat16* Acol) {
  __shared__ float sf[32][NIN + 1];
  const int lane = threadIdx.x & 31, c8 = threadIdx.x >> 5;
  const int s = blockIdx.x * 32 + lane;
  if (c8 == 0 && s < n) {
    float f[NIN];
    features(x + (size_t)s * NIN, nr, f);
#pragma unroll
    for (int i = 0; i < NIN; ++i) {
      xn[(size_t)s * NIN + i] = f[i];
      sf[lane][i] = f[i];
    }
  }
  __syncthreads();
  if (s >= n) return;
  float f[NIN];
#pragma unroll
  for (int i = 0; i < NIN; ++i) f[i] = sf[lane][i];
  float h[8], a[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int o = c8 * 8 + e;
    h[e] = P[OFF_B0 + o];
#pragma unroll
    for (int i = 0; i < NIN; ++i) h[e] = fmaf(P[OFF_W0 + o * NIN + i], f[i], h[e]);
    a[e] = gelu(h[e]);
    Acol[(size_t)o * n + s] = __float2bfloat16_rn(a[e]);
  }
  float4* hd = reinterpret_cast<float4*>(H0 + (size_t)s * H + c8 * 8);
  hd[0] = make_float4(h[0], h[1], h[2], h[3]);
  hd[1] = make_float4(h[4], h[5], h[6], h[7]);
  reinterpret_cast<uint4*>(Arow + (size_t)s * H)[c8] = pack8(a);
}

// output layer, loss and its gradient down to dH3: y = W4 gelu(H3) + b4,
// L = mean((y - t)^2) over n x 4, dy = 2 (y - t) / (4 n).  Four threads per
// sample (lane = 4 sample + quarter), each over 32 of the 128 inputs; the
// quarters' partial outputs are added by a butterfly (every thread of the
// sample gets the same sum).  loss_part: one partial per block of 32 samples.
constexpr int HEAD_THREADS = 128, HEAD_SAMPLES = HEAD_THREADS / 4;
__global__ void __launch_bounds__(HEAD_THREADS) k_head(const float* __restrict__ H3, const float* __restrict__ tgt,
                                                       const float* __restrict__ P, int n, float* dy,
                                                       __nv_bfloat16* dHrow, __nv_bfloat16* dHcol, float* loss_part) {
  __shared__ float red[HEAD_THREADS];
  const int qd = threadIdx.x & 3, s = blockIdx.x * HEAD_SAMPLES + (threadIdx.x >> 2);
  const bool valid = s < n;
  const int sc_ = valid ? s : 0;
  float h[32];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float4 v = reinterpret_cast<const float4*>(H3 + (size_t)sc_ * H + qd * 32)[j];
    h[4 * j] = v.x;
    h[4 * j + 1] = v.y;
    h[4 * j + 2] = v.z;
    h[4 * j + 3] = v.w;
  }
  float y[NOUT];
#pragma unroll
  for (int m = 0; m < NOUT; ++m) y[m] = 0.f;
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const float a = gelu(h[i]);
#pragma unroll
    for (int m = 0; m < NOUT; ++m) y[m] = fmaf(a, P[OFF_W4 + m * H + qd * 32 + i], y[m]);
  }
#pragma unroll
  for (int m = 0; m < NOUT; ++m) {
    y[m] += __shfl_xor_sync(0xffffffffu, y[m], 1);
    y[m] += __shfl_xor_sync(0xffffffffu, y[m], 2);
  }
  float l2 = 0.f;
  float g[NOUT];
  const float sc = 2.f / (4.f * (float)n);
#pragma unroll
  for (int m = 0; m < NOUT; ++m) {
    const float e = valid ? y[m] + P[OFF_B4 + m] - tgt[(size_t)s * NOUT + m] : 0.f;
    l2 = fmaf(e, e, l2);
    g[m] = sc * e;
    if (valid && qd == 0) dy[(size_t)s * NOUT + m] = g[m];
  }
  if (valid) {
#pragma unroll
    for (int c8 = 0; c8 < 4; ++c8) {
      float o[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int i = qd * 32 + c8 * 8 + e;
        float da = 0.f;
#pragma unroll
        for (int m = 0; m < NOUT; ++m) da = fmaf(P[OFF_W4 + m * H + i], g[m], da);
        o[e] = da * gelu_d(h[c8 * 8 + e]);
        dHcol[(size_t)i * n + s] = __float2bfloat16_rn(o[e]);
      }
      reinterpret_cast<uint4*>(dHrow + (size_t)s * H + qd * 32)[c8] = pack8(o);
    }
  }
  red[threadIdx.x] = qd == 0 ? l2 : 0.f;
  __syncthreads();
  for (int w = HEAD_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

// Gradients of the thin parameters (W0, b0..b3, W4, b4) in two passes of
// fixed order.  k_small_part: block c sums samples [c chunk, (c + 1) chunk),
// thread o its column: W0[o][0..6], b0..b3[o], W4[0..3][o] (SMALL_PER
// values at part[c][o SMALL_PER ..]) and, for o < 4, b4[o] (at H SMALL_PER + o).
// The samples come through shared memory in tiles of SMALL_TILE (dH0..dH3,
// H3, xn, dy rows), the next tile's asynchronous copies in flight while the
// current one is summed.  chunk: a multiple of SMALL_TILE.
constexpr int SMALL_PER = NIN + 4 + NOUT, SMALL_N = H * SMALL_PER + NOUT, SMALL_ZMAX = 512, SMALL_TILE = 16;
// one tile's buffer: dH0..dH3 (BF16), H3 (FP32), xn, dy
constexpr int ST_DH = 0, ST_H3 = ST_DH + 4 * SMALL_TILE * H * 2, ST_XN = ST_H3 + SMALL_TILE * H * 4,
              ST_DY = ST_XN + SMALL_TILE * NIN * 4, ST_BYTES = ST_DY + SMALL_TILE * NOUT * 4,
              SMALL_SMEM = 2 * ST_BYTES;
static_assert(ST_XN % 16 == 0 && ST_DY % 16 == 0 && ST_BYTES % 16 == 0 && (SMALL_TILE * NIN * 4) % 16 == 0,
              "16-byte copies");
__global__ void __launch_bounds__(H) k_small_part(const float* __restrict__ xn, const __nv_bfloat16* __restrict__ dH0,
                                                  const __nv_bfloat16* __restrict__ dH1,
                                                  const __nv_bfloat16* __restrict__ dH2,
                                                  const __nv_bfloat16* __restrict__ dH3, const float* __restrict__ H3,
                                                  const float* __restrict__ dy, int n, int chunk, float* part) {
  extern __shared__ __align__(16) uint8_t st_smem[];
  const int o = threadIdx.x, s0 = blockIdx.x * chunk, s1 = min(n, s0 + chunk);
  const int ntile = (s1 - s0) / SMALL_TILE;
  const uint32_t sbase = umma::smem_u32(st_smem);
  auto stage = [&](int k) {
    const int t0 = s0 + k * SMALL_TILE;
    const uint32_t b = sbase + (uint32_t)((k & 1) * ST_BYTES);
    const __nv_bfloat16* dh[4] = {dH0, dH1, dH2, dH3};
    constexpr int DH16 = SMALL_TILE * H * 2 / 16;  // 16-byte pieces of one dH tile
#pragma unroll
    for (int l = 0; l < 4; ++l)
      for (int q = o; q < DH16; q += H)
        cp_async16(b + ST_DH + (uint32_t)(l * DH16 + q) * 16u, reinterpret_cast<const uint8_t*>(dh[l] + (size_t)t0 * H) + q * 16);
    for (int q = o; q < SMALL_TILE * H * 4 / 16; q += H)
      cp_async16(b + ST_H3 + (uint32_t)q * 16u, reinterpret_cast<const uint8_t*>(H3 + (size_t)t0 * H) + q * 16);
    if (o < SMALL_TILE * NIN * 4 / 16)
      cp_async16(b + ST_XN + (uint32_t)o * 16u, reinterpret_cast<const uint8_t*>(xn + (size_t)t0 * NIN) + o * 16);
    if (o < SMALL_TILE * NOUT * 4 / 16)
      cp_async16(b + ST_DY + (uint32_t)o * 16u, reinterpret_cast<const uint8_t*>(dy + (size_t)t0 * NOUT) + o * 16);
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  float w0[NIN], b[4], w4[NOUT], b4 = 0.f;
#pragma unroll
  for (int i = 0; i < NIN; ++i) w0[i] = 0.f;
#pragma unroll
  for (int l = 0; l < 4; ++l) b[l] = 0.f;
#pragma unroll
  for (int m = 0; m < NOUT; ++m) w4[m] = 0.f;
  if (ntile > 0) stage(0);
  for (int k = 0; k < ntile; ++k) {
    if (k + 1 < ntile) {
      stage(k + 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const uint8_t* tb = st_smem + (k & 1) * ST_BYTES;
    const __nv_bfloat16* sdh = reinterpret_cast<const __nv_bfloat16*>(tb + ST_DH);
    const float* sh3 = reinterpret_cast<const float*>(tb + ST_H3);
    const float* sxn = reinterpret_cast<const float*>(tb + ST_XN);
    const float* sdy = reinterpret_cast<const float*>(tb + ST_DY);
#pragma unroll 4
    for (int s = 0; s < SMALL_TILE; ++s) {
      const float d0 = __bfloat162float(sdh[(0 * SMALL_TILE + s) * H + o]);
#pragma unroll
      for (int i = 0; i < NIN; ++i) w0[i] = fmaf(d0, sxn[s * NIN + i], w0[i]);
      b[0] += d0;
      b[1] += __bfloat162float(sdh[(1 * SMALL_TILE + s) * H + o]);
      b[2] += __bfloat162float(sdh[(2 * SMALL_TILE + s) * H + o]);
      b[3] += __bfloat162float(sdh[(3 * SMALL_TILE + s) * H + o]);
      const float a = gelu(sh3[s * H + o]);
#pragma unroll
      for (int m = 0; m < NOUT; ++m) w4[m] = fmaf(sdy[s * NOUT + m], a, w4[m]);
      if (o < NOUT) b4 += sdy[s * NOUT + o];
    }
    __syncthreads();  // the buffer is refilled by the next-but-one stage
  }
  float* p = part + (size_t)blockIdx.x * SMALL_N + o * SMALL_PER;
#pragma unroll
  for (int i = 0; i < NIN; ++i) p[i] = w0[i];
#pragma unroll
  for (int l = 0; l < 4; ++l) p[NIN + l] = b[l];
#pragma unroll
  for (int m = 0; m < NOUT; ++m) p[NIN + 4 + m] = w4[m];
  if (o < NOUT) part[(size_t)blockIdx.x * SMALL_N + H * SMALL_PER + o] = b4;
}

// The gradient vector from the partials, each summed in order: dW_1..3 over
// the z split-K partials of the hidden weight-gradient GEMMs, the thin
// parameters over the zs sample chunks of k_small_part.
__global__ void k_reduce_grads(const float* __restrict__ part, int z, const float* __restrict__ spart, int zs,
                               float* grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < 3 * H * H) {
    const int l = q / (H * H), e = q % (H * H);
    const float* p = part + (size_t)l * z * H * H;
    float a = 0.f;
#pragma unroll 8
    for (int k = 0; k < z; ++k) a += p[(size_t)k * H * H + e];
    grad[off_w(l + 1) + e] = a;
    return;
  }
  const int r = q - 3 * H * H;
  if (r >= SMALL_N) return;
  float a = 0.f;
#pragma unroll 8
  for (int k = 0; k < zs; ++k) a += spart[(size_t)k * SMALL_N + r];
  int dst;
  if (r < H * SMALL_PER) {
    const int o = r / SMALL_PER, k = r % SMALL_PER;
    dst = k < NIN ? OFF_W0 + o * NIN + k : k < NIN + 4 ? (k == NIN ? OFF_B0 : off_b(k - NIN)) + o
                                                       : OFF_W4 + (k - NIN - 4) * H + o;
  } else {
    dst = OFF_B4 + (r - H * SMALL_PER);
  }
  grad[dst] = a;
}

// the loss from k_head's partials: lane l sums partials l, l + 32, ... in
// order, then a butterfly over the lanes (one warp)
__global__ void k_loss_final(const float* part, int nb, int n, float* loss) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  float a = 0.f;
  for (int b = threadIdx.x; b < nb; b += 32) a += part[b];
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) a += __shfl_xor_sync(0xffffffffu, a, w);
  if (threadIdx.x == 0) *loss = a / (4.f * (float)n);
}

// Training batch number *it: `batch` pairs drawn with replacement from the n
// pairs (x: n x NIN, t: n x NOUT, row-major), pair index = splitmix64 (Steele,
// Lea and Flood, "Fast splittable pseudorandom number generators", 2014) of
// seed + (it * batch + i + 1) * golden gamma, modulo n; gathered into xb, tb.
__global__ void k_batch(const float* __restrict__ x, const float* __restrict__ t, long long n,
                        unsigned long long seed, const int* it, int batch, float* xb, float* tb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch) return;
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * ((unsigned long long)*it * (unsigned long long)batch +
                                                         (unsigned long long)i + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const long long j = (long long)(z % (unsigned long long)n);
#pragma unroll
  for (int k = 0; k < NIN; ++k) xb[(size_t)i * NIN + k] = x[(size_t)j * NIN + k];
#pragma unroll
  for (int k = 0; k < NOUT; ++k) tb[(size_t)i * NOUT + k] = t[(size_t)j * NOUT + k];
}

// End of training step k = *it of `steps`: the loss into hist[k] (if hist),
// the next Adam update's learning rate (cosine decay from lr at k = 0 to
// lr_end at k = steps - 1) and bias corrections 1 - beta^(t0 + k + 1) into
// sched, then *it = k + 1.
__global__ void k_train_tail(int* it, int steps, int t0, float lr, float lr_end, float b1, float b2,
                             const float* loss, float* hist, float* sched) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = *it;
  const double c = cos(3.141592653589793 * (double)k / (double)(steps > 1 ? steps - 1 : 1));
  sched[0] = (float)((double)lr_end + 0.5 * ((double)lr - (double)lr_end) * (1.0 + c));
  sched[1] = 1.f - powf(b1, (float)(t0 + k + 1));
  sched[2] = 1.f - powf(b2, (float)(t0 + k + 1));
  if (hist) hist[k] = *loss;
  *it = k + 1;
}

// sched (may be null): lr, bc1, bc2 of this step in device memory (k_train_tail)
__global__ void k_adam(float* p, float* m1, float* m2, const float* __restrict__ g, float lr, float b1, float b2,
                       float eps, float bc1, float bc2, const float* sched) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= NPARAM) return;
  if (sched) {
    lr = sched[0];
    bc1 = sched[1];
    bc2 = sched[2];
  }
  const float gq = g[q];
  const float a = b1 * m1[q] + (1.f - b1) * gq;
  const float b = b2 * m2[q] + (1.f - b2) * gq * gq;
  m1[q] = a;
  m2[q] = b;
  p[q] -= lr * (a / bc1) / (sqrtf(b / bc2) + eps);
}

// BF16 copies of the hidden weights: Wb[l][o][i] and WbT[l][i][o]
__global__ void k_pack(const float* __restrict__ p, __nv_bfloat16* Wb, __nv_bfloat16* WbT) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 3 * H * H) return;
  const int l = q / (H * H), o = (q % (H * H)) / H, i = q % H;
  const __nv_bfloat16 w = __float2bfloat16_rn(p[off_w(l + 1) + o * H + i]);
  Wb[q] = w;
  WbT[(size_t)l * H * H + i * H + o] = w;
}

// F16 weights of the inference kernel, swizzled in its shared-memory order
// (k_mlp_fwd16): hidden tiles, the layer-0 tile (K padded 7 -> 16 with zeros),
// the output tile (N padded 4 -> 16 with zeros).  Bytes of the tiles that the
// MMAs never read stay as the creation left them (zero).
// the F16 weights of k_mlp_fwd16: layers 1-4 times 1/2 (the epilogue forms
// 2 GELU), the layer-0 tile with b0 in K column 7 (the features' constant 1)
__global__ void k_pack16(const float* __restrict__ p, uint8_t* Wh) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int NH = 3 * H * H, N0 = H * 16, N4 = 16 * H;
  float v;
  uint32_t off;
  if (q < NH) {
    const int l = q / (H * H), o = (q % (H * H)) / H, i = q % H;
    v = 0.5f * p[off_w(l + 1) + o * H + i];
    off = (uint32_t)(l * TILE_BYTES) + umma::sw128_offset(o, i, 128);
  } else if (q < NH + N0) {
    const int o = (q - NH) / 16, i = (q - NH) % 16;
    v = i < NIN ? p[OFF_W0 + o * NIN + i] : i == NIN ? p[OFF_B0 + o] : 0.f;
    off = (uint32_t)F2_W0 + umma::sw128_offset(o, i, 128);
  } else if (q < NH + N0 + N4) {
    const int m = (q - NH - N0) / H, i = (q - NH - N0) % H;
    v = m < NOUT ? 0.5f * p[OFF_W4 + m * H + i] : 0.f;
    off = (uint32_t)F2_W4 + umma::sw128_offset(m, i, 16);
  } else {
    return;
  }
  *reinterpret_cast<__half*>(Wh + off) = __float2half_rn(v);
}
constexpr int PACK16_N = 3 * H * H + H * 16 + 16 * H;

}  // namespace mlp

// samples for training: raw features (T, p, Y1..Y4, dt) and targets
// z_k = dY_k / (c_k xi_s) (mlp::progress_scale; 1 where c_k xi_s is below
// the rounding of Y_k) from
// pairs of states (P before, P after dt) given in SoA layout
__global__ void k_surrogate_samples(const ThermoDev<4> th, const double* __restrict__ P0,
                                    const double* __restrict__ P1, const double* __restrict__ dt, int n, float* x,
                                    float* tgt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned e = 0;
  double Y[4], s = 0.0, Cp, gama, R, om[4];
  for (int k = 0; k < 3; ++k) { Y[k] = P0[(size_t)(4 + k) * n + i]; s = s + Y[k]; }
  Y[3] = 1.0 - s;
  const double p = P0[i], T = P0[(size_t)3 * n + i];
  gas<4>(th, Y, T, Cp, gama, R, e);
  const double rho = p / (T * R);
  production<4>(th, T, rho, Y, om);
  float* xi = x + (size_t)i * 7;
  xi[0] = (float)T; xi[1] = (float)p;
  for (int k = 0; k < 4; ++k) xi[2 + k] = (float)Y[k];
  xi[6] = (float)dt[i];
  const double xs = mlp::progress_scale(th, Y, om, dt[i], rho);
  for (int k = 0; k < 4; ++k) {
    float z = 1.f;
    const double sc = k < 3 ? th.prodc[k] * xs : 0.0;
    // below 1e-10 of the mass fraction the change is lost in the rounding of
    // Y and the explicit limit z = 1 is exact to that order
    if (fabs(sc) > 1e-10 * fmax(fabs(Y[k]), 1e-3)) {
      const double dY = P1[(size_t)(4 + k) * n + i] - P0[(size_t)(4 + k) * n + i];
      z = (float)(dY / sc);
    }
    tgt[(size_t)i * 4 + k] = z;
  }
}

}  // namespace rc

using namespace rc;

struct rc_mlp {
  int device = 0;
  float* params = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  __nv_bfloat16* Wb = nullptr;
  __nv_bfloat16* WbT = nullptr;
  uint8_t* Wh = nullptr;  // F16 weights of the inference kernel (k_pack16)
  unsigned* derr = nullptr;
  mlp::Norm norm{};
  int step = 0;
  // training work buffers for up to cap samples
  int cap = 0, zsplit = 1;
  std::vector<void*> work;
  float *xn = nullptr, *Hs[4] = {}, *dy = nullptr, *loss_part = nullptr, *loss = nullptr, *part = nullptr,
        *grad = nullptr;
  float* spart = nullptr;                                // k_small_part's partials
  cudaStream_t side = nullptr;                           // the weight-gradient branch
  cudaEvent_t ev_dh[4] = {}, ev_join = nullptr;          // dH_l ready / the branch done
  float *xb = nullptr, *tb = nullptr, *sched = nullptr;  // rc_mlp_train: the batch, the step's schedule
  int* it = nullptr;                                     // rc_mlp_train: the step counter
  __nv_bfloat16 *Arow[3] = {}, *Acol[3] = {}, *dHrow[4] = {}, *dHcol[4] = {};
  std::string err;
};

namespace {

int mlp_fail(rc_mlp* m, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RC_OK;
  if (m) m->err = std::string(what) + ": " + cudaGetErrorString(e);
  return RC_ERR_CUDA;
}
#define MLP_CU(call)                                          \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return mlp_fail(m, e_, #call);     \
  } while (0)

int fused_grid(int device, int n) {
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  const int ctas = ((n + 127) / 128 + mlp::FG - 1) / mlp::FG;
  return ctas < nsm ? (ctas > 0 ? ctas : 1) : nsm;
}

template <class T>
int alloc_work(rc_mlp* m, size_t count, T** out) {
  void* p = nullptr;
  MLP_CU(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
  m->work.push_back(p);
  *out = static_cast<T*>(p);
  return RC_OK;
}

// split-K slices of the hidden weight-gradient GEMMs, at most
constexpr int ZSPLIT_MAX = 64;
int ensure_work(rc_mlp* m, int n) {
  if (n <= m->cap) return RC_OK;
  for (void* p : m->work) cudaFree(p);
  m->work.clear();
  const size_t N = (size_t)n, Hh = mlp::H;
  int st = 0;
  st |= alloc_work(m, N * mlp::NIN, &m->xn);
  for (int l = 0; l < 4; ++l) st |= alloc_work(m, N * Hh, &m->Hs[l]);
  for (int l = 0; l < 3; ++l) {
    st |= alloc_work(m, N * Hh, &m->Arow[l]);
    st |= alloc_work(m, N * Hh, &m->Acol[l]);
  }
  for (int l = 0; l < 4; ++l) {
    st |= alloc_work(m, N * Hh, &m->dHrow[l]);
    st |= alloc_work(m, N * Hh, &m->dHcol[l]);
  }
  st |= alloc_work(m, N * mlp::NOUT, &m->dy);
  st |= alloc_work(m, (N + mlp::HEAD_SAMPLES - 1) / mlp::HEAD_SAMPLES, &m->loss_part);
  st |= alloc_work(m, (size_t)1, &m->loss);
  st |= alloc_work(m, N * mlp::NIN, &m->xb);
  st |= alloc_work(m, N * mlp::NOUT, &m->tb);
  st |= alloc_work(m, (size_t)4, &m->sched);
  st |= alloc_work(m, (size_t)1, &m->it);
  // split-K partials of the weight gradients, for up to n / 1024 splits
  m->zsplit = std::max(1, std::min(ZSPLIT_MAX, n / 256));
  st |= alloc_work(m, (size_t)3 * m->zsplit * Hh * Hh, &m->part);
  st |= alloc_work(m, (size_t)mlp::SMALL_ZMAX * mlp::SMALL_N, &m->spart);
  if (st) return st;
  m->cap = n;
  return RC_OK;
}

}  // namespace

namespace rc {
// inference over the cells of a solver context (NSP must be 4)
cudaError_t surrogate_source(const Dev& d, const void* th, const rc_mlp* net, float spread_tol, int* list,
                             unsigned* nlist, unsigned* nsurr, const int* mode, unsigned char* dec, cudaStream_t s) {
  mlp::IoSolver io{d, *static_cast<const ThermoDev<4>*>(th), spread_tol, list, nlist, nsurr, mode, dec};
  mlp::k_mlp_fwd16<mlp::IoSolver><<<fused_grid(net->device, d.NE), 128 * mlp::FG, mlp::F2_SMEM, s>>>(
      reinterpret_cast<const uint4*>(net->Wh), net->params, net->norm, io, d.NE, d.err);
  return cudaGetLastError();
}
// outside stream capture, once per context
cudaError_t surrogate_prepare() {
  return cudaFuncSetAttribute(mlp::k_mlp_fwd16<mlp::IoSolver>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              mlp::F2_SMEM);
}
cudaError_t surrogate_samples(const void* th, const double* P0, const double* P1, const double* dt, int n, float* x,
                              float* t, cudaStream_t s) {
  k_surrogate_samples<<<(n + 127) / 128, 128, 0, s>>>(*static_cast<const ThermoDev<4>*>(th), P0, P1, dt, n, x, t);
  return cudaGetLastError();
}
}  // namespace rc

extern "C" {

int rc_mlp_create(int device, rc_mlp** out) {
  if (!out) return RC_ERR_ARG;
  *out = nullptr;
  rc_mlp* m = new rc_mlp();
  m->device = device;
  auto bail = [&](int st) {
    rc_mlp_destroy(m);
    return st;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(RC_ERR_CUDA);
  const size_t P = mlp::NPARAM;
  if (cudaMalloc(&m->params, P * sizeof(float)) != cudaSuccess || cudaMalloc(&m->m1, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->m2, P * sizeof(float)) != cudaSuccess || cudaMalloc(&m->grad, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->Wb, 3 * mlp::H * mlp::H * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&m->WbT, 3 * mlp::H * mlp::H * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&m->Wh, mlp::WH_BYTES) != cudaSuccess || cudaMalloc(&m->derr, sizeof(unsigned)) != cudaSuccess)
    return bail(RC_ERR_CUDA);
  cudaMemset(m->Wh, 0, mlp::WH_BYTES);
  cudaMemset(m->params, 0, P * sizeof(float));
  cudaMemset(m->m1, 0, P * sizeof(float));
  cudaMemset(m->m2, 0, P * sizeof(float));
  cudaMemset(m->derr, 0, sizeof(unsigned));
  if (cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking) != cudaSuccess) return bail(RC_ERR_CUDA);
  for (auto& e : m->ev_dh)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bail(RC_ERR_CUDA);
  if (cudaEventCreateWithFlags(&m->ev_join, cudaEventDisableTiming) != cudaSuccess) return bail(RC_ERR_CUDA);
  // the fills run on the legacy stream; the network's kernels may run on
  // non-blocking streams, which are not ordered after it
  if (cudaDeviceSynchronize() != cudaSuccess) return bail(RC_ERR_CUDA);
  for (int i = 0; i < mlp::NIN; ++i) { m->norm.mean[i] = 0.f; m->norm.stdv[i] = 1.f; }
  const float dom[6] = {300.f, 6000.f, 1.0e2f, 2.0e7f, 1.0e-10f, 1.0e-4f};
  for (int i = 0; i < 6; ++i) m->norm.dom[i] = dom[i];
  if (cudaFuncSetAttribute(mlp::k_mlp_fwd16<mlp::IoRaw>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           mlp::F2_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(mlp::k_gemm<mlp::EPI_FWD, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::GEMM_SMEM) !=
          cudaSuccess ||
      cudaFuncSetAttribute(mlp::k_gemm<mlp::EPI_BWD, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::GEMM_SMEM) !=
          cudaSuccess ||
      cudaFuncSetAttribute(mlp::k_gemm<mlp::EPI_F32, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::GEMM_SMEM) !=
          cudaSuccess ||
      cudaFuncSetAttribute(mlp::k_small_part, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::SMALL_SMEM) !=
          cudaSuccess)
    return bail(RC_ERR_CUDA);
  *out = m;
  return RC_OK;
}

int rc_mlp_destroy(rc_mlp* m) {
  if (!m) return RC_OK;
  for (void* p : m->work) cudaFree(p);
  cudaFree(m->params); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->grad);
  cudaFree(m->Wb); cudaFree(m->WbT); cudaFree(m->Wh); cudaFree(m->derr);
  for (cudaEvent_t e : m->ev_dh)
    if (e) cudaEventDestroy(e);
  if (m->ev_join) cudaEventDestroy(m->ev_join);
  if (m->side) cudaStreamDestroy(m->side);
  delete m;
  return RC_OK;
}

const char* rc_mlp_last_error(rc_mlp* m) { return m ? m->err.c_str() : "no network"; }

int rc_mlp_set_params(rc_mlp* m, const float* params) {
  if (!m || !params) return RC_ERR_ARG;
  MLP_CU(cudaMemcpy(m->params, params, sizeof(float) * mlp::NPARAM, cudaMemcpyHostToDevice));
  MLP_CU(cudaMemset(m->m1, 0, sizeof(float) * mlp::NPARAM));
  MLP_CU(cudaMemset(m->m2, 0, sizeof(float) * mlp::NPARAM));
  m->step = 0;
  mlp::k_pack<<<(3 * mlp::H * mlp::H + 255) / 256, 256>>>(m->params, m->Wb, m->WbT);
  mlp::k_pack16<<<(mlp::PACK16_N + 255) / 256, 256>>>(m->params, m->Wh);
  MLP_CU(cudaGetLastError());
  MLP_CU(cudaDeviceSynchronize());
  return RC_OK;
}

int rc_mlp_get_params(rc_mlp* m, float* params) {
  if (!m || !params) return RC_ERR_ARG;
  MLP_CU(cudaMemcpy(params, m->params, sizeof(float) * mlp::NPARAM, cudaMemcpyDeviceToHost));
  return RC_OK;
}

int rc_mlp_set_norm(rc_mlp* m, const float* mean, const float* stdv, const float* domain) {
  if (!m || !mean || !stdv) return RC_ERR_ARG;
  for (int i = 0; i < mlp::NIN; ++i) {
    if (!(stdv[i] > 0.f)) return RC_ERR_ARG;
    m->norm.mean[i] = mean[i];
    m->norm.stdv[i] = stdv[i];
  }
  if (domain)
    for (int i = 0; i < 6; ++i) m->norm.dom[i] = domain[i];
  return RC_OK;
}

int rc_mlp_forward(rc_mlp* m, const float* d_x, int n, float* d_y, void* stream) {
  if (!m || n < 0 || (n > 0 && (!d_x || !d_y))) return RC_ERR_ARG;
  if (n == 0) return RC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mlp::IoRaw io{d_x, d_y};
  mlp::k_mlp_fwd16<mlp::IoRaw><<<fused_grid(m->device, n), 128 * mlp::FG, mlp::F2_SMEM, s>>>(
      reinterpret_cast<const uint4*>(m->Wh), m->params, m->norm, io, n, m->derr);
  MLP_CU(cudaGetLastError());
  return RC_OK;
}

}  // extern "C"

namespace {
// the kernels of one loss-and-gradient evaluation on n samples (work buffers
// sized for n), enqueued on s without synchronising
int enqueue_gradient(rc_mlp* m, const float* d_x, const float* d_t, int n, float* d_grad, cudaStream_t s) {
  using namespace mlp;
  // split-K of the weight gradients: about 2 chunks of 128 samples per CTA
  // (at most ZSPLIT_MAX splits), an exact divisor of the n / 128 chunks (each
  // split a whole number of chunks)
  int z = std::max(1, std::min(m->zsplit, n / 256));
  while ((n / 128) % z) --z;
  // sample chunks of the thin parameters' gradients: 64 samples or more, at
  // most SMALL_ZMAX chunks (n is a multiple of 128, so every chunk is whole tiles)
  const int chunk = 64 * ((n + 64 * SMALL_ZMAX - 1) / (64 * SMALL_ZMAX)), zs = (n + chunk - 1) / chunk;
  k_layer0<<<(n + 31) / 32, L0_THREADS, 0, s>>>(d_x, m->norm, m->params, n, m->xn, m->Hs[0], m->Arow[0], m->Acol[0]);
  // hidden layers 1..3 forward: H_l = A_{l-1} W_l^T + b_l
  for (int l = 1; l <= 3; ++l) {
    GemmArgs g{};
    g.A = m->Arow[l - 1]; g.lda = H;
    g.B = m->Wb + (size_t)(l - 1) * H * H; g.ldb = H;
    g.M = n; g.N = H; g.K = H;
    g.bias = m->params + off_b(l);
    g.Hout = m->Hs[l];
    g.Orow = l < 3 ? m->Arow[l] : m->dHrow[3];   // A3 row is not needed (the head recomputes it)
    g.Ocol = l < 3 ? m->Acol[l] : m->dHcol[3];   // scratch for l = 3, overwritten by the head
    g.err = m->derr;
    k_gemm<EPI_FWD, 64><<<dim3(H / 64, n / 128, 1), 128, GEMM_SMEM, s>>>(g);
  }
  k_head<<<(n + HEAD_SAMPLES - 1) / HEAD_SAMPLES, HEAD_THREADS, 0, s>>>(m->Hs[3], d_t, m->params, n, m->dy,
                                                                         m->dHrow[3], m->dHcol[3], m->loss_part);
  // backward data: dH_{l-1} = (dH_l W_l) * gelu'(H_{l-1}) on s; each weight
  // gradient dW_l = dH_l^T A_{l-1} (split-K partials) on the side stream as
  // soon as dH_l is ready, then the thin parameters' partials; s joins the
  // side stream before the reduction
  auto wgrad = [&](int l) {
    GemmArgs g{};
    g.A = m->dHcol[l]; g.lda = n;
    g.B = m->Acol[l - 1]; g.ldb = n;
    g.M = H; g.N = H; g.K = n;
    g.C = m->part + (size_t)(l - 1) * z * H * H;
    g.err = m->derr;
    k_gemm<EPI_F32, 128><<<dim3(1, 1, z), 128, GEMM_SMEM, m->side>>>(g);
  };
  MLP_CU(cudaEventRecord(m->ev_dh[3], s));
  MLP_CU(cudaStreamWaitEvent(m->side, m->ev_dh[3], 0));
  wgrad(3);
  for (int l = 3; l >= 1; --l) {
    GemmArgs g{};
    g.A = m->dHrow[l]; g.lda = H;
    g.B = m->WbT + (size_t)(l - 1) * H * H; g.ldb = H;
    g.M = n; g.N = H; g.K = H;
    g.Hin = m->Hs[l - 1];
    g.Orow = m->dHrow[l - 1];
    g.Ocol = m->dHcol[l - 1];
    g.err = m->derr;
    k_gemm<EPI_BWD, 64><<<dim3(H / 64, n / 128, 1), 128, GEMM_SMEM, s>>>(g);
    MLP_CU(cudaEventRecord(m->ev_dh[l - 1], s));
    MLP_CU(cudaStreamWaitEvent(m->side, m->ev_dh[l - 1], 0));
    if (l > 1) wgrad(l - 1);
  }
  k_small_part<<<zs, H, SMALL_SMEM, m->side>>>(m->xn, m->dHrow[0], m->dHrow[1], m->dHrow[2], m->dHrow[3], m->Hs[3],
                                              m->dy, n, chunk, m->spart);
  MLP_CU(cudaEventRecord(m->ev_join, m->side));
  MLP_CU(cudaStreamWaitEvent(s, m->ev_join, 0));
  k_reduce_grads<<<(3 * H * H + SMALL_N + 255) / 256, 256, 0, s>>>(m->part, z, m->spart, zs, d_grad);
  k_loss_final<<<1, 32, 0, s>>>(m->loss_part, (n + HEAD_SAMPLES - 1) / HEAD_SAMPLES, n, m->loss);
  MLP_CU(cudaGetLastError());
  return RC_OK;
}
}  // namespace

extern "C" {

int rc_mlp_gradient(rc_mlp* m, const float* d_x, const float* d_t, int n, float* d_grad, float* loss,
                    void* stream) {
  if (!m || !d_x || !d_t || !d_grad || n <= 0 || n % 128) return RC_ERR_ARG;
  if (int st = ensure_work(m, n)) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (int st = enqueue_gradient(m, d_x, d_t, n, d_grad, s)) return st;
  if (loss) {
    MLP_CU(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    unsigned e = 0;
    MLP_CU(cudaMemcpyAsync(&e, m->derr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    MLP_CU(cudaStreamSynchronize(s));
    if (e) {
      m->err = "tensor-core wait gave up";
      return (int)e;
    }
  }
  return RC_OK;
}

int rc_mlp_adam(rc_mlp* m, const float* d_grad, float lr, float beta1, float beta2, float eps, void* stream) {
  if (!m || !d_grad) return RC_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  m->step += 1;
  const float bc1 = 1.f - std::pow(beta1, (float)m->step), bc2 = 1.f - std::pow(beta2, (float)m->step);
  mlp::k_adam<<<(mlp::NPARAM + 255) / 256, 256, 0, s>>>(m->params, m->m1, m->m2, d_grad, lr, beta1, beta2, eps, bc1,
                                                       bc2, nullptr);
  mlp::k_pack<<<(3 * mlp::H * mlp::H + 255) / 256, 256, 0, s>>>(m->params, m->Wb, m->WbT);
  mlp::k_pack16<<<(mlp::PACK16_N + 255) / 256, 256, 0, s>>>(m->params, m->Wh);
  MLP_CU(cudaGetLastError());
  return RC_OK;
}

// Adam on `steps` batches drawn on the device (k_batch), the learning rate
// and bias corrections formed on the device (k_train_tail): one step (draw,
// loss and gradient, Adam, the packed weights) is captured once as a CUDA
// graph on a private stream and launched `steps` times on the caller's.
int rc_mlp_train(rc_mlp* m, const float* d_x, const float* d_t, long long n, int steps, int batch, float lr,
                 float lr_end, float beta1, float beta2, float eps, unsigned long long seed, float* d_loss,
                 void* stream) {
  if (!m || !d_x || !d_t || n <= 0 || steps < 0 || batch <= 0 || batch % 128) return RC_ERR_ARG;
  if (steps == 0) return RC_OK;
  if (int st = ensure_work(m, batch)) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  using namespace mlp;
  MLP_CU(cudaMemsetAsync(m->it, 0, sizeof(int), s));
  MLP_CU(cudaMemsetAsync(m->derr, 0, sizeof(unsigned), s));
  cudaStream_t cs = nullptr;
  MLP_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  int st = RC_OK;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    k_batch<<<(batch + 127) / 128, 128, 0, cs>>>(d_x, d_t, n, seed, m->it, batch, m->xb, m->tb);
    st = enqueue_gradient(m, m->xb, m->tb, batch, m->grad, cs);
    k_train_tail<<<1, 32, 0, cs>>>(m->it, steps, m->step, lr, lr_end, beta1, beta2, m->loss, d_loss, m->sched);
    k_adam<<<(NPARAM + 255) / 256, 256, 0, cs>>>(m->params, m->m1, m->m2, m->grad, lr, beta1, beta2, eps, 1.f, 1.f,
                                                m->sched);
    k_pack<<<(3 * H * H + 255) / 256, 256, 0, cs>>>(m->params, m->Wb, m->WbT);
    k_pack16<<<(PACK16_N + 255) / 256, 256, 0, cs>>>(m->params, m->Wh);
    const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    e = e2 != cudaSuccess ? e2 : cudaGetLastError();
  }
  if (e == cudaSuccess && st == RC_OK) e = cudaGraphInstantiate(&ge, g, 0);
  for (int k = 0; e == cudaSuccess && st == RC_OK && k < steps; ++k) e = cudaGraphLaunch(ge, s);
  unsigned derr = 0;
  if (e == cudaSuccess && st == RC_OK) e = cudaMemcpyAsync(&derr, m->derr, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && st == RC_OK) e = cudaStreamSynchronize(s);
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  if (st) return st;
  MLP_CU(e);
  m->step += steps;
  if (derr) {
    m->err = "tensor-core wait gave up";
    return (int)derr;
  }
  return RC_OK;
}

}  // extern "C"
