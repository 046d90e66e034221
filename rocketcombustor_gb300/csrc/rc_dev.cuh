// Device layout shared by the FP64 and mixed-precision kernels.
#pragma once
#include <cstdint>
#include <utility>

#include "rc_thermo.cuh"

namespace rc {

constexpr int MAXF = 4;  // faces per cell (triangles and quadrilaterals)

struct Dev {
  int NE, NF, NG;
  int bs;                        // threads per block of the cell and face kernels (32, 64 or 128)
  int cpw;                       // LU-SGS cells per warp (1, 2, 4 or 8; 4 lanes per cell)
  unsigned spin_limit;           // polls before a level wait of the persistent LU-SGS gives up
  // cells
  const double* vol;
  const double* rinv;            // [2*NE] 1./reflen
  const unsigned char* nface;    // KFace
  const unsigned char* cleft;    // bit q: cell is Neighbor(1,.) of its face q
  const int* cface;              // [4*NE] NeighF, 0-based
  const int* cother;             // [4*NE] cell across face q, -1 on a boundary
  const unsigned char* nnei;     // Neigh
  const int* cnei;               // [4*NE] NeighC(1:Neigh), 0-based
  const unsigned char* ngh;      // Num_ghostcell
  const int* cgh;                // [4*NE] Ghostcell, 0-based
  const double* wdis;            // [4*NE]
  const double* amls;            // [8*NE] AMLS(r,q,i) at (2q+r)*NE+i
  const double* lvvh;            // [8*NE] limiter basis values at the face midpoints
  // faces
  const int* fNL;                // 0-based
  const int* fNR;                // 0-based cell, or -BC code
  const double* fvec;            // [2*NF] VECX
  const double* fsav;            // max(|VECX|, small)
  const double* fsn;             // [2*NF] unit normal
  const double* fss;             // sqrt(dx*dx+dy*dy)
  const double* fs2;             // dx*dx+dy*dy
  const double* fvL;             // [2*NF] fbaseAll at the Gauss point for NL
  const double* fvR;             // [2*NF] fbaseAll at the Gauss point for NR
  const double* fdxk;            // |(x_L - x_R).n|
  const double* fdxkr;           // its reciprocal pair (2 planes), interior faces
  const double* fysn;            // [2*NF] yita*n
  // ghosts
  const int* gtype;
  const double* gsn;             // [2*NG] ghost-face unit normal
  // state and work arrays
  double* PA;
  double* WA;
  double* hWA;
  double* grad;
  double* GPA;
  double* step;
  double* dd;
  double* cst;                   // [(3+NSP)*NE]: rho, gamma, rho*E, h_k
  double* rcp;                   // [6*NE]: reciprocal pairs (h, l) of rho, gamma - 1 and dd
  double* src;                   // [(NSP-1)*NE]: vol*omega_k
  double* alpa;
  double* visL;
  double* visR;
  double* alpaF;
  double* Finv;                  // [V*NF]
  double* Fvis;                  // [(V-1)*NF], component 1 is identically zero
  unsigned* err;
  // mixed precision (allocated only for RC_PREC_MIXED)
  float* grad32;                 // [2*V*NE]
  float* GPA32;                  // [V*NG]
  float* Finv32;                 // [V*NF]
  float* Fvis32;                 // [(V-1)*NF]
  float* PA32;                   // [V*NE] FP32 copy of PA read by the FP32 sweeps
  float* cst32;                  // [(3+NSP)*NE] FP32 cell gas state
  float* dU32;                   // [V*NE] FP32 copy of dU written by the FP32 sweeps
  float* alpaF32;                // [NF]
  float* fvec32;                 // [2*NF]
  // LU-SGS sweep tables in level order, [0] forward / [1] backward: position t
  // holds cell swi[t]; slot q holds the neighbour read in that sweep
  // (swj[q*NE+t], -1 if none) and its face (swf[q*NE+t], bitwise-complemented
  // when the cell is the face's right cell, i.e. the normal is reversed).
  const int* swi[2];
  const int* swj[2];
  const int* swf[2];
  // boundary data per case (a batch of independent cases shares one mesh
  // numbering): row c of bctab holds case c's oxidizer / fuel inlet Y, T and
  // mass flux and its exit pressure (BC_* offsets); fcase / gcase give the case
  // of a face / ghost cell, or are null for a single case (row 0).
  const double* bctab;
  const float* bctab32;
  const int* fcase;
  const int* gcase;
  // unsteady dual-time BDF2 (allocated on first use)
  double* WP;                    // [V*NE] WA of the previous physical step
  double* WP2;                   // [V*NE] WA of the step before
  double* bfix;                  // [V*NE] vol/dt ((1+2 phi) WP - phi WP2)
  double* bmat;                  // [NE*V*(2V+4)] per cell, per row: equilibrated row, LU row, r, c, 1/U_rr (2)
  int* bperm;                    // [8*NE] per cell: source row of each row after the interchanges; [7] flags
  double* bnb;                   // [(11+2*NSP)*NE] gas state of each cell as seen by its neighbours' sweeps
  const double* bpar;            // {dt, phi}
};

// launch as a programmatic dependent of the previous kernel of the stream
// (cudaLaunchAttributeProgrammaticStreamSerialization)
template <class... Args, class... Act>
inline void launch_pdl(void (*kernel)(Args...), unsigned grid, unsigned block, cudaStream_t s, Act&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Act>(args)...);
}

constexpr int BCS = 13;                 // doubles per bctab row
constexpr int BC_Y = 0, BC_T = 8, BC_MFLOW = 10, BC_POUT = 12;  // + w*NSPMAX (Y) or + w (T, mass flux)
constexpr int BC_NSPMAX = 4;

__device__ __forceinline__ const double* bc_row(const Dev& d, const int* ids, int i) {
  return d.bctab + (ids ? ids[i] : 0) * BCS;
}
__device__ __forceinline__ const float* bc_row32(const Dev& d, const int* ids, int i) {
  return d.bctab32 + (ids ? ids[i] : 0) * BCS;
}

__device__ __forceinline__ void flag(const Dev& d, unsigned e) {
  if (e) atomicOr(d.err, e);
}

__device__ __forceinline__ void removedirection(double& vx, double& vy, double nx, double ny) {
  const double vn = vx * nx + vy * ny;  // flux_viscous.f90:352-361
  vx = vx - vn * nx;
  vy = vy - vn * ny;
}

// Programmatic dependent launch (kernels launched with
// cudaLaunchAttributeProgrammaticStreamSerialization): let the next kernel of
// the stream start its prologue now / wait until the previous kernel of the
// stream has completed and its writes are visible.  Without the attribute
// both are no-ops.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// WA += hWA and update_primitve_variables (update_flow_variables.f90:4-48).
template <int NSP>
__device__ __forceinline__ void update_cell(const Dev& d, const ThermoDev<NSP>& th, int i, unsigned& err) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
  double W[V];
#pragma unroll
  for (int k = 0; k < V; ++k) {
    W[k] = d.WA[k * NE + i] + d.hWA[k * NE + i];
    d.WA[k * NE + i] = W[k];
  }
  const double rho = W[0], u = W[1] / rho, v = W[2] / rho;
  double Y[NSP], s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { Y[k] = W[4 + k] / rho; s = s + Y[k]; }
  Y[NSP - 1] = 1.0 - s;
  double Rcpcv;
  const double t = newton_T<NSP>(th, W[3] / rho - 0.5 * (u * u + v * v), Y, d.PA[3 * NE + i], Rcpcv, err);
  d.PA[0 * NE + i] = rho * Rcpcv * t;
  d.PA[1 * NE + i] = u;
  d.PA[2 * NE + i] = v;
  d.PA[3 * NE + i] = t;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) d.PA[(4 + k) * NE + i] = Y[k];
  if (i == 0 && isnan(W[0])) err |= ERR_NAN;
}

// Level ordering of the persistent LU-SGS kernels.  wait_count: lane 0 of a
// warp waits until the completion count of the previous level reaches its
// number of chunks; the warp then reads what that level wrote.  The wait is
// bounded: after about `limit` polls, or as soon as another waiter has given up,
// ERR_SYNC is latched and false returned, and the kernel returns.
__device__ __forceinline__ bool wait_count(const unsigned* c, unsigned target, unsigned* err, unsigned limit) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    for (unsigned spin = 0; ld_acquire(c) < target; ++spin) {
      if (spin >= limit || ((spin & 255u) == 255u && (ld_acquire(err) & ERR_SYNC))) {
        atomicOr(err, ERR_SYNC);
        ok = 0;
        break;
      }
    }
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  __threadfence();
  return ok != 0;
}
// named barrier over the first `count` threads of the block (warp multiples)
__device__ __forceinline__ void bar_named(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// bar.arrive: count this warp in at barrier id without waiting
__device__ __forceinline__ void bar_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// Tables of the dataflow LU-SGS (k_lusgs_flow): cells are
// split into per-SM blocks, a pass is a run of at most 8 consecutive sweep
// positions of one level whose cells one block owns.
struct FlowDev {
  const int* pstart;   // first sweep position of pass p
  const int* pcount;   // its number of cells (1..8)
  const int* boff[2];  // passes of block b: blist[d][boff[d][b] .. boff[d][b+1]), d = 0 forward, 1 backward
  const int* blist[2];
  const int* doff;     // passes that pass p waits for: deps[doff[p] .. doff[p+1])
  const int* deps;
  unsigned* pflag;     // per pass: epoch of the launch that finished it
  unsigned* ctr;       // [0] epoch of the last finished launch, [1] finished blocks
  // compact passes only (k_lusgs_flowc; null otherwise): a pass is split into
  // G groups of consecutive cells; group g of pass p holds gcell[p*G + g]
  // cells (0..16) and the active (position, slot) pairs
  // plist[poff[p*G + g] .. poff[p*G + g + 1]) (0..32), each position << 2 | slot
  const int* gcell;
  const int* poff;
  const int* plist;
};
// Compact passes: at most FLOWC_PAIRS active pairs per group (one per lane
// of a warp) and flowc_cells(V) cells, the cells that 128 finishing lanes
// hold at V lanes per cell (18 for four species, 32 for one).
constexpr int FLOWC_PAIRS = 32;
__host__ __device__ constexpr int flowc_cells(int V) { return 128 / V < 32 ? 128 / V : 32; }

// Dataflow LU-SGS: pass flags.  wait_flag: the calling thread waits until
// the flag reaches `epoch` (acquire); bounded like wait_count.  set_flag
// publishes a pass (release: the block's earlier stores, ordered before the
// call by a block barrier, become visible with it).
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ bool wait_flag(const unsigned* f, unsigned epoch, unsigned* err, unsigned limit) {
  for (unsigned spin = 0; ld_acquire(f) < epoch; ++spin) {
    if (spin >= limit || ((spin & 255u) == 255u && (ld_acquire(err) & ERR_SYNC))) {
      atomicOr(err, ERR_SYNC);
      return false;
    }
  }
  return true;
}
// count_done: a warp's chunk of a level is done; every lane's stores are
// made visible, then lane 0 counts the chunk.
__device__ __forceinline__ void count_done(unsigned* c) {
  __threadfence();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) atomicAdd(c, 1u);
}

}  // namespace rc

