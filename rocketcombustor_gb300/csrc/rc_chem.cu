// Chemistry integrator kernels (FP64, --fmad=false): the integrated chemical
// source of the steady iteration and the batch integration of given states.
//
// The work per cell is uneven (1 to maxsub substeps, each with rejections), so
// both kernels are persistent work queues: every warp takes the next 32 items
// from a counter until none are left.  Results do not depend on which warp
// takes which item.
#include <cuda_runtime.h>

#include "rc_chem.cuh"
#include "rc_dev.cuh"

namespace rc {

constexpr int CHEM_THREADS = 128;

__device__ __forceinline__ int next_chunk(unsigned* counter) {
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = (int)atomicAdd(counter, 32u);
  return __shfl_sync(0xffffffffu, base, 0);
}

// Integrated source of cell i (sourceterm.f90:43-51 with omega replaced by
// the mean rate over the cell's pseudo time step):
//   src_k = vol * (rho * ((Y_k(step) - Y_k) / step)).
template <int NSP>
__device__ __forceinline__ void integrate_cell(const Dev& d, const ThermoDev<NSP>& th, int i, double tol, int maxsub,
                                               int* nsub, unsigned& err) {
  constexpr int V = 3 + NSP;
  const int NE = d.NE;
  double P[V], P0[V], Y[NSP], Cp, gama, Rcpcv;
#pragma unroll
  for (int k = 0; k < V; ++k) { P[k] = d.PA[k * NE + i]; P0[k] = P[k]; }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) { Y[k] = P[4 + k]; s = s + Y[k]; }
  Y[NSP - 1] = 1.0 - s;
  gas<NSP>(th, Y, P[3], Cp, gama, Rcpcv, err);
  const double rho = P[0] / (P[3] * Rcpcv);
  const double dt = d.step[i];
  nsub[i] = chem_integrate<NSP>(th, P, dt, tol, maxsub, err);
  const double vol = d.vol[i];
#pragma unroll
  for (int k = 0; k < NSP - 1; ++k) d.src[k * NE + i] = vol * (rho * ((P[4 + k] - P0[4 + k]) / dt));
}

// Cells are taken in `order` (longest previous integration first, so the long
// cells start early and warps hold cells of similar cost), or in cell order
// when order is null.
template <int NSP>
__global__ void __launch_bounds__(CHEM_THREADS) k_chem_source(const Dev d, const ThermoDev<NSP> th, double tol,
                                                              int maxsub, int* __restrict__ nsub,
                                                              const int* __restrict__ order, unsigned* counter) {
  const int NE = d.NE;
  unsigned err = 0;
  for (;;) {
    const int base = next_chunk(counter);
    if (base >= NE) break;
    const int q = base + (threadIdx.x & 31);
    if (q < NE) integrate_cell<NSP>(d, th, order ? order[q] : q, tol, maxsub, nsub, err);
  }
  flag(d, err);
}

// Counting sort of the cells by their previous substep count, descending
// (bucket 255 - min(nsub, 255)); the order inside a bucket does not matter.
constexpr int NBUCKET = 256;
__global__ void k_chem_hist(const int* __restrict__ nsub, int n, unsigned* hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&hist[NBUCKET - 1 - min(max(nsub[i], 0), NBUCKET - 1)], 1u);
}
__global__ void k_chem_scan(unsigned* hist) {  // one block of NBUCKET threads: exclusive scan in place
  __shared__ unsigned sh[NBUCKET];
  const int t = threadIdx.x;
  sh[t] = hist[t];
  __syncthreads();
  for (int o = 1; o < NBUCKET; o <<= 1) {
    const unsigned v = t >= o ? sh[t - o] : 0u;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  hist[t] = t ? sh[t - 1] : 0u;
}
__global__ void k_chem_scatter(const int* __restrict__ nsub, int n, unsigned* cursor, int* __restrict__ order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) order[atomicAdd(&cursor[NBUCKET - 1 - min(max(nsub[i], 0), NBUCKET - 1)], 1u)] = i;
}

// The same for the cells list[0 .. *nlist) (the surrogate's fallbacks).
template <int NSP>
__global__ void __launch_bounds__(CHEM_THREADS) k_chem_list(const Dev d, const ThermoDev<NSP> th, double tol,
                                                            int maxsub, int* __restrict__ nsub,
                                                            const int* __restrict__ list,
                                                            const unsigned* __restrict__ nlist, unsigned* counter) {
  const int n = (int)min(*nlist, (unsigned)d.NE);
  unsigned err = 0;
  for (;;) {
    const int base = next_chunk(counter);
    if (base >= n) break;
    const int q = base + (threadIdx.x & 31);
    if (q < n) integrate_cell<NSP>(d, th, list[q], tol, maxsub, nsub, err);
  }
  flag(d, err);
}

// n primitive states in SoA ([k*n + i]) integrated over dt[i].
template <int NSP>
__global__ void __launch_bounds__(CHEM_THREADS) k_chem_batch(const ThermoDev<NSP> th, const double* __restrict__ Pin,
                                                             const double* __restrict__ dts, int n,
                                                             double* __restrict__ Pout, int* __restrict__ nsub,
                                                             double tol, int maxsub, unsigned* counter,
                                                             unsigned* errp) {
  constexpr int V = 3 + NSP;
  unsigned err = 0;
  for (;;) {
    const int base = next_chunk(counter);
    if (base >= n) break;
    const int i = base + (threadIdx.x & 31);
    if (i < n) {
      double P[V];
#pragma unroll
      for (int k = 0; k < V; ++k) P[k] = Pin[(size_t)k * n + i];
      nsub[i] = chem_integrate<NSP>(th, P, dts[i], tol, maxsub, err);
#pragma unroll
      for (int k = 0; k < V; ++k) Pout[(size_t)k * n + i] = P[k];
    }
  }
  if (err) atomicOr(errp, err);
}

// Grid of the persistent launches: enough resident warps to fill every SM.
template <class K>
static int chem_grid(K kernel, int items) {
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, CHEM_THREADS, 0);
  const int need = (items + CHEM_THREADS - 1) / CHEM_THREADS;
  int g = (nsm > 0 ? nsm : 1) * (occ > 0 ? occ : 1);
  return g < need ? g : (need > 0 ? need : 1);
}

// order/hist: work arrays of NE ints and NBUCKET unsigned (order null: cell order)
template <int NSP>
void chem_source(const Dev& d, const void* th, double tol, int maxsub, int* nsub, int* order, unsigned* hist,
                 unsigned* counter, cudaStream_t s) {
  if (order) {
    const int nb = (d.NE + 255) / 256;
    cudaMemsetAsync(hist, 0, sizeof(unsigned) * NBUCKET, s);
    k_chem_hist<<<nb, 256, 0, s>>>(nsub, d.NE, hist);
    k_chem_scan<<<1, NBUCKET, 0, s>>>(hist);
    k_chem_scatter<<<nb, 256, 0, s>>>(nsub, d.NE, hist, order);
  }
  const int grid = chem_grid(k_chem_source<NSP>, d.NE);
  cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
  k_chem_source<NSP><<<grid, CHEM_THREADS, 0, s>>>(d, *static_cast<const ThermoDev<NSP>*>(th), tol, maxsub, nsub,
                                                   order, counter);
}

template <int NSP>
void chem_list(const Dev& d, const void* th, double tol, int maxsub, int* nsub, const int* list,
               const unsigned* nlist, unsigned* counter, cudaStream_t s) {
  const int grid = chem_grid(k_chem_list<NSP>, d.NE);
  cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
  k_chem_list<NSP><<<grid, CHEM_THREADS, 0, s>>>(d, *static_cast<const ThermoDev<NSP>*>(th), tol, maxsub, nsub, list,
                                                 nlist, counter);
}

template <int NSP>
void chem_batch(const void* th, const double* P, const double* dt, int n, double* out, int* nsub, double tol,
                int maxsub, unsigned* counter, unsigned* errp, cudaStream_t s) {
  cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
  const int grid = chem_grid(k_chem_batch<NSP>, n);
  k_chem_batch<NSP><<<grid, CHEM_THREADS, 0, s>>>(*static_cast<const ThermoDev<NSP>*>(th), P, dt, n, out, nsub, tol,
                                                  maxsub, counter, errp);
}

#define RC_CHEM_INST(N)                                                                                  \
  template void chem_source<N>(const Dev&, const void*, double, int, int*, int*, unsigned*, unsigned*,   \
                               cudaStream_t);                                                            \
  template void chem_list<N>(const Dev&, const void*, double, int, int*, const int*, const unsigned*,      \
                             unsigned*, cudaStream_t);                                                   \
  template void chem_batch<N>(const void*, const double*, const double*, int, double*, int*, double, int, \
                              unsigned*, unsigned*, cudaStream_t);
RC_CHEM_INST(1)
RC_CHEM_INST(4)

}  // namespace rc
