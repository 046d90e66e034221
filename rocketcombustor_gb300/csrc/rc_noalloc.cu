// Residual norms without any device allocation (rc_residual_noalloc).
//
// Some hosts cannot call cudaMalloc: a host whose device arrays all come from
// its own allocator or from another runtime (for instance a Fortran code whose
// device copies of hWA/WA/VOL are managed by its CUDA Fortran or OpenACC
// runtime), or a long-running solver loop that must not allocate once set up,
// since cudaMalloc can synchronise the whole device.  This entry point takes
// the caller's device arrays and uses a fixed scratch area compiled into the
// library instead of memory from rc_init.
//
// The scratch is one file-scope __device__ array.  Every GPU that loads the
// library holds it (about 41 KB) until the process exits.  Host code may not
// use the array's name as a device address, so every call looks the address
// up with cudaGetSymbolAddress, with the caller's device and context current.
// The lookup is cheap next to the call's own stream synchronisation, and a
// per-call lookup stays right where a cached one would not: after
// cudaDeviceReset (the module is loaded again, possibly elsewhere) and under a
// driver-API context that is not the device's primary one.
//
// Sums use the same fixed-shape block decomposition as rc_residual, so the
// results are deterministic run to run.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "rc_gpu.h"

namespace {

constexpr int NA_BLOCKS = 304;                   // blocks of the partial-sum pass
constexpr int NA_THREADS = 256;
constexpr int NA_SLOTS = RC_NOALLOC_MAX_NVAR + 1; // NVar sums + max(WA(1,:))

// [partials: NA_SLOTS x NA_BLOCKS | results: NA_SLOTS]
static __device__ __align__(256) double g_noalloc_scratch[NA_SLOTS * NA_BLOCKS + NA_SLOTS];

__device__ __forceinline__ double dmax(double a, double b) { return (b > a) ? b : a; }

// Partial sums of vol*|hWA(k,:)| and max WA(1,:) over one contiguous chunk of
// cells per block; hWA, WA in the Fortran (NVar, NE) layout.
__global__ void __launch_bounds__(NA_THREADS) k_na_partial(const double* __restrict__ hWA,
                                                           const double* __restrict__ WA,
                                                           const double* __restrict__ vol, int NE, int V,
                                                           double* scratch) {
  __shared__ double sh[NA_THREADS];
  const int per = (NE + NA_BLOCKS - 1) / NA_BLOCKS;
  const int lo = blockIdx.x * per, hi = min(NE, lo + per);
  for (int k = 0; k <= V; ++k) {
    double a = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += NA_THREADS)
      a = (k == V) ? dmax(a, WA[(size_t)i * V]) : a + vol[i] * fabs(hWA[(size_t)i * V + k]);
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int w = NA_THREADS / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w)
        sh[threadIdx.x] = (k == V) ? dmax(sh[threadIdx.x], sh[threadIdx.x + w]) : sh[threadIdx.x] + sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) scratch[k * NA_BLOCKS + blockIdx.x] = sh[0];
    __syncthreads();
  }
}

__global__ void k_na_final(int V, double total_volume, double* scratch) {
  const int k = threadIdx.x;
  if (k > V) return;
  double a = 0.0;
  for (int b = 0; b < NA_BLOCKS; ++b)
    a = (k == V) ? dmax(a, scratch[k * NA_BLOCKS + b]) : a + scratch[k * NA_BLOCKS + b];
  scratch[NA_SLOTS * NA_BLOCKS + k] = (k == V) ? a : a / total_volume;
}

int fail(int code, const std::string& msg) {
  std::fprintf(stderr, "rc_residual_noalloc: %s\n", msg.c_str());
  return code;
}

// Device address of the scratch array in the context current on this thread.
int scratch_in_current_context(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) return fail(RC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  *out = static_cast<double*>(p);
  return RC_OK;
}

}  // namespace

extern "C" {

int rc_residual_noalloc(const double* d_hWA, const double* d_WA, const double* d_VOL, int NE, int NVar,
                        double total_volume, void* cuda_stream, double* res, double* romax) {
  if (!d_hWA || !d_WA || !d_VOL || !res || !romax) return fail(RC_ERR_ARG, "null pointer argument");
  if (NE < 1) return fail(RC_ERR_ARG, "NE must be at least 1");
  if (NVar < 1 || NVar > RC_NOALLOC_MAX_NVAR)
    return fail(RC_ERR_ARG, "NVar " + std::to_string(NVar) + " is outside 1.." + std::to_string(RC_NOALLOC_MAX_NVAR) +
                                " (RC_NOALLOC_MAX_NVAR, the size of the built-in scratch)");
  double* scratch = nullptr;
  int st = scratch_in_current_context(&scratch);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  k_na_partial<<<NA_BLOCKS, NA_THREADS, 0, s>>>(d_hWA, d_WA, d_VOL, NE, NVar, scratch);
  k_na_final<<<1, 32, 0, s>>>(NVar, total_volume, scratch);
  cudaError_t e = cudaGetLastError();
  double h[NA_SLOTS];
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h, scratch + NA_SLOTS * NA_BLOCKS, sizeof(double) * (NVar + 1), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(RC_ERR_CUDA, cudaGetErrorString(e));
  for (int k = 0; k < NVar; ++k) res[k] = h[k];
  *romax = h[NVar];
  return RC_OK;
}

}  // extern "C"
