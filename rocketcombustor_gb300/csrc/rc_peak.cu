// FP64 instruction rate of the current GPU (rc_fp64_rate).
//
// The plain FP64 path is built without FMA contraction, so its arithmetic is
// DADD and DMUL; on this part those run on a narrow FP64 pipe, and the face
// and cell kernels are bound by it rather than by HBM.  This measures the
// pipe's rate so that the kernels' FP64 fraction has a measured denominator:
// every thread runs 8 independent chains of alternating DADD and DMUL, enough
// warps on every SM to keep the pipe busy, timed with CUDA events.
#include <cuda_runtime.h>

#include "rc_gpu.h"

namespace {

constexpr int PK_CHAINS = 8, PK_THREADS = 256, PK_BLOCKS_PER_SM = 8;

__global__ void __launch_bounds__(PK_THREADS) k_fp64_rate(int iters, double a, double b, double* out) {
  double x[PK_CHAINS];
#pragma unroll
  for (int c = 0; c < PK_CHAINS; ++c) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) {
      x[c] = x[c] * a;  // a = 1 - 2^-30, b = 2^-31: stays near 1, never subnormal
      x[c] = x[c] + b;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < PK_CHAINS; ++c) s += x[c];
  if (s == -1.0) out[blockIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

extern "C" int rc_fp64_rate(void* cuda_stream, int iters, double* ops_per_s, double* seconds) {
  if (!ops_per_s || iters < 1) return RC_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return RC_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const int blocks = nsm * PK_BLOCKS_PER_SM;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = RC_OK;
  if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess) return RC_ERR_CUDA;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) st = RC_ERR_CUDA;
  const double a = 1.0 - 1.0 / (1u << 30), b = 1.0 / (double)(1u << 31);
  if (st == RC_OK) {
    k_fp64_rate<<<blocks, PK_THREADS, 0, s>>>(iters / 4 + 1, a, b, out);  // warm-up
    cudaEventRecord(e0, s);
    k_fp64_rate<<<blocks, PK_THREADS, 0, s>>>(iters, a, b, out);
    cudaEventRecord(e1, s);
    float ms = 0.f;
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f)
      st = RC_ERR_CUDA;
    else {
      const double ops = 2.0 * PK_CHAINS * (double)iters * PK_THREADS * (double)blocks;
      *ops_per_s = ops / (ms * 1e-3);
      if (seconds) *seconds = ms * 1e-3;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return st;
}
