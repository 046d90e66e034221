// Test program: rcm::exp, rcm::log and rcm::pow (include/rc_math.h) evaluated
// on the GPU and on the host CPU for the same pseudo-random arguments, compared
// bit for bit.  exp takes x in [-750, 712]; log takes positive doubles with
// random exponents (subnormals included) and arguments within 2^-6 of 1; pow
// takes x = 2^u, u in [-20, 12], and y in [-3, 3].  Prints the counts; exits 1
// on any bit difference.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rc_math.h"

__host__ __device__ uint64_t mix(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}
__host__ __device__ double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

__host__ __device__ void args(uint64_t i, double& xe, double& xl, double& xp, double& yp) {
  const uint64_t h1 = mix(3 * i + 1), h2 = mix(3 * i + 2), h3 = mix(3 * i + 3);
  xe = -750.0 + 1462.0 * unit(h1);
  if (i & 1) {
    const uint64_t e = (h2 >> 52) % 2046;  // 0 (subnormal) .. 2045
    xl = rcm::from_bits((int64_t)((e << 52) | (h2 & ((1ULL << 52) - 1))));
    if (xl == 0.0) xl = 1.0;
  } else {
    xl = 1.0 + (unit(h2) - 0.5) * (1.0 / 32.0);
  }
  xp = rcm::exp(0.6931471805599453 * (-20.0 + 32.0 * unit(h3)));
  yp = -3.0 + 6.0 * unit(mix(h3));
}

__global__ void run(unsigned long long n, double* out) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    double xe, xl, xp, yp;
    args(i, xe, xl, xp, yp);
    out[3 * i] = rcm::exp(xe);
    out[3 * i + 1] = rcm::log(xl);
    out[3 * i + 2] = rcm::pow(xp, yp);
  }
}

int main(int argc, char** argv) {
  const unsigned long long n = argc > 1 ? strtoull(argv[1], nullptr, 10) : (1ULL << 22);
  double* d = nullptr;
  if (cudaMalloc(&d, 3 * n * sizeof(double)) != cudaSuccess) return 2;
  run<<<152 * 8, 256>>>(n, d);
  std::vector<double> g(3 * n);
  const cudaError_t e = cudaMemcpy(g.data(), d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  unsigned long long bad[3] = {0, 0, 0};
  for (unsigned long long i = 0; i < n; ++i) {
    double xe, xl, xp, yp;
    args(i, xe, xl, xp, yp);
    const double h[3] = {rcm::exp(xe), rcm::log(xl), rcm::pow(xp, yp)};
    for (int k = 0; k < 3; ++k) bad[k] += rcm::bits(h[k]) != rcm::bits(g[3 * i + k]);
  }
  printf("status %s samples %llu mismatches exp %llu log %llu pow %llu\n", cudaGetErrorString(e), n, bad[0], bad[1],
         bad[2]);
  return (e != cudaSuccess || bad[0] + bad[1] + bad[2] != 0) ? 1 : 0;
}
