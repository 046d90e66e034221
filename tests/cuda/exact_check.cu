// Test program: rc::half_of and rc::plus_zero (0.5 * x and 0.0 + x done on
// the bit pattern, csrc/rc_div.cuh) against the FP64 multiply and add, bit
// for bit, on random bit patterns of every exponent (subnormals, the smallest
// normals, infinities and NaNs included) and on a list of edge values.
// Prints the counts; exits 1 on any difference (NaNs compare as NaN == NaN).
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "rc_div.cuh"

__device__ uint64_t mix(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}
__device__ bool same(double a, double b) {
  if (isnan(a) || isnan(b)) return isnan(a) && isnan(b);
  return __double_as_longlong(a) == __double_as_longlong(b);
}
__global__ void check(unsigned long long n, unsigned long long* bad, unsigned long long* slow) {
  const uint64_t edge[] = {0x0ULL, 0x8000000000000000ULL, 0x1ULL, 0x800fffffffffffffULL, 0x000fffffffffffffULL,
                           0x0010000000000000ULL, 0x8010000000000000ULL, 0x0020000000000000ULL,
                           0x001fffffffffffffULL, 0x7fefffffffffffffULL, 0x7ff0000000000000ULL,
                           0xfff0000000000000ULL, 0x7ff8000000000000ULL, 0x3ff0000000000000ULL};
  unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long nb = 0, ns = 0;
  for (; i < n; i += stride) {
    uint64_t b = mix(i + 977);
    if (i < sizeof(edge) / sizeof(edge[0])) b = edge[i];
    else if ((i & 7) == 1) b = (b & 0x800fffffffffffffULL) | ((mix(i) % 4) << 52);  // exponent fields 0..3
    const double x = __longlong_as_double((long long)b);
    const volatile double half = 0.5, zero = 0.0;
    nb += !same(rc::half_of(x), half * x);
    nb += !same(rc::plus_zero(x), zero + x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    ns += !(e - 2u < 0x7fdu);
  }
  atomicAdd(bad, nb);
  atomicAdd(slow, ns);
}
int main(int argc, char** argv) {
  const unsigned long long n = argc > 1 ? strtoull(argv[1], nullptr, 10) : (1ULL << 28);
  unsigned long long* c = nullptr;
  if (cudaMalloc(&c, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemset(c, 0, 2 * sizeof(unsigned long long));
  check<<<152 * 8, 256>>>(n, c, c + 1);
  unsigned long long h[2] = {0, 0};
  const cudaError_t e = cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  printf("status %s samples %llu multiply-path %llu mismatches %llu\n", cudaGetErrorString(e), n, h[1], h[0]);
  return (e != cudaSuccess || h[0] != 0) ? 1 : 0;
}
