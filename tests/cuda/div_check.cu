// Test program: rc::div_rn (the sweeps' division with a precomputed reciprocal
// pair) against the IEEE FP64 division on random operands: exponents in
// [-450, 450] (so both the Markstein path and the IEEE fallback run), random
// mantissas, every fourth divisor with an all-ones mantissa tail, every eighth
// a power of two, every sixteenth numerator a signed zero.  Prints the counts;
// exits 1 on any bit difference.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "rc_div.cuh"

__device__ uint64_t mix(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}
__global__ void check(unsigned long long n, unsigned long long seed, unsigned long long* bad, unsigned long long* fast) {
  unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long nb = 0, nf = 0;
  for (; i < n; i += stride) {
    const uint64_t h1 = mix(i * 2 + seed), h2 = mix(i * 2 + 1 + seed * 7);
    const uint64_t ea = 1023 - 450 + (h1 >> 52) % 901, eb = 1023 - 450 + (h2 >> 52) % 901;
    const uint64_t ma = h1 & ((1ULL << 52) - 1);
    uint64_t mb = h2 & ((1ULL << 52) - 1);
    if ((i & 3) == 0) mb |= ((1ULL << 52) - 1) & ~((1ULL << ((h1 >> 3) % 20)) - 1);
    if ((i & 7) == 1) mb = 0;
    double a = __longlong_as_double((long long)((ea << 52) | ma | ((h1 & 1) << 63)));
    if ((i & 15) == 5) a = (h1 & 1) ? -0.0 : 0.0;
    const double b = __longlong_as_double((long long)((eb << 52) | mb | ((h2 & 2) << 62)));
    const rc::Recip y = rc::recip_of(b);
    const double q = rc::div_rn(a, b, y.h, y.l);
    nb += __double_as_longlong(q) != __double_as_longlong(a / b);
    nf += rc::div_rn_safe(a, b);
  }
  atomicAdd(bad, nb);
  atomicAdd(fast, nf);
}
int main(int argc, char** argv) {
  const unsigned long long n = argc > 1 ? strtoull(argv[1], nullptr, 10) : (1ULL << 28);
  unsigned long long* c = nullptr;
  if (cudaMalloc(&c, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemset(c, 0, 2 * sizeof(unsigned long long));
  check<<<152 * 8, 256>>>(n, 12345, c, c + 1);
  unsigned long long h[2] = {0, 0};
  const cudaError_t e = cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  printf("status %s samples %llu markstein %llu mismatches %llu\n", cudaGetErrorString(e), n, h[1], h[0]);
  return (e != cudaSuccess || h[0] != 0) ? 1 : 0;
}
