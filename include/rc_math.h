// Portable FP64 exp, log and pow with identical results on the host (C++) and
// on the GPU (CUDA).
//
// The reference evaluates exp/log/pow through the host libm.  Two libms
// (glibc on the CPU, the CUDA math library on the GPU) differ by an ulp here
// and there, and the steady iteration can amplify such differences: the
// explicit, clipped chemical source of a nearly depleted species multiplies
// them at every iteration.  Every FP64 hot-path evaluation of exp/log/pow, on
// the CPU and on the GPU, therefore goes through these functions.  They use
// only IEEE-754 +, -, *, integer operations on the bit patterns, table reads
// and explicitly fused multiply-adds (correctly rounded on both sides:
// std::fma / __fma_rn), so one input gives one output everywhere; exp and log
// are within 1 ulp of the exact values (about 0.5 ulp over most of the range)
// and tests/test_math.py checks them against the host libm.
//
// Methods: the table-driven reductions of P. T. P. Tang ("Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989; "... of the logarithm function", ACM TOMS
// 16(4), 1990), restated with FMAs and tables generated by tests/test_math.py
// in exact decimal arithmetic:
//   exp(x): x = (128 m + j) ln2/128 + r with |r| <= ln2/256 (j = 0..127; the
//           integer 128 m + j comes from the shifted sum x*128/ln2 + 1.5*2^52,
//           r from a two-constant reduction whose first step is exact);
//           exp(x) = 2^m * 2^(j/128) * e^r with 2^(j/128) as a lead + trail
//           pair from the table and e^r - 1 by its Taylor polynomial of
//           degree 5.
//   log(x): x = 2^e z with z in [1 - 2^-9, 2 - 2^-8), split by integer
//           arithmetic on the bit pattern; seven bits of z pick a centre
//           c = 1 + j/128 with tabulated invc = RN(1/c) and -log(invc) (lead
//           + trail); log x = e ln2 - log(invc) + log1p(z invc - 1), with
//           |z invc - 1| <= 2^-8 and log1p by its Taylor polynomial of degree
//           7; the leading sum is formed without rounding error.
//   pow(x,y), x > 0: exp(y log x) with the rounding error of y*log(x) carried
//           to first order.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define RCM_HD __host__ __device__ __forceinline__
#else
#define RCM_HD inline
#endif

namespace rcm {

RCM_HD double fma_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
RCM_HD int64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
RCM_HD double from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// Reduction constants (generated in exact decimal arithmetic):
// INV_LN2_128 = RN(128/ln2); ln2/128 = LN2_128_HI + LN2_128_LO; ln2 = LN2_HI42 +
// LN2_LO42 with LN2_HI42 a multiple of 2^-42 (so that e*LN2_HI42 is exact for
// |e| < 2^11).
constexpr double INV_LN2_128 = 0x1.71547652b82fep+7;
constexpr double LN2_128_HI = 0x1.62e42fefa39efp-8;
constexpr double LN2_128_LO = 0x1.abc9e3b39803fp-63;
constexpr double LN2_HI42 = 0x1.62e42fefa3800p-1;
constexpr double LN2_LO42 = 0x1.ef35793c76730p-45;
// 1.5 * 2^52: adding it to |t| < 2^51 rounds t to an integer held in the low
// bits of the sum
constexpr double SHIFT = 0x1.8p+52;

// 2^k for integer k with a normal result
RCM_HD double pow2i(int k) { return from_bits((int64_t)(k + 1023) << 52); }

// Range and special-value tests compare bit patterns (integer operations):
// for non-negative doubles the integer order of the patterns is the
// floating-point order.
constexpr int64_t ABS_MASK = 0x7fffffffffffffffLL;
constexpr int64_t INF_BITS = 0x7ff0000000000000LL;
constexpr int64_t EXP_HI_BITS = 0x40862e42fefa39efLL;  // 709.782712893384
constexpr int64_t EXP_LO_BITS = 0x40874910d52d3052LL;  // 745.1332191019412
constexpr int64_t LOG_OFF = 0x3feff00000000000LL;      // 1 - 2^-9

// 2^(j/128), j = 0..127, as lead RN(2^(j/128)) and trail RN(2^(j/128) - lead)
#define RCM_EXP_TAB_VALUES \
  { \
    0x1.0000000000000p+0, 0x0.0p+0, \
    0x1.0163da9fb3335p+0, 0x1.b61299ab8cdb7p-54, \
    0x1.02c9a3e778061p+0, -0x1.19083535b085dp-56, \
    0x1.04315e86e7f85p+0, -0x1.0a31c1977c96ep-54, \
    0x1.059b0d3158574p+0, 0x1.d73e2a475b465p-55, \
    0x1.0706b29ddf6dep+0, -0x1.c91dfe2b13c27p-55, \
    0x1.0874518759bc8p+0, 0x1.186be4bb284ffp-57, \
    0x1.09e3ecac6f383p+0, 0x1.1487818316136p-54, \
    0x1.0b5586cf9890fp+0, 0x1.8a62e4adc610bp-54, \
    0x1.0cc922b7247f7p+0, 0x1.01edc16e24f71p-54, \
    0x1.0e3ec32d3d1a2p+0, 0x1.03a1727c57b53p-59, \
    0x1.0fb66affed31bp+0, -0x1.b9bedc44ebd7bp-57, \
    0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54, \
    0x1.12abdc06c31ccp+0, -0x1.1b514b36ca5c7p-58, \
    0x1.1429aaea92de0p+0, -0x1.32fbf9af1369ep-54, \
    0x1.15a98c8a58e51p+0, 0x1.2406ab9eeab0ap-55, \
    0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55, \
    0x1.18af9388c8deap+0, -0x1.11023d1970f6cp-54, \
    0x1.1a35beb6fcb75p+0, 0x1.e5b4c7b4968e4p-55, \
    0x1.1bbe084045cd4p+0, -0x1.95386352ef607p-54, \
    0x1.1d4873168b9aap+0, 0x1.e016e00a2643cp-54, \
    0x1.1ed5022fcd91dp+0, -0x1.1df98027bb78cp-54, \
    0x1.2063b88628cd6p+0, 0x1.dc775814a8495p-55, \
    0x1.21f49917ddc96p+0, 0x1.2a97e9494a5eep-55, \
    0x1.2387a6e756238p+0, 0x1.9b07eb6c70573p-54, \
    0x1.251ce4fb2a63fp+0, 0x1.ac155bef4f4a4p-55, \
    0x1.26b4565e27cddp+0, 0x1.2bd339940e9d9p-55, \
    0x1.284dfe1f56381p+0, -0x1.a4c3a8c3f0d7ep-54, \
    0x1.29e9df51fdee1p+0, 0x1.612e8afad1255p-55, \
    0x1.2b87fd0dad990p+0, -0x1.10adcd6381aa4p-59, \
    0x1.2d285a6e4030bp+0, 0x1.0024754db41d5p-54, \
    0x1.2ecafa93e2f56p+0, 0x1.1ca0f45d52383p-56, \
    0x1.306fe0a31b715p+0, 0x1.6f46ad23182e4p-55, \
    0x1.32170fc4cd831p+0, 0x1.a9ce78e18047cp-55, \
    0x1.33c08b26416ffp+0, 0x1.32721843659a6p-54, \
    0x1.356c55f929ff1p+0, -0x1.b5cee5c4e4628p-55, \
    0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54, \
    0x1.38cae6d05d866p+0, -0x1.e958d3c9904bdp-54, \
    0x1.3a7db34e59ff7p+0, -0x1.5e436d661f5e3p-56, \
    0x1.3c32dc313a8e5p+0, -0x1.efff8375d29c3p-54, \
    0x1.3dea64c123422p+0, 0x1.ada0911f09ebcp-55, \
    0x1.3fa4504ac801cp+0, -0x1.7d023f956f9f3p-54, \
    0x1.4160a21f72e2ap+0, -0x1.ef3691c309278p-58, \
    0x1.431f5d950a897p+0, -0x1.1c7dde35f7999p-55, \
    0x1.44e086061892dp+0, 0x1.89b7a04ef80d0p-59, \
    0x1.46a41ed1d0057p+0, 0x1.c944bd1648a76p-54, \
    0x1.486a2b5c13cd0p+0, 0x1.3c1a3b69062f0p-56, \
    0x1.4a32af0d7d3dep+0, 0x1.9cb62f3d1be56p-54, \
    0x1.4bfdad5362a27p+0, 0x1.d4397afec42e2p-56, \
    0x1.4dcb299fddd0dp+0, 0x1.8ecdbbc6a7833p-54, \
    0x1.4f9b2769d2ca7p+0, -0x1.4b309d25957e3p-54, \
    0x1.516daa2cf6642p+0, -0x1.f768569bd93efp-55, \
    0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55, \
    0x1.551a4ca5d920fp+0, -0x1.d689cefede59bp-55, \
    0x1.56f4736b527dap+0, 0x1.9bb2c011d93adp-54, \
    0x1.58d12d497c7fdp+0, 0x1.295e15b9a1de8p-55, \
    0x1.5ab07dd485429p+0, 0x1.6324c054647adp-54, \
    0x1.5c9268a5946b7p+0, 0x1.c4b1b816986a2p-60, \
    0x1.5e76f15ad2148p+0, 0x1.ba6f93080e65ep-54, \
    0x1.605e1b976dc09p+0, -0x1.3e2429b56de47p-54, \
    0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54, \
    0x1.6434634ccc320p+0, -0x1.c483c759d8933p-55, \
    0x1.6623882552225p+0, -0x1.bb60987591c34p-54, \
    0x1.68155d44ca973p+0, 0x1.038ae44f73e65p-57, \
    0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54, \
    0x1.6c012750bdabfp+0, -0x1.2895667ff0b0dp-56, \
    0x1.6dfb23c651a2fp+0, -0x1.bbe3a683c88abp-57, \
    0x1.6ff7df9519484p+0, -0x1.83c0f25860ef6p-55, \
    0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55, \
    0x1.73f9a48a58174p+0, -0x1.0a8d96c65d53cp-54, \
    0x1.75feb564267c9p+0, -0x1.0245957316dd3p-54, \
    0x1.780694fde5d3fp+0, 0x1.866b80a02162dp-54, \
    0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55, \
    0x1.7c1ed0130c132p+0, 0x1.f124cd1164dd6p-54, \
    0x1.7e2f336cf4e62p+0, 0x1.05d02ba15797ep-56, \
    0x1.80427543e1a12p+0, -0x1.27c86626d972bp-54, \
    0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54, \
    0x1.8471a4623c7adp+0, -0x1.8d684a341cdfbp-55, \
    0x1.868d99b4492edp+0, -0x1.fc6f89bd4f6bap-54, \
    0x1.88ac7d98a6699p+0, 0x1.994c2f37cb53ap-54, \
    0x1.8ace5422aa0dbp+0, 0x1.6e9f156864b27p-54, \
    0x1.8cf3216b5448cp+0, -0x1.0d55e32e9e3aap-56, \
    0x1.8f1ae99157736p+0, 0x1.5cc13a2e3976cp-55, \
    0x1.9145b0b91ffc6p+0, -0x1.dd6792e582524p-54, \
    0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57, \
    0x1.95a44cbc8520fp+0, -0x1.64b7c96a5f039p-56, \
    0x1.97d829fde4e50p+0, -0x1.d185b7c1b85d1p-54, \
    0x1.9a0f170ca07bap+0, -0x1.173bd91cee632p-54, \
    0x1.9c49182a3f090p+0, 0x1.c7c46b071f2bep-56, \
    0x1.9e86319e32323p+0, 0x1.824ca78e64c6ep-56, \
    0x1.a0c667b5de565p+0, -0x1.359495d1cd533p-54, \
    0x1.a309bec4a2d33p+0, 0x1.6305c7ddc36abp-54, \
    0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54, \
    0x1.a799e1330b358p+0, 0x1.bcb7ecac563c7p-54, \
    0x1.a9e6b5579fdbfp+0, 0x1.0fac90ef7fd31p-54, \
    0x1.ac36bbfd3f37ap+0, -0x1.f9234cae76cd0p-55, \
    0x1.ae89f995ad3adp+0, 0x1.7a1cd345dcc81p-54, \
    0x1.b0e07298db666p+0, -0x1.bdef54c80e425p-54, \
    0x1.b33a2b84f15fbp+0, -0x1.2805e3084d708p-57, \
    0x1.b59728de5593ap+0, -0x1.c71dfbbba6de3p-54, \
    0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56, \
    0x1.ba5b030a1064ap+0, -0x1.efcd30e54292ep-54, \
    0x1.bcc1e904bc1d2p+0, 0x1.23dd07a2d9e84p-55, \
    0x1.bf2c25bd71e09p+0, -0x1.efdca3f6b9c73p-54, \
    0x1.c199bdd85529cp+0, 0x1.11065895048ddp-55, \
    0x1.c40ab5fffd07ap+0, 0x1.b4537e083c60ap-54, \
    0x1.c67f12e57d14bp+0, 0x1.2884dff483cadp-54, \
    0x1.c8f6d9406e7b5p+0, 0x1.1acbc48805c44p-56, \
    0x1.cb720dcef9069p+0, 0x1.503cbd1e949dbp-56, \
    0x1.cdf0b555dc3fap+0, -0x1.dd83b53829d72p-55, \
    0x1.d072d4a07897cp+0, -0x1.cbc3743797a9cp-54, \
    0x1.d2f87080d89f2p+0, -0x1.d487b719d8578p-54, \
    0x1.d5818dcfba487p+0, 0x1.2ed02d75b3707p-55, \
    0x1.d80e316c98398p+0, -0x1.11ec18beddfe8p-54, \
    0x1.da9e603db3285p+0, 0x1.c2300696db532p-54, \
    0x1.dd321f301b460p+0, 0x1.2da5778f018c3p-54, \
    0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54, \
    0x1.e264614f5a129p+0, -0x1.7b627817a1496p-54, \
    0x1.e502ee78b3ff6p+0, 0x1.39e8980a9cc8fp-55, \
    0x1.e7a51fbc74c83p+0, 0x1.2d522ca0c8de2p-54, \
    0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54, \
    0x1.ecf482d8e67f1p+0, -0x1.c93f3b411ad8cp-54, \
    0x1.efa1bee615a27p+0, 0x1.dc7f486a4b6b0p-54, \
    0x1.f252b376bba97p+0, 0x1.3a1a5bf0d8e43p-54, \
    0x1.f50765b6e4540p+0, 0x1.9d3e12dd8a18bp-54, \
    0x1.f7bfdad9cbe14p+0, -0x1.dbb12d006350ap-54, \
    0x1.fa7c1819e90d8p+0, 0x1.74853f3a5931ep-55, \
    0x1.fd3c22b8f71f1p+0, 0x1.2eb74966579e7p-57, \
  }

// For log: per interval j of the reduced argument (centre c = 1 + j/128; c = 1
// for j = 0): invc = RN(1/c), then -log(invc) as lead (a multiple of 2^-42)
// and trail; the fourth double pads a row to 32 bytes.
#define RCM_LOG_TAB_VALUES \
  { \
    0x1.0000000000000p+0, 0x0.0p+0, 0x0.0p+0, 0x0.0p+0, \
    0x1.fc07f01fc07f0p-1, 0x1.fe02a6b100000p-8, 0x1.9e63f0dda40e4p-46, 0x0.0p+0, \
    0x1.f81f81f81f820p-1, 0x1.fc0a8b0fc0000p-7, 0x1.e1e7cf6d3a69cp-50, 0x0.0p+0, \
    0x1.f44659e4a4271p-1, 0x1.7b91b07d60000p-6, -0x1.3b685b602ace4p-44, 0x0.0p+0, \
    0x1.f07c1f07c1f08p-1, 0x1.f829b0e780000p-6, 0x1.97c267c7e09e4p-45, 0x0.0p+0, \
    0x1.ecc07b301ecc0p-1, 0x1.39e87b9fe8000p-5, 0x1.eb3d480ad9015p-44, 0x0.0p+0, \
    0x1.e9131abf0b767p-1, 0x1.77458f6330000p-5, -0x1.1807ce586af09p-44, 0x0.0p+0, \
    0x1.e573ac901e574p-1, 0x1.b42dd71198000p-5, -0x1.c8d7ae5d6704cp-46, 0x0.0p+0, \
    0x1.e1e1e1e1e1e1ep-1, 0x1.f0a30c0118000p-5, -0x1.d579e83368e91p-45, 0x0.0p+0, \
    0x1.de5d6e3f8868ap-1, 0x1.16536eea38000p-4, -0x1.472de768fa309p-46, 0x0.0p+0, \
    0x1.dae6076b981dbp-1, 0x1.341d7961bc000p-4, 0x1.1cfb299837610p-44, 0x0.0p+0, \
    0x1.d77b654b82c34p-1, 0x1.51b073f060000p-4, 0x1.83ba9278e686ap-44, 0x0.0p+0, \
    0x1.d41d41d41d41dp-1, 0x1.6f0d28ae58000p-4, -0x1.4b2241b664613p-44, 0x0.0p+0, \
    0x1.d0cb58f6ec074p-1, 0x1.8c345d6318000p-4, 0x1.b22b5acb42a66p-44, 0x0.0p+0, \
    0x1.cd85689039b0bp-1, 0x1.a926d3a4ac000p-4, 0x1.561c50bd22a9cp-44, 0x0.0p+0, \
    0x1.ca4b3055ee191p-1, 0x1.c5e548f5bc000p-4, 0x1.d0c97585fbe06p-46, 0x0.0p+0, \
    0x1.c71c71c71c71cp-1, 0x1.e27076e2b0000p-4, -0x1.a2c2c2af0003cp-45, 0x0.0p+0, \
    0x1.c3f8f01c3f8f0p-1, 0x1.fec9131dc0000p-4, -0x1.54455d1ae6607p-44, 0x0.0p+0, \
    0x1.c0e070381c0e0p-1, 0x1.0d77e7cd08000p-3, 0x1.cb6cd2ee2f482p-44, 0x0.0p+0, \
    0x1.bdd2b899406f7p-1, 0x1.1b72ad52f6000p-3, 0x1.e86041811a396p-45, 0x0.0p+0, \
    0x1.bacf914c1bad0p-1, 0x1.29552f8200000p-3, -0x1.5bd67f4471dfcp-44, 0x0.0p+0, \
    0x1.b7d6c3dda338bp-1, 0x1.371fc201e8000p-3, 0x1.eea079b2d8abcp-44, 0x0.0p+0, \
    0x1.b4e81b4e81b4fp-1, 0x1.44d2b6ccb8000p-3, -0x1.71f416135783cp-46, 0x0.0p+0, \
    0x1.b2036406c80d9p-1, 0x1.526e5e3a1c000p-3, -0x1.790aa37fc5238p-44, 0x0.0p+0, \
    0x1.af286bca1af28p-1, 0x1.5ff3070a7a000p-3, -0x1.8546f183bebf2p-44, 0x0.0p+0, \
    0x1.ac5701ac5701bp-1, 0x1.6d60fe719e000p-3, -0x1.bc91557134767p-44, 0x0.0p+0, \
    0x1.a98ef606a63bep-1, 0x1.7ab890210e000p-3, -0x1.be51072534a58p-45, 0x0.0p+0, \
    0x1.a6d01a6d01a6dp-1, 0x1.87fa06520c000p-3, 0x1.22130401202fcp-44, 0x0.0p+0, \
    0x1.a41a41a41a41ap-1, 0x1.9525a9cf46000p-3, -0x1.294937d9f158fp-44, 0x0.0p+0, \
    0x1.a16d3f97a4b02p-1, 0x1.a23bc1fe2c000p-3, -0x1.53d6d91dc9f0bp-44, 0x0.0p+0, \
    0x1.9ec8e951033d9p-1, 0x1.af3c94e80c000p-3, -0x1.92e633fcd9066p-52, 0x0.0p+0, \
    0x1.9c2d14ee4a102p-1, 0x1.bc286742d8000p-3, 0x1.9a873f39d121cp-44, 0x0.0p+0, \
    0x1.999999999999ap-1, 0x1.c8ff7c79aa000p-3, -0x1.7814f689f8434p-45, 0x0.0p+0, \
    0x1.970e4f80cb872p-1, 0x1.d5c216b4fc000p-3, -0x1.1b0d1bbca681bp-45, 0x0.0p+0, \
    0x1.948b0fcd6e9e0p-1, 0x1.e27076e2b0000p-3, -0x1.a302c2af0003cp-44, 0x0.0p+0, \
    0x1.920fb49d0e229p-1, 0x1.ef0adcbdc6000p-3, -0x1.b2a179c86af24p-45, 0x0.0p+0, \
    0x1.8f9c18f9c18fap-1, 0x1.fb9186d5e4000p-3, -0x1.d6b2aab993c87p-47, 0x0.0p+0, \
    0x1.8d3018d3018d3p-1, 0x1.0402594b4d000p-2, 0x1.037b89ef42d7fp-48, 0x0.0p+0, \
    0x1.8acb90f6bf3aap-1, 0x1.0a324e2739000p-2, 0x1.c4dee7ef4030ep-47, 0x0.0p+0, \
    0x1.886e5f0abb04ap-1, 0x1.1058bf9ae5000p-2, -0x1.4affd817d52cdp-44, 0x0.0p+0, \
    0x1.8618618618618p-1, 0x1.1675cababa000p-2, 0x1.83c0e731f55c4p-44, 0x0.0p+0, \
    0x1.83c977ab2beddp-1, 0x1.1c898c169a000p-2, -0x1.81260e5c62affp-44, 0x0.0p+0, \
    0x1.8181818181818p-1, 0x1.22941fbcf8000p-2, -0x1.a6876f5eb0963p-44, 0x0.0p+0, \
    0x1.7f405fd017f40p-1, 0x1.2895a13de8000p-2, 0x1.a917ad24c13f0p-44, 0x0.0p+0, \
    0x1.7d05f417d05f4p-1, 0x1.2e8e2bae12000p-2, -0x1.6791e99b72bd8p-45, 0x0.0p+0, \
    0x1.7ad2208e0ecc3p-1, 0x1.347dd9a988000p-2, -0x1.5522dd4c58092p-45, 0x0.0p+0, \
    0x1.78a4c8178a4c8p-1, 0x1.3a64c55694000p-2, 0x1.7a81cbcd735d0p-44, 0x0.0p+0, \
    0x1.767dce434a9b1p-1, 0x1.404308686a000p-2, 0x1.f8f043049f7d3p-44, 0x0.0p+0, \
    0x1.745d1745d1746p-1, 0x1.4618bc21c6000p-2, -0x1.3e02f484c84ccp-46, 0x0.0p+0, \
    0x1.724287f46debcp-1, 0x1.4be5f95778000p-2, -0x1.d7c52cd9ad824p-44, 0x0.0p+0, \
    0x1.702e05c0b8170p-1, 0x1.51aad872e0000p-2, -0x1.f49d8db0a7cc1p-44, 0x0.0p+0, \
    0x1.6e1f76b4337c7p-1, 0x1.5767717456000p-2, -0x1.650fd9524d7cap-44, 0x0.0p+0, \
    0x1.6c16c16c16c17p-1, 0x1.5d1bdbf581000p-2, -0x1.8d97dc9c7c238p-44, 0x0.0p+0, \
    0x1.6a13cd1537290p-1, 0x1.62c82f2b9c000p-2, 0x1.e57bdbd7c8a98p-44, 0x0.0p+0, \
    0x1.6816816816817p-1, 0x1.686c81e9b1000p-2, 0x1.2b5710af84054p-44, 0x0.0p+0, \
    0x1.661ec6a5122f9p-1, 0x1.6e08eaa2ba000p-2, 0x1.e390139318d71p-46, 0x0.0p+0, \
    0x1.642c8590b2164p-1, 0x1.739d7f6bbd000p-2, 0x1.c7389314feb50p-52, 0x0.0p+0, \
    0x1.623fa77016240p-1, 0x1.792a55fdd4000p-2, 0x1.e85f057691feap-44, 0x0.0p+0, \
    0x1.6058160581606p-1, 0x1.7eaf83b82b000p-2, -0x1.f05a62d0c25adp-49, 0x0.0p+0, \
    0x1.5e75bb8d015e7p-1, 0x1.842d1da1e9000p-2, -0x1.39eab13ae687cp-44, 0x0.0p+0, \
    0x1.5c9882b931057p-1, 0x1.89a3386c14000p-2, 0x1.2d92d38c40882p-45, 0x0.0p+0, \
    0x1.5ac056b015ac0p-1, 0x1.8f11e87366000p-2, 0x1.643f0bb4eab4cp-45, 0x0.0p+0, \
    0x1.58ed2308158edp-1, 0x1.947941c211000p-2, 0x1.bec89337451f4p-44, 0x0.0p+0, \
    0x1.571ed3c506b3ap-1, 0x1.99d958117e000p-2, 0x1.1367525dd88f0p-47, 0x0.0p+0, \
    0x1.5555555555555p-1, 0x1.9f323ecbfa000p-2, -0x1.ecc3525ca2643p-44, 0x0.0p+0, \
    0x1.5390948f40febp-1, 0x1.a484090e5c000p-2, -0x1.3da000d6523c5p-44, 0x0.0p+0, \
    0x1.51d07eae2f815p-1, 0x1.a9cec9a9a1000p-2, -0x1.ed86adec02b43p-44, 0x0.0p+0, \
    0x1.5015015015015p-1, 0x1.af12932478000p-2, -0x1.e53ab31eed7a9p-44, 0x0.0p+0, \
    0x1.4e5e0a72f0539p-1, 0x1.b44f77bcc9000p-2, -0x1.38068224aa2cep-47, 0x0.0p+0, \
    0x1.4cab88725af6ep-1, 0x1.b985896931000p-2, 0x1.f9831f629f11ep-47, 0x0.0p+0, \
    0x1.4afd6a052bf5bp-1, 0x1.beb4d9da72000p-2, -0x1.21641e78b2151p-44, 0x0.0p+0, \
    0x1.49539e3b2d067p-1, 0x1.c3dd7a7cdb000p-2, -0x1.5968261f5a42bp-45, 0x0.0p+0, \
    0x1.47ae147ae147bp-1, 0x1.c8ff7c79aa000p-2, -0x1.77acf689f8434p-44, 0x0.0p+0, \
    0x1.460cbc7f5cf9ap-1, 0x1.ce1af0b85f000p-2, 0x1.f5e9be95e5568p-45, 0x0.0p+0, \
    0x1.446f86562d9fbp-1, 0x1.d32fe7e00f000p-2, -0x1.0ab5884dcd050p-44, 0x0.0p+0, \
    0x1.42d6625d51f87p-1, 0x1.d83e7258a3000p-2, -0x1.83c75d48ba26dp-47, 0x0.0p+0, \
    0x1.4141414141414p-1, 0x1.dd46a04c1c000p-2, 0x1.283fb989a9274p-44, 0x0.0p+0, \
    0x1.3fb013fb013fbp-1, 0x1.e24881a7c7000p-2, -0x1.ecefa1385d356p-45, 0x0.0p+0, \
    0x1.3e22cbce4a902p-1, 0x1.e744261d68000p-2, 0x1.e25cdf68dbcf3p-44, 0x0.0p+0, \
    0x1.3c995a47babe7p-1, 0x1.ec399d2469000p-2, -0x1.9f865188d6065p-45, 0x0.0p+0, \
    0x1.3b13b13b13b14p-1, 0x1.f128f5faf0000p-2, 0x1.baecd720ec44cp-44, 0x0.0p+0, \
    0x1.3991c2c187f63p-1, 0x1.f6123fa703000p-2, -0x1.d4baaea4f0d25p-44, 0x0.0p+0, \
    0x1.3813813813814p-1, 0x1.faf588f78f000p-2, 0x1.8e9cd7d9f2754p-45, 0x0.0p+0, \
    0x1.3698df3de0748p-1, 0x1.ffd2e0857f000p-2, 0x1.25bd65f40d932p-44, 0x0.0p+0, \
    0x1.3521cfb2b78c1p-1, 0x1.02552a5a5d000p-1, 0x1.fe3d38d2bafddp-46, 0x0.0p+0, \
    0x1.33ae45b57bcb2p-1, 0x1.04bdf9da92800p-1, -0x1.2dce033eff74ep-45, 0x0.0p+0, \
    0x1.323e34a2b10bfp-1, 0x1.0723e5c1ce000p-1, -0x1.7e0b50d38edddp-46, 0x0.0p+0, \
    0x1.30d190130d190p-1, 0x1.0986f4f573800p-1, -0x1.6f937012b5806p-44, 0x0.0p+0, \
    0x1.2f684bda12f68p-1, 0x1.0be72e4252800p-1, 0x1.419b4c4bdd99fp-44, 0x0.0p+0, \
    0x1.2e025c04b8097p-1, 0x1.0e44985d1d000p-1, -0x1.ba038a8d10b4bp-44, 0x0.0p+0, \
    0x1.2c9fb4d812ca0p-1, 0x1.109f39e2d5000p-1, -0x1.b4c10e09b27a4p-44, 0x0.0p+0, \
    0x1.2b404ad012b40p-1, 0x1.12f719593f000p-1, -0x1.0cb3fb7398e0cp-47, 0x0.0p+0, \
    0x1.29e4129e4129ep-1, 0x1.154c3d2f4d800p-1, -0x1.0af338662e34dp-44, 0x0.0p+0, \
    0x1.288b01288b013p-1, 0x1.179eabbd89800p-1, 0x1.9ff1c60e6fa08p-45, 0x0.0p+0, \
    0x1.27350b8812735p-1, 0x1.19ee6b467c800p-1, 0x1.6ee05cbdd7782p-45, 0x0.0p+0, \
    0x1.25e22708092f1p-1, 0x1.1c3b81f714000p-1, -0x1.ed90b58389902p-44, 0x0.0p+0, \
    0x1.2492492492492p-1, 0x1.1e85f5e704000p-1, 0x1.a17bd8b34be7cp-46, 0x0.0p+0, \
    0x1.23456789abcdfp-1, 0x1.20cdcd192a800p-1, 0x1.b6caa81e87baep-44, 0x0.0p+0, \
    0x1.21fb78121fb78p-1, 0x1.23130d7bec000p-1, -0x1.7aba4392f1ba7p-46, 0x0.0p+0, \
    0x1.20b470c67c0d9p-1, 0x1.2555bce98f800p-1, -0x1.accfde292977ep-48, 0x0.0p+0, \
    0x1.1f7047dc11f70p-1, 0x1.2795e1289b000p-1, 0x1.1b6b783f3db97p-45, 0x0.0p+0, \
    0x1.1e2ef3b3fb874p-1, 0x1.29d37fec2b000p-1, 0x1.1680b9ad974bap-46, 0x0.0p+0, \
    0x1.1cf06ada2811dp-1, 0x1.2c0e9ed449000p-1, -0x1.74628563ce45dp-45, 0x0.0p+0, \
    0x1.1bb4a4046ed29p-1, 0x1.2e47436e40000p-1, 0x1.34212a10c3491p-44, 0x0.0p+0, \
    0x1.1a7b9611a7b96p-1, 0x1.307d7334f1000p-1, 0x1.7c7f6b2143eadp-46, 0x0.0p+0, \
    0x1.19453808ca29cp-1, 0x1.32b1339122000p-1, -0x1.4762fd54a4c27p-44, 0x0.0p+0, \
    0x1.1811811811812p-1, 0x1.34e289d9ce000p-1, 0x1.d22eeb92d885dp-45, 0x0.0p+0, \
    0x1.16e0689427379p-1, 0x1.37117b5474800p-1, -0x1.29808bf6deec9p-47, 0x0.0p+0, \
    0x1.15b1e5f75270dp-1, 0x1.393e0d3562800p-1, 0x1.0cd8e221301b7p-44, 0x0.0p+0, \
    0x1.1485f0e0acd3bp-1, 0x1.3b6844a000000p-1, -0x1.ee4738909f3d3p-44, 0x0.0p+0, \
    0x1.135c81135c811p-1, 0x1.3d9026a715800p-1, -0x1.04f7fbd9c2f53p-45, 0x0.0p+0, \
    0x1.12358e75d3033p-1, 0x1.3fb5b84d17000p-1, -0x1.79bd62c55f46bp-46, 0x0.0p+0, \
    0x1.1111111111111p-1, 0x1.41d8fe8467000p-1, 0x1.5742325e617a3p-44, 0x0.0p+0, \
    0x1.0fef010fef011p-1, 0x1.43f9fe2f9d000p-1, -0x1.98878d84649f1p-45, 0x0.0p+0, \
    0x1.0ecf56be69c90p-1, 0x1.4618bc21c6000p-1, -0x1.3dc2f484c84ccp-45, 0x0.0p+0, \
    0x1.0db20a88f4696p-1, 0x1.48353d1ea8800p-1, 0x1.bd5fabd176604p-46, 0x0.0p+0, \
    0x1.0c9714fbcda3bp-1, 0x1.4a4f85db04000p-1, -0x1.4575d840b8591p-45, 0x0.0p+0, \
    0x1.0b7e6ec259dc8p-1, 0x1.4c679afccf000p-1, -0x1.c71e971322ce8p-45, 0x0.0p+0, \
    0x1.0a6810a6810a7p-1, 0x1.4e7d811b75800p-1, 0x1.d7d4584c2b22cp-44, 0x0.0p+0, \
    0x1.0953f39010954p-1, 0x1.50913cc016800p-1, 0x1.accf2ce96c2d6p-47, 0x0.0p+0, \
    0x1.0842108421084p-1, 0x1.52a2d265bc800p-1, -0x1.2a68c41ba8752p-44, 0x0.0p+0, \
    0x1.073260a47f7c6p-1, 0x1.54b2467999800p-1, -0x1.b3c1755eba5e1p-44, 0x0.0p+0, \
    0x1.0624dd2f1a9fcp-1, 0x1.56bf9d5b3f000p-1, 0x1.cc888e310b9b2p-44, 0x0.0p+0, \
    0x1.05197f7d73404p-1, 0x1.58cadb5cd7800p-1, 0x1.895892f25d931p-45, 0x0.0p+0, \
    0x1.0410410410410p-1, 0x1.5ad404c35a000p-1, -0x1.a509acaab41fcp-46, 0x0.0p+0, \
    0x1.03091b51f5e1ap-1, 0x1.5cdb1dc6c1800p-1, -0x1.35ae12387451fp-46, 0x0.0p+0, \
    0x1.0204081020408p-1, 0x1.5ee02a9241800p-1, -0x1.8a6f29f6a02dcp-45, 0x0.0p+0, \
    0x1.0101010101010p-1, 0x1.60e32f4478800p-1, 0x1.b1d4f912b416ap-46, 0x0.0p+0, \
  }

// One copy of each table for host code and one in device memory for device
// code; the functions pick theirs at compile time.
alignas(16) static const double exp_tab_host[256] = RCM_EXP_TAB_VALUES;
alignas(32) static const double log_tab_host[512] = RCM_LOG_TAB_VALUES;
#ifdef __CUDACC__
alignas(16) static __device__ const double exp_tab_dev[256] = RCM_EXP_TAB_VALUES;
alignas(32) static __device__ const double log_tab_dev[512] = RCM_LOG_TAB_VALUES;
#endif

RCM_HD void exp_tab(int j, double& lead, double& trail) {
#ifdef __CUDA_ARCH__
  const double2 v = __ldg(reinterpret_cast<const double2*>(exp_tab_dev) + j);
  lead = v.x;
  trail = v.y;
#else
  lead = exp_tab_host[2 * j];
  trail = exp_tab_host[2 * j + 1];
#endif
}

RCM_HD void log_tab(int j, double& invc, double& lead, double& trail) {
#ifdef __CUDA_ARCH__
  const double2 a = __ldg(reinterpret_cast<const double2*>(log_tab_dev) + 2 * j);
  invc = a.x;
  lead = a.y;
  trail = __ldg(log_tab_dev + 4 * j + 2);
#else
  invc = log_tab_host[4 * j];
  lead = log_tab_host[4 * j + 1];
  trail = log_tab_host[4 * j + 2];
#endif
}

RCM_HD double exp(double x) {
  const int64_t b = bits(x);
  if ((b & ABS_MASK) > INF_BITS) return x;                 // NaN
  if (b > EXP_HI_BITS) return HUGE_VAL;                    // x > 709.782712893384
  if (b < 0 && (b & ABS_MASK) > EXP_LO_BITS) return 0.0;  // x < -745.1332191019412
  // x = (128 m + j) ln2/128 + r, |r| <= ln2/256 (to rounding)
  const double t = fma_(x, INV_LN2_128, SHIFT);
  const double kd = t - SHIFT;
  const int k = (int)(int32_t)(uint32_t)(uint64_t)bits(t);
  double r = fma_(-kd, LN2_128_HI, x);  // exact
  r = fma_(-kd, LN2_128_LO, r);
  // e^r - 1 = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120); the first omitted
  // term is below 2^-60
  const double r2 = r * r;
  double q = fma_(1.0 / 120.0, r, 1.0 / 24.0);
  q = fma_(q, r, 1.0 / 6.0);
  q = fma_(q, r, 0.5);
  const double p = fma_(r2, q, r);
  double th, tl;
  exp_tab(k & 127, th, tl);
  const double y = th + fma_(th, p, tl);  // 2^(j/128) e^r, in [0.99, 2)
  const int m = k >> 7;
  if (m >= -1022 && m <= 1023) return y * pow2i(m);
  const int m1 = m / 2;  // subnormal or near-overflow results: two exact factors
  return (y * pow2i(m1)) * pow2i(m - m1);
}

RCM_HD double log(double x) {
  int64_t b = bits(x);
  if ((b & ABS_MASK) > INF_BITS) return x;                                    // NaN
  if (b <= 0)                                                                 // x <= 0 (incl. -0)
    return (b & ABS_MASK) == 0 ? -HUGE_VAL : (x - x) / (x - x);
  if (b == INF_BITS) return x;
  int eadj = 0;
  if ((b >> 52) == 0) {  // subnormal: scale by 2^54 (exact)
    b = bits(x * 18014398509481984.0);
    eadj = -54;
  }
  // x = 2^e z with z in [1 - 2^-9, 2 - 2^-8); j = the 7 bits of z that select
  // the interval [c - 2^-8, c + 2^-8) around c = 1 + j/128 ([1 - 2^-9, 1 + 2^-8)
  // for j = 0)
  const int64_t tmp = b - LOG_OFF;
  const int e = (int)(tmp >> 52) + eadj;
  const int j = (int)((tmp >> 45) & 127);
  const double z = from_bits(b - (tmp & (int64_t)0xfff0000000000000ULL));
  double invc, lh, ll;
  log_tab(j, invc, lh, ll);
  // log x = e ln2 - log(invc) + log1p(r), r = z invc - 1, |r| <= 2^-8
  const double r = fma_(z, invc, -1.0);
  const double ed = (double)e;
  const double t1 = fma_(ed, LN2_HI42, lh);  // exact
  const double lo = fma_(ed, LN2_LO42, ll);
  // log1p(r) - r = r^2 (-1/2 + r/3 - r^2/4 + r^3/5 - r^4/6 + r^5/7); the first
  // omitted term is below 2^-67
  const double r2 = r * r;
  double q = fma_(1.0 / 7.0, r, -1.0 / 6.0);
  q = fma_(q, r, 1.0 / 5.0);
  q = fma_(q, r, -0.25);
  q = fma_(q, r, 1.0 / 3.0);
  q = fma_(q, r, -0.5);
  const double p = fma_(r2, q, lo);
  // t1 + r without rounding error (|t1| > |r| whenever t1 != 0): s + serr
  const double s = t1 + r;
  const double serr = (t1 - s) + r;
  return s + (serr + p);
}

// x > 0 (the reference only takes powers of positive quantities)
RCM_HD double pow(double x, double y) {
  const int64_t bx = bits(x), by = bits(y);
  if (bx == 0x3ff0000000000000LL || (by & ABS_MASK) == 0) return 1.0;  // x == 1 or y == 0
  if ((bx & ABS_MASK) == 0) return (by > 0 && (by & ABS_MASK) <= INF_BITS) ? 0.0 : HUGE_VAL;  // x == 0
  const double L = log(x);
  const double t = y * L;
  const double terr = fma_(y, L, -t);
  const double p = exp(t);
  return fma_(p, terr, p);
}

}  // namespace rcm
