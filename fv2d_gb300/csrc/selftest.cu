// selftest.cu -- checks the integer-pipe binary64 routines of softfp.cuh bit
// for bit against the hardware instructions on this GPU: op 0 division,
// 1 square root, 2 comparisons, 3 fmax / fmin, 4 scalings by powers of two,
// 5 multiplication.
#include <cuda_runtime.h>

#include "../../include/fv2d_gpu.h"
#include "softfp.cuh"
#include "step_kernel.cuh"

namespace {

__device__ __forceinline__ uint64_t mix(uint64_t z) {  // SplitMix64 finaliser
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Operand of class `mode` from a 64-bit random word:
//  0: random significand, exponent in [-60, 60]      1: any bit pattern
//  2: significand with few set bits (exact quotients, ties, perfect squares)
//  3: exponent near the overflow/underflow limits
//  4: significand within 4096 ulps above or below a power of two (the
//     divisor's reciprocal word is then near 2^64 - 1 or near 0)
__device__ __forceinline__ double operand(uint64_t r, uint64_t r2, int mode) {
  uint64_t bits;
  switch (mode) {
    case 0: bits = (r & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 60 + (int)(r2 % 121)) << 52); break;
    case 1: bits = r; break;
    case 2: bits = (r & 0x800FF00000000000ull) | ((uint64_t)(1023 - 8 + (int)(r2 % 17)) << 52); break;
    case 3: {
      const int e = (r2 & 1) ? 1 + (int)(r2 % 40) : 2046 - (int)(r2 % 40);
      bits = (r & 0x800FFFFFFFFFFFFFull) | ((uint64_t)e << 52);
      break;
    }
    default: {
      const uint64_t small = r & 0xFFFull, frac = (r2 & 1) ? small : 0xFFFFFFFFFFFFFull - small;
      bits = (r & 0x8000000000000000ull) | frac | ((uint64_t)(1023 - 8 + (int)((r2 >> 1) % 17)) << 52);
    }
  }
  return __longlong_as_double((long long)bits);
}

__global__ void selftest_kernel(int op, uint64_t n, uint64_t seed, unsigned long long *bad, double *ex) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t r0 = mix(seed ^ (i * 4)), r1 = mix(seed ^ (i * 4 + 1)), r2 = mix(seed ^ (i * 4 + 2)),
                   r3 = mix(seed ^ (i * 4 + 3));
    const int mode = (int)((r3 >> 32) % 5);
    double a = operand(r0, r2, mode), b = operand(r1, r3 >> 8, mode);
    if (op == 0 && mode == 2 && (r3 & 4)) {  // a = b * k +- 1 ulp: quotients next to representable values
      const double k = operand(r2, r0, 2);
      a = b * k;
      a = __longlong_as_double(__double_as_longlong(a) + ((r3 & 8) ? 1 : -1));
    }
    if (op == 1 && mode == 2 && (r3 & 4)) {  // perfect squares +- 1 ulp
      a = b * b;
      a = __longlong_as_double(__double_as_longlong(a) + ((r3 & 8) ? 1 : ((r3 & 16) ? 0 : -1)));
    }
    if (((r3 >> 20) & 15) == 0) a = copysign(0.0, a);  // zero dividends / radicands
    if (((r3 >> 24) & 63) == 0) b = copysign(0.0, b);  // division by zero
    if (op >= 2 && ((r3 >> 30) & 3) == 0) b = a;  // equal operands
    if (op >= 2 && ((r3 >> 44) & 7) == 0) b = -a;  // opposite operands (incl. +0 / -0)
    namespace sf = fv2d::softfp;
    double h, s, h2 = 0.0, s2 = 0.0;
    if (op == 0) {  // single quotient, and a pair sharing the divisor
      h = a / b;
      s = sf::div_rn(a, b);
      const double c = ((r3 >> 56) & 3) == 0 ? 0.0 : operand(r2, r0, mode);
      const double2 q2 = sf::div2_rn(a, c, b);
      const double s1 = q2.x;
      s2 = q2.y;
      h2 = c / b;
      if (__double_as_longlong(s1) != __double_as_longlong(s) && !(s1 != s1 && s != s)) s2 = h2 + 1.0;
    } else if (op == 1) {
      a = fabs(a);
      h = sqrt(a);
      s = sf::sqrt_rn(a);
    } else if (op == 2) {  // comparisons, one bit each
      h = (double)((a > 0.0) | (a < 0.0) << 1 | (a >= 0.0) << 2 | (a <= 0.0) << 3 | (a < b) << 4 |
                   (fabs(a) < fabs(b)) << 5 | (a * b < 0.0) << 6 | (isnan(a) ? 1 : 0) << 7);
      s = (double)(sf::gt0(a) | sf::lt0(a) << 1 | sf::ge0(a) << 2 | sf::le0(a) << 3 | sf::lt(a, b) << 4 |
                   sf::lt_abs(a, b) << 5 | sf::prod_neg(a, b) << 6 | sf::isnan_b(sf::bits(a)) << 7);
    } else if (op == 3) {  // fmax / fmin; +0 / -0 ties are ordered -0 < +0 by the bit forms
      const bool zeros = a == 0.0 && b == 0.0;
      h = zeros ? 0.0 : fmax(a, b);
      s = zeros ? 0.0 : sf::fmax_nm(a, b);
      h2 = zeros ? 0.0 : fmin(a, b);
      s2 = zeros ? 0.0 : sf::fmin_nm(a, b);
    } else if (op == 5) {  // products, including results next to the overflow and subnormal limits
      if (((r3 >> 50) & 3) == 0) {
        const int ea = (int)((__double_as_longlong(a) >> 52) & 0x7FF);
        const int target = ((r3 >> 52) & 1) ? (int)((r3 >> 53) % 7) - 3 : 2044 + (int)((r3 >> 53) % 7);
        const int eb = target - ea + 1023;
        if (eb >= 1 && eb <= 2046)
          b = __longlong_as_double((long long)((r1 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)eb << 52)));
      }
      h = a * b;
      s = sf::mul_rn(a, b);
    } else {  // scalings by powers of two, including into and out of the subnormal range
      const int k = (int)((r2 >> 40) % 121) - 60;
      const double y = ldexp(1.0, k);
      h = a * y;
      s = sf::mul_pow2(a, y, k);
      h2 = a * 0.5;
      s2 = sf::half(a);
    }
    const bool same = (__double_as_longlong(h) == __double_as_longlong(s) || (h != h && s != s)) &&
                      (__double_as_longlong(h2) == __double_as_longlong(s2) || (h2 != h2 && s2 != s2));
    if (!same) {
      const unsigned long long k = atomicAdd(bad, 1ull);
      if (k == 0) {
        ex[0] = a;
        ex[1] = b;
        ex[2] = s;
      }
    }
  }
}

}  // namespace

extern "C" int fv2d_selftest_arith(int op, uint64_t n, uint64_t seed, uint64_t *mismatches, double example[3]) {
  if (op < 0 || op > 5 || !mismatches) return FV2D_ERR_INVALID;
  unsigned long long *bad = nullptr;
  double *ex = nullptr;
  if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess || cudaMalloc(&ex, 3 * sizeof(double)) != cudaSuccess) {
    cudaFree(bad);
    return FV2D_ERR_NOMEM;
  }
  cudaMemset(bad, 0, sizeof(*bad));
  cudaMemset(ex, 0, 3 * sizeof(double));
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  selftest_kernel<<<sms * 8, 256>>>(op, n, seed, bad, ex);
  unsigned long long h = 0;
  double hx[3] = {0, 0, 0};
  const cudaError_t e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaMemcpy(hx, ex, sizeof(hx), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  cudaFree(ex);
  if (e != cudaSuccess) return FV2D_ERR_CUDA;
  *mismatches = h;
  if (example)
    for (int k = 0; k < 3; ++k) example[k] = hx[k];
  return FV2D_OK;
}

namespace {
// A wait that nothing will end: an mbarrier expecting one arrival that never
// comes, waited on with the step kernel's bounded wait.
__global__ void wait_timeout_kernel(uint32_t limit, int *flag) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    fv2d::mbar_init(&bar, 1);
    fv2d::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) fv2d::mbar_wait_bounded(&bar, flag, limit);
}
}  // namespace

extern "C" int fv2d_selftest_wait_timeout(uint32_t limit, int *timed_out) {
  if (!timed_out || limit == 0 || limit > (1u << 20)) return FV2D_ERR_INVALID;
  int *flag = nullptr;
  if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return FV2D_ERR_NOMEM;
  cudaMemset(flag, 0, sizeof(int));
  wait_timeout_kernel<<<1, 32>>>(limit, flag);
  int h = 0;
  const cudaError_t e = cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(flag);
  if (e != cudaSuccess) return FV2D_ERR_CUDA;
  *timed_out = h;
  return FV2D_OK;
}
