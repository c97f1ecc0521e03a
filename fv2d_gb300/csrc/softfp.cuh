// softfp.cuh -- binary64 arithmetic computed on the integer and FP32 pipes:
// correctly rounded division, square root and multiplication, comparisons,
// fmin / fmax and scalings by powers of two.
//
// GB300 executes binary64 at 1/64 of its FP32 rate; a hardware double
// division or square root occupies that pipe for ~7-8 DFMA-equivalents while
// the integer pipes stay idle in the FP64 step kernel.  These routines return
// exactly the IEEE round-to-nearest-even result (the same bits as x / y,
// sqrt(x), x * y) for finite normal operands with a normal result and for zero
// operands, and defer every other case (subnormals, infinities, NaNs,
// division by zero, overflow, underflow) to the hardware instruction.
//
// Division: the divisor's 53-bit significand is normalised to a 64-bit word d;
// its reciprocal word v = floor((2^128 - 1) / d) - 2^64 (the definition of
// Moller & Granlund, "Improved division by invariant integers", IEEE TC 2011)
// is seeded from the FP32 reciprocal, refined by two Newton-Raphson steps in
// 64-bit fixed point and made exact by a final check; their 2-by-1 division
// step then yields the exact 53-bit quotient and remainder, from which the
// rounding is decided (compare twice the remainder with the divisor).
//
// Division, square root and multiplication are called rather than inlined:
// the step kernel uses them a dozen times per cell, and one shared copy keeps
// its code within the instruction caches (measured ~3 % faster).
//
// Square root: the FP32 reciprocal square root seeds a Newton-Raphson
// iteration for 1/sqrt in 64-bit fixed point; the product with the operand
// gives the integer square root within a few units, which the exact remainder
// M - S^2 corrects; round up when the remainder exceeds S.
#pragma once

#include <stdint.h>

namespace fv2d {
namespace softfp {

// The moves are opaque to the optimiser: a plain bit cast lets it recognise
// the integer tests below as floating-point classifications and lower them
// back to binary64 instructions (abs.f64 + setp).
__device__ __forceinline__ uint64_t bits(double x) {
  uint64_t b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
__device__ __forceinline__ double from_bits(uint64_t b) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(b));
  return x;
}

// Hardware instructions for the special cases, behind calls so that the
// compiler cannot if-convert their expansion into the common path (issued
// predicated-off instructions still occupy the binary64 pipe).
static __device__ __noinline__ double div_hw(double a, double b) { return a / b; }
static __device__ __noinline__ double sqrt_hw(double x) { return sqrt(x); }

// The seeds are assembled from bit fields rather than by int64 <-> float
// conversions, which issue on the binary64 pipe.
__device__ __forceinline__ uint64_t recip_word(uint64_t d) {
  // f = d / 2^63 truncated to 24 bits, in [1, 2); r ~ 1/f in (1/2, 1]
  const float f = __uint_as_float(0x3F800000u | ((uint32_t)(d >> 40) & 0x7FFFFFu));
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
  // x = (2 r - 1) 2^64: the fraction field of 2 r shifted up, clamped to
  // [0, 2^64 - 1] when the approximation leaves [1/2, 1)
  const uint32_t rb = __float_as_uint(r);
  uint64_t x = rb >= 0x3F800000u ? ~0ull : rb < 0x3F000000u ? 0ull : (uint64_t)(rb & 0x7FFFFFu) << 41;
  for (int it = 0; it < 2; ++it) {
    // e = 2^128 - d (2^64 + x); x += (2^64 + x) e / 2^128
    const uint64_t lo = d * x, hi = __umul64hi(d, x);
    const uint64_t s_hi = hi + d;
    const int64_t e_hi = (int64_t)(0ull - s_hi - (lo != 0));
    const int64_t corr = e_hi + (int64_t)(__umul64hi(x, (uint64_t)e_hi) - (e_hi < 0 ? x : 0ull));
    // A Newton step from an overestimate lands below the root by about the
    // squared error (2^-46 relative after the FP32 seed).  For a divisor
    // just below a power of two (d > 2^64 - 2^19) the root v is smaller than
    // that and the step would cross 2^64 + 0, wrapping the fraction word:
    // clamp at zero, an underestimate the next step refines.
    x = (corr < 0 && (uint64_t)(-corr) > x) ? 0ull : x + (uint64_t)corr;
  }
  // exact: d (2^64 + x) <= 2^128 - 1 < d (2^64 + x + 1)
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    const uint64_t lo = d * x, hi = __umul64hi(d, x);
    const uint64_t s_hi = hi + d;
    if (s_hi < d) {
      --x;
      continue;
    }
    const uint64_t lo2 = lo + d;
    const uint64_t s_hi2 = s_hi + (lo2 < lo);
    if (s_hi2 < s_hi) break;
    ++x;
  }
  return x;
}

// a / b, round to nearest even, in two halves so that quotients with a
// common divisor share its reciprocal word: div_begin classifies the operands
// and aligns the dividend, div_finish forms the quotient from v = recip_word(d)
// (needed only when some quotient takes the fast path).
struct DivOp {
  uint64_t ia, ib, d, u1, u0;
  int e;
  bool fast;
};

__device__ __forceinline__ DivOp div_begin(double a, double b) {
  DivOp o;
  o.ia = bits(a);
  o.ib = bits(b);
  const int ea = (int)((o.ia >> 52) & 0x7ff), eb = (int)((o.ib >> 52) & 0x7ff);
  const uint64_t ma = (o.ia & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const uint64_t mb = (o.ib & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const bool big = ma >= mb;
  o.e = ea - eb + 1023 - (big ? 0 : 1);
  o.fast = !(ea == 0 || ea == 0x7ff || eb == 0 || eb == 0x7ff || o.e <= 0 || o.e >= 0x7fe);
  // Q = floor(n 2^52 / mb) with n = ma or 2 ma, i.e. (n 2^63) / (mb 2^11)
  o.d = mb << 11;
  const uint64_t n = big ? ma : (ma << 1);
  o.u1 = n >> 1;
  o.u0 = n << 63;
  return o;
}

__device__ __forceinline__ double div_finish(const DivOp &o, double a, double b, uint64_t v) {
  if (!o.fast) {
    // +-0 / (finite nonzero normal) is a zero with the xor of the signs;
    // quiescent regions (zero momentum) make this the common special case.
    const int eb = (int)((o.ib >> 52) & 0x7ff);
    if ((o.ia << 1) == 0 && eb != 0 && eb != 0x7ff) return from_bits((o.ia ^ o.ib) & 0x8000000000000000ull);
    return div_hw(a, b);
  }
  const uint64_t d = o.d, u1 = o.u1, u0 = o.u0;
  uint64_t q0 = v * u1, q1 = __umul64hi(v, u1);
  const uint64_t s0 = q0 + u0;
  q1 = q1 + u1 + (s0 < q0) + 1;
  q0 = s0;
  uint64_t r = u0 - q1 * d;
  if (r > q0) {
    --q1;
    r += d;
  }
  if (r >= d) {
    ++q1;
    r -= d;
  }
  // nearest even: compare 2 r with d
  uint64_t Q = q1 + ((r > d - r) || (r == d - r && (q1 & 1)));
  int e = o.e;
  if (Q >> 53) {
    Q >>= 1;
    ++e;
  }
  const uint64_t out = ((uint64_t)e << 52) | (Q & 0xFFFFFFFFFFFFFull) | ((o.ia ^ o.ib) & 0x8000000000000000ull);
  return from_bits(out);
}

static __device__ __noinline__ double div_rn(double a, double b) {
  const DivOp o = div_begin(a, b);
  const uint64_t v = o.fast ? recip_word(o.d) : 0ull;
  return div_finish(o, a, b, v);
}

// {a1 / b, a2 / b} (returned by value: outputs through references would live
// on the stack across the call)
static __device__ __noinline__ double2 div2_rn(double a1, double a2, double b) {
  const DivOp o1 = div_begin(a1, b), o2 = div_begin(a2, b);
  const uint64_t v = (o1.fast || o2.fast) ? recip_word(o1.d) : 0ull;
  return make_double2(div_finish(o1, a1, b, v), div_finish(o2, a2, b, v));
}

// Quotients by one divisor b: recip_of(b) computes its reciprocal word once
// (0 when b is zero, subnormal, infinite or NaN: the hardware handles every
// quotient by such a b), div_by(a, b, v) forms each quotient.
static __device__ __noinline__ uint64_t recip_of(double b) {
  const uint64_t ib = bits(b);
  const int eb = (int)((ib >> 52) & 0x7ff);
  if (eb == 0 || eb == 0x7ff) return 0ull;
  return recip_word(((ib & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11);
}
static __device__ __noinline__ double div_by(double a, double b, uint64_t v) {
  const DivOp o = div_begin(a, b);
  // a normal divisor's reciprocal word is never 0 (it is at least 2^11)
  if (o.fast && v == 0ull) return div_rn(a, b);
  return div_finish(o, a, b, v);
}

// recip_of(b) for a divisor known on the host (the mesh spacings): the same
// word from its definition, floor((2^128 - 1) / d) - 2^64 with d the
// divisor's significand aligned to bit 63; the quotient lies in
// [2^64, 2^65), so its low 64 bits are the word.
inline uint64_t recip_of_host(double b) {
  union {
    double f;
    uint64_t u;
  } c{b};
  const int eb = (int)((c.u >> 52) & 0x7ff);
  if (eb == 0 || eb == 0x7ff) return 0ull;
  const uint64_t d = ((c.u & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11;
  return (uint64_t)(~(unsigned __int128)0 / d);
}

// sqrt(x), round to nearest even.
static __device__ __noinline__ double sqrt_rn(double x) {
  const uint64_t ix = bits(x);
  const int E = (int)(ix >> 52);  // sign bit included: negative values fail the range test
  if ((ix << 1) == 0) return x;   // sqrt(+-0) = +-0
  if (E == 0 || E >= 0x7ff) return sqrt_hw(x);
  const uint64_t m = (ix & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int t = E - 1075;  // x = m 2^t
  const int odd = t & 1;
  // M = m 2^(52 + odd) in [2^104, 2^106); S = floor(sqrt(M)) in [2^52, 2^53)
  const uint64_t Z = m << (10 + odd);  // M / 2^42, in [2^62, 2^64)
  // Y ~ 2^94 / sqrt(Z), in (2^62, 2^63]: with g = Z / 2^62 = (m / 2^52) 2^odd
  // in [1, 4) truncated to 24 bits, Y = rsqrt(g) 2^63 and rsqrt(g) in (1/2, 1]
  const float g = __uint_as_float((uint32_t)((127 + odd) << 23) | (uint32_t)((m >> 29) & 0x7FFFFFu));
  float rs;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rs) : "f"(g));
  const uint32_t sb = __float_as_uint(rs);
  uint64_t Y = (uint64_t)((sb & 0x7FFFFFu) | 0x800000u) << (39 + (int)(sb >> 23) - 126);
  for (int it = 0; it < 2; ++it) {
    // U = Z Y^2 / 2^128 ~ 2^60; Y <- Y (3 2^60 - U) / 2^61
    const uint64_t W = __umul64hi(Y, Y);
    const uint64_t U = __umul64hi(Z, W);
    Y = __umul64hi(Y, (0x3000000000000000ull - U) << 2) << 1;
  }
  // sqrt(M) = sqrt(Z) 2^21 = Z Y / 2^73
  uint64_t S = __umul64hi(Z, Y) >> 9;
  // exact remainder R = M - S^2 (small; the low 64 bits carry it)
  const uint64_t Mlo = m << (52 + odd);
  int64_t R = (int64_t)(Mlo - S * S);
#pragma unroll 1
  for (int k = 0; k < 4 && R < 0; ++k) {
    R += (int64_t)(2 * S - 1);
    --S;
  }
#pragma unroll 1
  for (int k = 0; k < 4 && R > (int64_t)(2 * S); ++k) {
    R -= (int64_t)(2 * S + 1);
    ++S;
  }
  uint64_t Q = S + (R > (int64_t)S);
  int e = ((t - odd) >> 1) + 26 + 1023;  // sqrt(x) = Q 2^((t - odd)/2 - 26), Q in [2^52, 2^53]
  if (Q >> 53) {
    Q >>= 1;
    ++e;
  }
  return from_bits(((uint64_t)e << 52) | (Q & 0xFFFFFFFFFFFFFull));
}

// ---------------------------------------------------------------------------
// Comparisons and power-of-two scalings on the bit patterns.  Each returns
// exactly what the IEEE operation returns (NaN compares false; +0 == -0),
// so a binary64 DSETP / DMUL on the 1/64-rate pipe becomes a few integer
// instructions.  Operands outside the cheap range (results that would be
// subnormal, overflow, NaN/inf inputs of a product) go to the hardware
// instruction through a call that is not if-converted.



constexpr uint64_t MAG = 0x7FFFFFFFFFFFFFFFull, INF_BITS = 0x7FF0000000000000ull, SIGN = 0x8000000000000000ull;

__device__ __forceinline__ bool isnan_b(uint64_t b) { return (b & MAG) > INF_BITS; }

static __device__ __noinline__ double mul_hw(double x, double y) { return x * y; }
static __device__ __noinline__ bool prod_neg_hw(double x, double y) { return x * y < 0.0; }

// x > 0, x < 0, x >= 0, x <= 0
__device__ __forceinline__ bool gt0(double x) { return bits(x) - 1ull < INF_BITS; }
__device__ __forceinline__ bool lt0(double x) { return bits(x) - (SIGN + 1ull) < INF_BITS; }
__device__ __forceinline__ bool ge0(double x) {
  const uint64_t b = bits(x);
  return b <= INF_BITS || b == SIGN;
}
__device__ __forceinline__ bool le0(double x) {
  const uint64_t b = bits(x);
  return (b & MAG) == 0 || b - SIGN <= INF_BITS;
}

// Order key with -0 == +0 (IEEE comparison order for non-NaN values).
__device__ __forceinline__ int64_t key_ieee(uint64_t b) {
  const int64_t m = (int64_t)(b & MAG);
  return (int64_t)b < 0 ? -m : m;
}
// x < y (IEEE: false when either is NaN)
__device__ __forceinline__ bool lt(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  return !isnan_b(a) && !isnan_b(b) && key_ieee(a) < key_ieee(b);
}

// maximumNumber / minimumNumber: a NaN operand yields the other one; -0 < +0.
// (The C fmax / fmin of the aarch64 C library, FMAXNM / FMINNM.)
__device__ __forceinline__ int64_t key_total(uint64_t b) { return (int64_t)(b ^ ((uint64_t)((int64_t)b >> 63) >> 1)); }
__device__ __forceinline__ double fmax_nm(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  if (isnan_b(b)) return x;
  if (isnan_b(a)) return y;
  return key_total(a) > key_total(b) ? x : y;
}
__device__ __forceinline__ double fmin_nm(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  if (isnan_b(b)) return x;
  if (isnan_b(a)) return y;
  return key_total(a) < key_total(b) ? x : y;
}

// |x| < |y|
__device__ __forceinline__ bool lt_abs(double x, double y) {
  const uint64_t a = bits(x) & MAG, b = bits(y) & MAG;
  return a < b && b <= INF_BITS;
}

// x * y < 0.  Nonzero non-NaN factors of opposite signs give a negative
// product unless it underflows to -0, impossible when the biased exponents
// sum to at least 972 (|x y| >= 2^-1074); smaller products go to hardware.
__device__ __forceinline__ bool prod_neg(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  const uint64_t ma = a & MAG, mb = b & MAG;
  if (!((a ^ b) & SIGN) || ma == 0 || mb == 0 || ma > INF_BITS || mb > INF_BITS) return false;
  const int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
  if (ea != 0 && eb != 0 && ea + eb >= 972) return true;
  return prod_neg_hw(x, y);
}

// x * 2^k for y == 2^k (k = unbiased exponent of y): exact exponent shift
// when x and the result are normal; zeros keep their sign.
__device__ __forceinline__ double mul_pow2(double x, double y, int k) {
  const uint64_t a = bits(x);
  const int e = (int)((a >> 52) & 0x7FF);
  if ((a & MAG) == 0) return x;
  if ((unsigned)(e - 1) < 0x7FEu && (unsigned)(e + k - 1) < 0x7FEu) return from_bits(a + ((uint64_t)(int64_t)k << 52));
  return mul_hw(x, y);
}

// x * 0.5
__device__ __forceinline__ double half(double x) { return mul_pow2(x, 0.5, -1); }

// x * y, round to nearest even, for normal operands with a normal result
// (and zero times finite): the 106-bit product of the significands, cut at
// bit 52 or 53 with the remainder deciding the rounding.  Subnormal, infinite
// or NaN operands and results that overflow or fall below 2^-1022 (where the
// subnormal grid changes the rounding) use the hardware instruction.
static __device__ __noinline__ double mul_rn(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  const uint64_t sgn = (a ^ b) & SIGN;
  const int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  if ((a & MAG) == 0 || (b & MAG) == 0) {
    if (ea != 0x7FF && eb != 0x7FF) return from_bits(sgn);
    return mul_hw(x, y);
  }
  int e = ea + eb - 1023;
  if ((unsigned)(ea - 1) >= 0x7FEu || (unsigned)(eb - 1) >= 0x7FEu || (unsigned)(e - 1) >= 0x7FDu)
    return mul_hw(x, y);
  const uint64_t ma = (a & 0xFFFFFFFFFFFFFull) | (1ull << 52), mb = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const uint64_t lo = ma * mb, hi = __umul64hi(ma, mb);  // P = hi 2^64 + lo in [2^104, 2^106)
  const int top = (int)(hi >> 41);                        // bit 105 of P
  e += top;
  const int s = 52 + top;
  uint64_t M = (hi << (64 - s)) | (lo >> s);              // P >> s in [2^52, 2^53)
  const uint64_t R = lo & ((1ull << s) - 1), H = 1ull << (s - 1);
  M += (R > H) || (R == H && (M & 1));
  if (M >> 53) {
    M >>= 1;
    ++e;
  }
  if (e >= 0x7FF) return mul_hw(x, y);
  return from_bits(sgn | ((uint64_t)e << 52) | (M & 0xFFFFFFFFFFFFFull));
}

}  // namespace softfp
}  // namespace fv2d
