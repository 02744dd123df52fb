// ev_softfp.cuh -- IEEE-754 binary64 multiplication and addition, round to
// nearest even, computed on the integer pipes.
//
// GB300's FP64 pipe retires about 0.53e12 fused multiply-adds per second,
// far below its integer and FP32 pipes, and the complex128 gate passes are
// bound by it.  A correctly rounded product is a fixed function of its
// operands, so a product formed here from the 106-bit integer product of the
// significands is bit-identical to the hardware's: the tile passes send part
// of their products through this path and the rest through the FP64 pipe,
// with unchanged results.
//
// The fast path covers operands that are normal with biased exponents in
// [512, 1534], where a product can neither underflow nor lose its exponent
// range; it reports every other operand (zero, subnormal, infinite, NaN, or
// far from 1) so the caller computes that product with the FP64 pipe.  The
// rounding follows the standard's definition: keep the top 53 bits of the
// exact product, round up when the discarded part exceeds half an ulp, or
// equals it and the kept part is odd.
//
// The header compiles for the host too (g++), where the CPU tests compare it
// with the host's own multiplication and addition.
#pragma once

#include <stdint.h>
#ifndef __CUDACC__
#include <string.h>
#endif

#ifdef __CUDACC__
#define EV_SOFT_FN __host__ __device__ __forceinline__
#else
#define EV_SOFT_FN static inline
#endif

namespace ev {
namespace softfp {

EV_SOFT_FN uint64_t to_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

EV_SOFT_FN double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

// The 128-bit product of two 64-bit integers: *hi gets the top 64 bits,
// the return value is nonzero when the low 64 bits are.
EV_SOFT_FN uint32_t mul_128(uint64_t a, uint64_t b, uint64_t* hi) {
#ifdef __CUDA_ARCH__
  const uint32_t al = (uint32_t)a, ah = (uint32_t)(a >> 32);
  const uint32_t bl = (uint32_t)b, bh = (uint32_t)(b >> 32);
  uint32_t r0, r1, r2, r3;
  // schoolbook product of 32-bit limbs, carries chained through the .cc flag
  asm("mul.lo.u32 %0, %4, %6;\n\t"
      "mul.hi.u32 %1, %4, %6;\n\t"
      "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
      "madc.hi.u32 %2, %4, %7, 0;\n\t"
      "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
      "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
      "madc.hi.u32 %3, %5, %7, 0;\n\t"
      "mad.lo.cc.u32 %2, %5, %7, %2;\n\t"
      "addc.u32 %3, %3, 0;"
      : "=&r"(r0), "=&r"(r1), "=&r"(r2), "=&r"(r3)
      : "r"(al), "r"(ah), "r"(bl), "r"(bh));
  *hi = ((uint64_t)r3 << 32) | r2;
  return r0 | r1;
#else
  const unsigned __int128 p = (unsigned __int128)a * b;
  *hi = (uint64_t)(p >> 64);
  return (uint64_t)p != 0;
#endif
}

// An operand unpacked once and used in several products: the significand
// with its leading 1 at bit 63, and the word holding the sign bit (bit 31)
// and the biased exponent minus 512 in the exponent field's place (bits
// 20..30).  Adding two such words adds the exponents and, as the exponent
// sum stays below 2^11, leaves the xor of the signs in bit 31.
struct Unpacked {
  uint64_t sig;
  uint32_t ex;
  uint32_t ok;  // normal, biased exponent in [512, 1534]
};

EV_SOFT_FN Unpacked unpack(double x) {
  const uint64_t u = to_bits(x);
  const uint32_t w = (uint32_t)(u >> 32);
  Unpacked r;
  r.sig = (u << 11) | (1ull << 63);
  // An exponent below 512 wraps the field to [1536, 2047]; one above 1534
  // leaves it in [1023, 1535]; the sign bit is not borrowed from in range.
  r.ex = (w & 0xFFF00000u) - (512u << 20);
  r.ok = (r.ex & 0x7FFFFFFFu) <= (1022u << 20);
  return r;
}

// RN(a * b) for a.ok && b.ok; any value otherwise.
EV_SOFT_FN double mul(const Unpacked& a, const Unpacked& b) {
  // a.sig * b.sig = P * 2^22 with P the 106-bit product of the 53-bit
  // significands; hi holds its top 64 bits, in [2^62, 2^64).
  uint64_t hi;
  const uint32_t sticky = mul_128(a.sig, b.sig, &hi);
  const uint32_t top = (uint32_t)(hi >> 63);  // P >= 2^105
  // The 53 kept bits are hi >> sh.  Fold the bits below hi into bit 0
  // (below the half-ulp bit sh - 1 in both cases), then add half an ulp
  // minus one plus the kept part's lowest bit: the sum carries into bit sh
  // exactly when the discarded part exceeds half an ulp, or equals it and
  // the kept part is odd.  hi <= 2^64 - 2^12, so the sum cannot overflow.
  const uint32_t sh = 10u + top;
  const uint64_t h = hi | (uint64_t)(sticky != 0);
  const uint32_t lsb = ((uint32_t)h >> sh) & 1u;
  const uint64_t m = (h + ((1ull << (sh - 1)) - 1u + lsb)) >> sh;  // in [2^52, 2^53]
  // Sign (bit 31) and the biased exponent minus one in place (in [0, 2045]):
  // adding the significand with its leading 1 at bit 52 completes the
  // exponent, and a significand that rounded up to 2^53 carries into it.
  const uint32_t word = a.ex + b.ex + (top << 20);
  return from_bits(((uint64_t)word << 32) + m);
}

// Leading zeros of a nonzero 64-bit value.
EV_SOFT_FN uint32_t clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__clzll((long long)x);
#else
  return (uint32_t)__builtin_clzll(x);
#endif
}

// True when x and y are both in the add's domain: normal, biased exponent in
// [512, 1534] (the product's domain), where a sum can neither overflow nor
// fall below the normal range.
EV_SOFT_FN bool add_ok(double x, double y) {
  const uint32_t ex = (uint32_t)(to_bits(x) >> 52) & 0x7FFu, ey = (uint32_t)(to_bits(y) >> 52) & 0x7FFu;
  return ex - 512u <= 1022u && ey - 512u <= 1022u;
}

// RN(x + y) for add_ok(x, y); any value otherwise.  The larger magnitude
// fixes the sign and exponent; the smaller significand is aligned to it with
// a sticky bit (10 guard bits below the 53, so an alignment of 0 or 1 bit is
// exact and a larger one leaves at most one left shift after a subtraction);
// the sum is normalised with a leading-zero count and rounded to nearest
// even.  An exact cancellation gives +0, as round to nearest does.  Written
// from the IEEE-754 definition of addition; it costs ~60 integer
// instructions, against one FP64 add.
EV_SOFT_FN double add(double x, double y) {
  const uint64_t kSign = 1ull << 63, kFrac = (1ull << 52) - 1, kHidden = 1ull << 52;
  uint64_t ux = to_bits(x), uy = to_bits(y);
  uint64_t ax = ux & ~kSign, ay = uy & ~kSign;
  if (ax < ay) {
    const uint64_t tu = ux, ta = ax;
    ux = uy;
    uy = tu;
    ax = ay;
    ay = ta;
  }
  const uint32_t ex = (uint32_t)(ax >> 52), ey = (uint32_t)(ay >> 52);
  const uint32_t d = ex - ey;
  const uint64_t X = ((ax & kFrac) | kHidden) << 10;  // leading 1 at bit 62
  const uint64_t Y = ((ay & kFrac) | kHidden) << 10;
  uint64_t yd;
  if (d == 0)
    yd = Y;
  else if (d < 64)
    yd = (Y >> d) | (uint64_t)((Y << (64 - d)) != 0);
  else
    yd = 1;  // below every kept and rounding bit: a sticky bit only
  const uint64_t S = ((ux ^ uy) & kSign) ? X - yd : X + yd;
  if (S == 0) return 0.0;
  const uint32_t lz = clz64(S);  // 0: a carry into bit 63; 1: none; more: cancellation
  const uint64_t sn = S << lz;   // leading 1 at bit 63
  const uint64_t kept = sn >> 11;
  const uint32_t low = (uint32_t)sn & 0x7FFu;
  // round up above half an ulp, or at half with an odd kept part; a sticky
  // bit from the alignment leaves low odd below bit 10, never at half
  const uint64_t m = kept + (uint64_t)((low + (uint32_t)(kept & 1)) > 0x400u);  // [2^52, 2^53]
  // the value's exponent is ex + 1 - lz; the significand's leading 1 (or a
  // rounding carry to 2^53) adds the one back into the exponent field
  return from_bits((ux & kSign) + ((uint64_t)(ex - lz) << 52) + m);
}

}  // namespace softfp
}  // namespace ev
