// ev_device.cuh -- device arithmetic that reproduces the reference's
// rounding steps.
//
// The CPU crate multiplies complex numbers in FMA form
//   re = fma(a.re, b.re, -(a.im*b.im)),  im = fma(a.re, b.im, a.im*b.re)
// (src/complex.rs:115-124) and adds them component-wise.  Every helper here
// spells each rounding step with an explicit round-to-nearest intrinsic so
// that neither the compiler's contraction nor reassociation can change a
// result: in complex128 the engine's gate arithmetic is bit-identical to the
// reference's (signed zeros aside).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ev {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y)),
                      __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)),
                     __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
// (r + 0i) * b in FMA form collapses to a rounded product per component:
// fma(r, x, -(0*y)) == r*x for finite x, y.
__device__ __forceinline__ double2 rmul(double r, double2 b) {
  return make_double2(__dmul_rn(r, b.x), __dmul_rn(r, b.y));
}
__device__ __forceinline__ float2 rmul(float r, float2 b) {
  return make_float2(__fmul_rn(r, b.x), __fmul_rn(r, b.y));
}
__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }

// norm_sqr = re.mul_add(re, im*im) (src/complex.rs:80-82), always in f64.
__device__ __forceinline__ double nsq(double2 a) { return __fma_rn(a.x, a.x, __dmul_rn(a.y, a.y)); }
__device__ __forceinline__ double nsq(float2 a) {
  const double x = a.x, y = a.y;
  return __fma_rn(x, x, __dmul_rn(y, y));
}

template <typename V>
struct Real;
template <>
struct Real<double2> {
  using T = double;
};
template <>
struct Real<float2> {
  using T = float;
};

template <typename V>
__device__ __forceinline__ V mkv(double re, double im);
template <>
__device__ __forceinline__ double2 mkv<double2>(double re, double im) {
  return make_double2(re, im);
}
template <>
__device__ __forceinline__ float2 mkv<float2>(double re, double im) {
  return make_float2(float(re), float(im));
}

// Inserts a 0 bit at position k of i (src/kernel.rs:39-44).
__device__ __forceinline__ uint64_t insert0(uint64_t i, int k) {
  const uint64_t low = (uint64_t(1) << k) - 1;
  return ((i >> k) << (k + 1)) | (i & low);
}

// ---- double-float arithmetic on the FP32 pipe ------------------------------
// GB300 issues FP64 at a small fraction of the FP32 rate, so complex64
// reductions keep their per-element work in FP32 without giving up FP64-level
// accuracy: a product of two floats is split exactly into p + e
// (e = fma(a, b, -p)), and sums are carried as unevaluated pairs hi + lo
// (Knuth's TwoSum, then a Fast2Sum renormalisation), a representation with
// about 48 significant bits.

// Exact float -> double by bit manipulation on the integer pipe: normal
// numbers and zeros directly, subnormals, infinities and NaNs through the
// conversion instruction.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  if (e == 0u && (u & 0x7FFFFFu) == 0u) return __longlong_as_double((long long)(uint64_t(u) << 32));
  if (e == 0u || e == 0xFFu) return double(f);
  const uint64_t bits = (uint64_t(u & 0x80000000u) << 32) | (uint64_t(e + 896u) << 52) |
                        (uint64_t(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}

struct FF {
  float hi = 0.f, lo = 0.f;
  // (hi, lo) += x
  __device__ __forceinline__ void add(float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    const float t = __fadd_rn(lo, err);
    hi = __fadd_rn(s, t);
    lo = __fsub_rn(t, __fsub_rn(hi, s));
  }
  // (hi, lo) += a * b, the product taken exactly
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    lo = __fadd_rn(lo, __fmaf_rn(a, b, -p));
    add(p);
  }
  __device__ __forceinline__ double value() const { return f2d_exact(hi) + f2d_exact(lo); }
};

// RN(hi + lo) as an f64 for a renormalised double-float pair (|lo| at most
// half an ulp of hi), formed on the integer pipes.  With d = eh - el >= 24
// the exact sum is the integer (Mh 2^d +- Ml) 2^(el - 150); for d > 39 Ml is
// first shifted right by d - 39 with the bits it loses folded into bit 0
// (they lie far below the rounding position, so only their presence
// matters), which keeps the sum within 64 bits.  It is rounded to 53 bits
// with ties to even.  Zeros, subnormals, infinities, NaNs and pairs that are
// not renormalised take the FP64 add (the same value).
__device__ __forceinline__ double ff_to_f64(float hi, float lo) {
  const uint32_t uh = __float_as_uint(hi), ul = __float_as_uint(lo);
  const int eh = int((uh >> 23) & 0xFFu);
  int el = int((ul >> 23) & 0xFFu);
  int d = eh - el;
  if ((ul & 0x7FFFFFFFu) == 0u) return f2d_exact(hi);
  if (eh == 0 || eh == 0xFF || el == 0 || el == 0xFF || d < 24) return f2d_exact(hi) + f2d_exact(lo);
  const uint64_t mh = uint64_t((uh & 0x7FFFFFu) | 0x800000u);
  uint64_t ml = uint64_t((ul & 0x7FFFFFu) | 0x800000u);
  if (d > 39) {
    const int s = d - 39;
    ml = s >= 25 ? 1u : ((ml >> s) | uint64_t((ml & ((uint64_t(1) << s) - 1)) != 0));
    el += s;
    d = 39;
  }
  const uint64_t S = ((uh ^ ul) >> 31) ? (mh << d) - ml : (mh << d) + ml;  // > 0
  // the leading bit is at 23 + d, or 22 + d after a borrow
  const int p = (S >> (23 + d)) ? 23 + d : 22 + d;
  const int sh = p - 52;  // bits below 2^sh are dropped (sh >= -7)
  uint64_t m;
  if (sh <= 0) {
    m = S << (-sh);
  } else {
    const uint64_t kept = S >> sh, rem = S & ((uint64_t(1) << sh) - 1), half = uint64_t(1) << (sh - 1);
    m = kept + ((rem > half || (rem == half && (kept & 1u))) ? 1u : 0u);
  }
  // value = m 2^(el - 150 + sh), m in [2^52, 2^53]: the leading 1 (and a
  // round-up to 2^53) carries into the exponent field
  const uint64_t ebits = uint64_t(el - 150 + sh + 1074) << 52;
  return __longlong_as_double((long long)((uint64_t(uh >> 31) << 63) | (ebits + m)));
}

}  // namespace ev

namespace ev {
// xoshiro256++ seeded through SplitMix64 (the reference's Rng,
// src/rng.rs:18-58), for uniforms drawn on the device.
struct DevRng {
  uint64_t s[4];
  __device__ explicit DevRng(uint64_t seed) {
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      seed += 0x9E3779B97F4A7C15ULL;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      s[w] = z ^ (z >> 31);
    }
  }
  __device__ static uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
  __device__ uint64_t next_u64() {
    const uint64_t result = rotl(s[0] + s[3], 23) + s[0];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  __device__ double next_f64() { return double(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
};
}  // namespace ev
