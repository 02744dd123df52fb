// ev_ozaki.cuh -- complex128 fused unitaries on the FP16 tensor cores by
// digit slicing: the Ozaki scheme (K. Ozaki, T. Ogita, S. Oishi, S. M. Rump,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numerical Algorithms 59
// (2012) 95-118), in a fixed-point form with one scale per row and column.
//
// A fused 5-qubit block is the real GEMM y = x W with K = N = 64 (see
// ev_fused.cu).  Every row x of a step shares one scale: with E the largest
// biased f64 exponent in the row, each value becomes the integer
//     M = trunc(x * 2^(1077 - E)),          |M| < 2^55,
// written in balanced base 256 as seven digits
//     M = sum_{i=0..6} X_i 256^(6-i),   X_i in [-128, 127], X_0 in [-128, 128].
// Column n of W gets the same treatment on the host with its own exponent
// F_n.  A digit is exact in FP16, the product of two digits (|.| <= 2^14) is
// exact, and the sum over K of the products of one diagonal d = i + j
// (d + 1 digit pairs, 64 (d + 1) products) stays within 7 * 2^20 < 2^24, so
// the f32 accumulator of the tensor core holds every partial sum exactly.
// Diagonals 0..6 are kept, each in its own TMEM accumulator, and
// recombined in int64 on the integer pipes:
//     acc = D0 2^40 + D1 2^32 + D2 2^24 + D3 2^16 + D4 2^8 + D5 + round(D6 2^-8),
// |acc| < 2^61, and y = acc * 2^(E + F_n - 2098) is assembled from acc's
// bits with one rounding to nearest even.  No step runs on the FP64 pipe.
// Error per output, in units u = 2^(E + F_n - 2098): 0.5 from D6's
// rounding, the dropped pairs i + j >= 7 (at most 2^(7 - 16) * 8 * 2^20 =
// 128 u, about 2 u for digits of random sign), the truncation of x and W to
// 55 bits below their row / column maximum (64 u each at most), and the
// final rounding to f64.  2^8 u is 2^-53 of the largest value a row times a
// column can reach (64 times the row's largest value times the column's).
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#include <cmath>
#endif

namespace ev {
namespace oz {

constexpr int kDigits = 7;  // 8-bit digits per value (56 bits)
constexpr int kK = 64;      // reals per row: 32 amplitudes of a 5-qubit block

// The two digit counts the engine runs.  Seven digits (EV_FUSED_OZAKI) carry
// 55 bits below each row's (column's) maximum; six digits
// (EV_FUSED_OZAKI6) carry 47 bits, M = trunc(x * 2^(1069 - E)) with
// |M| < 2^47, drop the diagonals d >= 6 and recombine
//     acc = D0 2^32 + D1 2^24 + D2 2^16 + D3 2^8 + D4 + round(D5 2^-8),
// |acc| < 2^53, y = acc * 2^(E + F_n - 2090).  Every diagonal sum stays below
// 6 * 64 * 2^14 < 2^24, so the f32 accumulator still holds it exactly.  The
// error per output, in units u = 2^(E + F_n - 2090) (2^-44 of the largest
// value times the largest column entry): 0.5 from D5's rounding, the dropped
// pairs (at most ~113 u, ~2 u for digits of random sign), the truncation of
// x and W (32 u each at most, ~4 u typical) and the final rounding -- 256
// times the seven-digit form's, about 7e-14 of the row's largest value.
template <int ND>
struct Fmt;
template <>
struct Fmt<7> {
  static constexpr int kBits = 55;                  // |M| < 2^55
  static constexpr uint64_t kBias = 0x808080808080ull;
  static constexpr int kPow2Bias = 2098;
};
template <>
struct Fmt<6> {
  static constexpr int kBits = 47;                  // |M| < 2^47
  static constexpr uint64_t kBias = 0x8080808080ull;
  static constexpr int kPow2Bias = 2090;
};

// M = trunc(x * 2^(1022 + kBits - E)) for the f64 with the given bit halves
// (E the row's largest biased exponent): 1077 - E for seven digits, 1069 - E
// for six.  Zero, subnormal values and values 2^53 times below the maximum
// give 0.
template <int ND>
__host__ __device__ __forceinline__ int64_t fixed(uint32_t hi, uint32_t lo, int E) {
  const int e = int((hi >> 20) & 0x7FFu);
  const int sh = E - e + (53 - Fmt<ND>::kBits);
  if (e == 0 || sh >= 53) return 0;
  const uint64_t mant = (uint64_t((hi & 0xFFFFFu) | 0x100000u) << 32) | lo;
  const uint64_t m = sh < 0 ? mant << (-sh) : mant >> sh;
  return (hi >> 31) ? -int64_t(m) : int64_t(m);
}

// Digit i (0 = most significant) of M in balanced base 256.
template <int ND>
__host__ __device__ __forceinline__ int digit_of(int64_t M, int i) {
  const uint64_t b = uint64_t(M) + Fmt<ND>::kBias;
  if (i == 0) return int(int64_t(b) >> (8 * (ND - 1)));
  return int((b >> (8 * (ND - 1 - i))) & 0xFFu) - 128;
}

// M = trunc(x * 2^(1077 - E)) for the f64 with the given bit halves, where E
// is the largest biased exponent of its row (or column).  Zero, subnormal
// values and values 2^53 times below the maximum give 0.
__host__ __device__ __forceinline__ int64_t fixed55(uint32_t hi, uint32_t lo, int E) {
  const int e = int((hi >> 20) & 0x7FFu);
  const int sh = E - e - 2;  // M = mant * 2^(e - E + 2), sh >= -2
  if (e == 0 || sh >= 53) return 0;
  const uint64_t mant = (uint64_t((hi & 0xFFFFFu) | 0x100000u) << 32) | lo;
  const uint64_t m = sh < 0 ? mant << (-sh) : mant >> sh;
  return (hi >> 31) ? -int64_t(m) : int64_t(m);
}

// The bias that turns the six low balanced digits into bytes:
// M + kBias = sum_{k<6} (X_{6-k} + 128) 256^k + X_0 256^6.
constexpr uint64_t kBias = 0x808080808080ull;

// Digit i (0 = most significant) of M, as an int.
__host__ __device__ __forceinline__ int digit(int64_t M, int i) {
  const uint64_t b = uint64_t(M) + kBias;
  if (i == 0) return int(int32_t(uint32_t(b >> 32)) >> 16);
  return int((b >> (8 * (6 - i))) & 0xFFu) - 128;
}

// Recombination of the seven diagonal sums (exact integers held in f32).
// D0..D3 (|D| <= 2^22) become integers by the magic constant 1.5 * 2^23
// (the integer sits in the low mantissa bits of D + 1.5 * 2^23); D4 and D5
// (|D| < 2^23) by a rounding conversion, exact for an integer; D6 by the
// magic constant 1.5 * 2^31, which leaves round(D6 / 2^8).
constexpr int kPow2Bias = 2098;  // y = acc * 2^(E + F - kPow2Bias)

__host__ __device__ __forceinline__ float f32_of(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

__host__ __device__ __forceinline__ uint32_t f32_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

__host__ __device__ __forceinline__ float add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}

// acc += the contribution of diagonal d whose f32 sum is D.
template <int d>
__host__ __device__ __forceinline__ void accumulate(int64_t& acc, float D) {
  if constexpr (d < 4) {
    const int32_t v = int32_t(f32_bits(add_rn(D, f32_of(0x4B400000u))) - 0x4B400000u);
    acc += int64_t(v) * (int64_t(1) << (40 - 8 * d));
  } else if constexpr (d < 6) {
#ifdef __CUDA_ARCH__
    const int32_t v = __float2int_rn(D);
#else
    const int32_t v = int32_t(D);  // D is an integer: the conversion is exact
#endif
    acc += int64_t(v) * (int64_t(1) << (40 - 8 * d));
  } else {
    const int32_t v = int32_t(f32_bits(add_rn(D, f32_of(0x4F400000u))) - 0x4F400000u);
    acc += int64_t(v);
  }
}

// The seven diagonals of one output combined at once, with the same result
// as accumulate<0..6>: the digit bounds keep three partial sums inside int32,
//   G3 = 2^8 I0 + I1 (< 2^29),  G2 = 2^8 I2 + I3 (< 2^30),
//   G1 = 2^8 I4 + I5 + round(D6 / 2^8) (< 2^31),
// and acc = 2^32 G3 + 2^16 G2 + G1.  The magic constants of the f32-to-int
// conversions cancel in the wrapping 32-bit sums.
// (G3, G2) from D0..D3, G1 from D4..D6 (callers can release D0..D3 first).
__host__ __device__ __forceinline__ void combine_hi(float D0, float D1, float D2, float D3,
                                                    int32_t& g3, int32_t& g2) {
  constexpr uint32_t kM = 0x4B400000u;
  const uint32_t b0 = f32_bits(add_rn(D0, f32_of(kM))), b1 = f32_bits(add_rn(D1, f32_of(kM)));
  const uint32_t b2 = f32_bits(add_rn(D2, f32_of(kM))), b3 = f32_bits(add_rn(D3, f32_of(kM)));
  g3 = int32_t((b0 << 8) + b1 - ((kM << 8) + kM));
  g2 = int32_t((b2 << 8) + b3 - ((kM << 8) + kM));
}
__host__ __device__ __forceinline__ int32_t combine_lo(float D4, float D5, float D6) {
  const uint32_t b6 = f32_bits(add_rn(D6, f32_of(0x4F400000u)));
#ifdef __CUDA_ARCH__
  const uint32_t i4 = uint32_t(__float2int_rn(D4)), i5 = uint32_t(__float2int_rn(D5));
#else
  const uint32_t i4 = uint32_t(int32_t(D4)), i5 = uint32_t(int32_t(D5));
#endif
  return int32_t((i4 << 8) + i5 + b6 - 0x4F400000u);
}
__host__ __device__ __forceinline__ int64_t combine_g(int32_t g3, int32_t g2, int32_t g1) {
  return (int64_t(g3) << 32) + (int64_t(g2) << 16) + int64_t(g1);
}
__host__ __device__ __forceinline__ int64_t combine7(const float D[7]) {
  int32_t g3, g2;
  combine_hi(D[0], D[1], D[2], D[3], g3, g2);
  return combine_g(g3, g2, combine_lo(D[4], D[5], D[6]));
}

// acc += the contribution of diagonal d of an ND-digit product whose f32 sum
// is D (the forms of accumulate<d> above, weights 2^(8 (ND - 2 - d))).
template <int ND, int d>
__host__ __device__ __forceinline__ void accumulate_nd(int64_t& acc, float D) {
  if constexpr (d < 4) {
    const int32_t v = int32_t(f32_bits(add_rn(D, f32_of(0x4B400000u))) - 0x4B400000u);
    acc += int64_t(v) * (int64_t(1) << (8 * (ND - 2 - d)));
  } else if constexpr (d < ND - 1) {
#ifdef __CUDA_ARCH__
    const int32_t v = __float2int_rn(D);
#else
    const int32_t v = int32_t(D);
#endif
    acc += int64_t(v) * (int64_t(1) << (8 * (ND - 2 - d)));
  } else {
    const int32_t v = int32_t(f32_bits(add_rn(D, f32_of(0x4F400000u))) - 0x4F400000u);
    acc += int64_t(v);
  }
}

// The six-digit grouped form: (g3, g2) from D0..D3 as combine_hi forms them,
// g0 = I4 + round(D5 / 2^8) (< 2^23), acc = 2^24 g3 + 2^8 g2 + g0.
__host__ __device__ __forceinline__ int32_t combine_lo6(float D4, float D5) {
  const uint32_t b5 = f32_bits(add_rn(D5, f32_of(0x4F400000u)));
#ifdef __CUDA_ARCH__
  const uint32_t i4 = uint32_t(__float2int_rn(D4));
#else
  const uint32_t i4 = uint32_t(int32_t(D4));
#endif
  return int32_t(i4 + b5 - 0x4F400000u);
}
__host__ __device__ __forceinline__ int64_t combine_g6(int32_t g3, int32_t g2, int32_t g0) {
  return (int64_t(g3) << 24) + (int64_t(g2) << 8) + int64_t(g0);
}

template <int ND>
__host__ __device__ __forceinline__ int64_t combine_nd(const float* D) {
  int32_t g3, g2;
  combine_hi(D[0], D[1], D[2], D[3], g3, g2);
  if constexpr (ND == 7)
    return combine_g(g3, g2, combine_lo(D[4], D[5], D[6]));
  else
    return combine_g6(g3, g2, combine_lo6(D[4], D[5]));
}

// acc * 2^pow2 as an f64 (|acc| < 2^62), rounded to nearest even once,
// assembled from acc's bits.
__host__ __device__ __forceinline__ double scaled(int64_t acc, int pow2) {
  if (acc == 0) return 0.0;
  const uint64_t sign = uint64_t(acc) & 0x8000000000000000ull;
  const uint64_t mag = acc < 0 ? uint64_t(-acc) : uint64_t(acc);
#ifdef __CUDA_ARCH__
  const int lz = __clzll(int64_t(mag));
#else
  const int lz = __builtin_clzll(mag);
#endif
  const int eb = 1086 - lz + pow2;  // biased exponent of the result
  if (eb <= 0 || eb >= 2047) {      // subnormal or out of range: rare, FP64 path
#ifdef __CUDA_ARCH__
    return scalbn(__ll2double_rn(acc), pow2);
#else
    return std::scalbn(double(acc), pow2);
#endif
  }
  const uint64_t norm = mag << lz;  // leading one at bit 63
  uint64_t mant = norm >> 11;       // 53 bits
  const uint64_t rest = norm & 0x7FFu;
  mant += (rest > 0x400u || (rest == 0x400u && (mant & 1))) ? 1 : 0;
  // a carry out of the mantissa moves into the exponent field, as it should
  const uint64_t bits = sign | ((uint64_t(eb - 1) << 52) + mant);
  double y;
  std::memcpy(&y, &bits, 8);
  return y;
}

#ifdef __CUDACC__
// The same value as scaled(), formed on the FP64 pipe: the conversion of acc
// rounds to nearest even as scaled() does, and a power-of-two scaling that
// keeps the result normal is exact, an exponent-field add.  The complex128
// fused pass sends part of its outputs here, where the FP64 pipe is idle
// while the integer pipes recombine.
__device__ __forceinline__ double scaled_fp64(int64_t acc, int pow2) {
  const double x = __ll2double_rn(acc);
  const uint64_t b = uint64_t(__double_as_longlong(x));
  const int e = int((b >> 52) & 0x7FFu);
  if (acc == 0 || e + pow2 <= 0 || e + pow2 >= 2047) return acc == 0 ? 0.0 : scalbn(x, pow2);
  return __longlong_as_double((long long)(b + (uint64_t(int64_t(pow2)) << 52)));
}
#endif

// Largest biased exponent among 64-bit values given by their high words.
__host__ __device__ __forceinline__ int exp_of(uint32_t hi) { return int((hi >> 20) & 0x7FFu); }

}  // namespace oz
}  // namespace ev
