// ev_measure.cu -- FP64 reductions, Born-rule measurement, collapse and
// shot sampling.
//
// measure_qubit (src/measure.rs:15-51) makes two passes: p1 = sum of
// |a_j|^2 over j with bit k set, then outcome = u < p1 and the surviving half
// is scaled by 1/sqrt(surviving) while the other half is zeroed.  Here:
//   pass 1  k_reduce<P1>  one HBM read of the bit-k half; fixed-order block
//                         partials, so results are deterministic run to run
//   decide  k_decide      one thread: the reference's outcome and scale
//                         formulas, with IEEE sqrt and division
//   pass 2  k_collapse    reads only the kept half, writes both halves
// The sum order differs from the reference's left-to-right loop, so p1 (and
// the scale) agree to rounding (~1e-16 relative), not bit for bit; outcomes
// agree unless u lies within that rounding of p1.
//
// State observables (src/state.rs:94-185) use the same reduction with other
// terms.  Every reduction accumulates in f64 for both storage types.
#include <cmath>
#include <cstring>
#include <mutex>

#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_softfp.cuh"

namespace ev {

enum RedOp { R_NORM = 0, R_P1, R_BLOCH, R_OVERLAP };

constexpr int kRedThreads = 256;

template <int OP, typename V>
__device__ __forceinline__ void red_term(const V* __restrict__ a, const V* __restrict__ b,
                                         uint64_t i, int k, double acc[4]) {
  if constexpr (OP == R_NORM) {
    acc[0] += nsq(a[i]);
  } else if constexpr (OP == R_P1) {
    acc[0] += nsq(a[insert0(i, k) | (uint64_t(1) << k)]);
  } else if constexpr (OP == R_BLOCH) {
    const uint64_t j0 = insert0(i, k), j1 = j0 | (uint64_t(1) << k);
    const V x = a[j0], y = a[j1];
    const double2 x2 = make_double2(x.x, x.y), y2 = make_double2(y.x, -double(y.y));
    acc[0] += nsq(x2);
    acc[1] += nsq(y2);
    const double2 r = cmul(x2, y2);  // amp * partner.conj()
    acc[2] += r.x;
    acc[3] += r.y;
  } else {  // R_OVERLAP: conj(other_j) * self_j
    const V x = a[i], y = b[i];
    const double2 r = cmul(make_double2(y.x, -double(y.y)), make_double2(x.x, x.y));
    acc[0] += r.x;
    acc[1] += r.y;
  }
}

// Block-wide sum of 4 per-thread accumulators in a fixed tree order; thread
// 0..3 write the block's partials.
__device__ __forceinline__ void block_partials(double acc[4], double* __restrict__ partials) {
  __shared__ double sh[4][kRedThreads];
#pragma unroll
  for (int c = 0; c < 4; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int c = 0; c < 4; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 4) partials[blockIdx.x * 4 + threadIdx.x] = sh[threadIdx.x][0];
}

// Block b reduces the contiguous counter range [b*chunk, (b+1)*chunk) and
// writes 4 partials; the tree inside the block has a fixed shape.  (Bloch
// vectors and complex128 overlaps; the hot sums have kernels of their own
// below.)
template <int OP, typename V>
__global__ void __launch_bounds__(kRedThreads)
    k_reduce(const V* __restrict__ a, const V* __restrict__ b, uint64_t count, uint64_t chunk,
             int k, double* __restrict__ partials, const uint8_t* pred) {
  if (pred != nullptr && *pred == 0) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += kRedThreads) red_term<OP>(a, b, i, k, acc);
  block_partials(acc, partials);
}

// Terms are taken in pairs (2q, 2q+1) so that every access is a 16-byte (or
// 32-byte) contiguous load; a block's range starts on an even term.
constexpr int kFlush = 32;  // pairs per double-float run before the f64 flush

__device__ __forceinline__ float4 ld4(const float2* p) { return *reinterpret_cast<const float4*>(p); }

// The two amplitudes of terms 2q, 2q+1: all amplitudes (norm) or those with
// bit k set (p1).
template <int OP, typename V>
__device__ __forceinline__ void sq_pair(const V* __restrict__ a, uint64_t q, int k, V* t0, V* t1) {
  if constexpr (OP == R_NORM) {
    *t0 = a[2 * q];
    *t1 = a[2 * q + 1];
  } else {
    if (k > 0) {
      const uint64_t j = insert0(2 * q, k) | (uint64_t(1) << k);
      *t0 = a[j];
      *t1 = a[j + 1];
    } else {
      *t0 = a[4 * q + 1];
      *t1 = a[4 * q + 3];
    }
  }
}

// Sum of |a_j|^2 (norm, p1).  complex64: double-float on the FP32 pipe,
// flushed to f64 every kFlush pairs (agrees with an f64 sum to ~1e-14
// relative); complex128: two f64 FMAs per amplitude.  Each thread issues a
// group of kGroup loads before any arithmetic, so enough bytes are in flight
// to cover HBM latency.
constexpr int kGroup = 8;

template <int OP>
__device__ __forceinline__ float4 sq_load_c64(const float2* __restrict__ a, uint64_t q, int k) {
  if (OP == R_NORM) return ld4(a + 2 * q);
  if (k > 0) return ld4(a + (insert0(2 * q, k) | (uint64_t(1) << k)));
  const float4 u0 = ld4(a + 4 * q), u1 = ld4(a + 4 * q + 2);
  return make_float4(u0.z, u0.w, u1.z, u1.w);
}

template <int OP, typename V>
__global__ void __launch_bounds__(kRedThreads)
    k_reduce_sq(const V* __restrict__ a, uint64_t count, uint64_t chunk, int k,
                double* __restrict__ partials, const uint8_t* pred) {
  if (pred != nullptr && *pred == 0) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  const uint64_t q0 = lo / 2, q1 = hi / 2;
  for (uint64_t base = q0 + threadIdx.x; base < q1; base += uint64_t(kFlush) * kRedThreads) {
    if constexpr (sizeof(V) == 8) {
      const float2* af = reinterpret_cast<const float2*>(a);
      FF f;
      for (int g = 0; g < kFlush; g += kGroup) {
        float4 v[kGroup];
#pragma unroll
        for (int r = 0; r < kGroup; ++r) {
          const uint64_t q = base + uint64_t(g + r) * kRedThreads;
          v[r] = q < q1 ? sq_load_c64<OP>(af, q, k) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < kGroup; ++r) {
          f.add_prod(v[r].x, v[r].x);
          f.add_prod(v[r].y, v[r].y);
          f.add_prod(v[r].z, v[r].z);
          f.add_prod(v[r].w, v[r].w);
        }
      }
      acc[0] += f.value();
    } else {
      for (int g = 0; g < kFlush; g += kGroup) {
        V t[kGroup][2];
#pragma unroll
        for (int r = 0; r < kGroup; ++r) {
          const uint64_t q = base + uint64_t(g + r) * kRedThreads;
          if (q < q1) {
            sq_pair<OP>(a, q, k, &t[r][0], &t[r][1]);
          } else {
            t[r][0] = t[r][1] = make_double2(0.0, 0.0);
          }
        }
#pragma unroll
        for (int r = 0; r < kGroup; ++r) {
          acc[r & 1] = __fma_rn(t[r][0].x, t[r][0].x, acc[r & 1]);
          acc[r & 1] = __fma_rn(t[r][0].y, t[r][0].y, acc[r & 1]);
          acc[r & 1] = __fma_rn(t[r][1].x, t[r][1].x, acc[r & 1]);
          acc[r & 1] = __fma_rn(t[r][1].y, t[r][1].y, acc[r & 1]);
        }
      }
    }
  }
  // an odd count leaves one term for the last block
  if ((count & 1) && hi == count && hi > lo && threadIdx.x == 0) {
    const uint64_t i = count - 1;
    const V x = OP == R_NORM ? a[i] : a[insert0(i, k) | (uint64_t(1) << k)];
    acc[2] += nsq(x);
  }
  acc[0] += acc[1] + acc[2];
  acc[1] = acc[2] = 0.0;
  block_partials(acc, partials);
}

// <other|self> for two complex128 states: re and im each as a chain of f64
// FMAs (4 per amplitude instead of a complex product and two adds).
__global__ void __launch_bounds__(kRedThreads)
    k_overlap_c128(const double2* __restrict__ a, const double2* __restrict__ b, uint64_t count,
                   uint64_t chunk, double* __restrict__ partials) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  for (uint64_t base = lo + threadIdx.x; base < hi; base += uint64_t(kGroup) * kRedThreads) {
    double2 x[kGroup], y[kGroup];
#pragma unroll
    for (int r = 0; r < kGroup; ++r) {
      const uint64_t i = base + uint64_t(r) * kRedThreads;
      x[r] = i < hi ? a[i] : make_double2(0.0, 0.0);
      y[r] = i < hi ? b[i] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int r = 0; r < kGroup; ++r) {
      acc[0] = __fma_rn(y[r].x, x[r].x, acc[0]);
      acc[0] = __fma_rn(y[r].y, x[r].y, acc[0]);
      acc[1] = __fma_rn(y[r].x, x[r].y, acc[1]);
      acc[1] = __fma_rn(-y[r].y, x[r].x, acc[1]);
    }
  }
  block_partials(acc, partials);
}

// <other|self> = sum conj(other_j) * self_j for two complex64 states:
// double-float products and sums, flushed to f64 every kFlush pairs.
__global__ void __launch_bounds__(kRedThreads)
    k_overlap_c64(const float2* __restrict__ a, const float2* __restrict__ b, uint64_t count,
                  uint64_t chunk, double* __restrict__ partials) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  const uint64_t q0 = lo / 2, q1 = hi / 2;
  for (uint64_t base = q0 + threadIdx.x; base < q1; base += uint64_t(kFlush) * kRedThreads) {
    FF re, im;
#pragma unroll 4
    for (int r = 0; r < kFlush; ++r) {
      const uint64_t q = base + uint64_t(r) * kRedThreads;
      if (q < q1) {
        const float4 x = ld4(a + 2 * q), y = ld4(b + 2 * q);
        re.add_prod(y.x, x.x);
        re.add_prod(y.y, x.y);
        im.add_prod(y.x, x.y);
        im.add_prod(-y.y, x.x);
        re.add_prod(y.z, x.z);
        re.add_prod(y.w, x.w);
        im.add_prod(y.z, x.w);
        im.add_prod(-y.w, x.z);
      }
    }
    acc[0] += re.value();
    acc[1] += im.value();
  }
  if ((count & 1) && hi == count && hi > lo && threadIdx.x == 0) {
    const float2 x = a[count - 1], y = b[count - 1];
    const double2 r = cmul(make_double2(y.x, -double(y.y)), make_double2(x.x, x.y));
    acc[0] += r.x;
    acc[1] += r.y;
  }
  block_partials(acc, partials);
}

// <other|self> for states of different amplitude types (both promoted to f64).
template <typename VA, typename VB>
__global__ void __launch_bounds__(kRedThreads)
    k_overlap_mixed(const VA* __restrict__ a, const VB* __restrict__ b, uint64_t count,
                    uint64_t chunk, double* __restrict__ partials) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += kRedThreads) {
    const VA x = a[i];
    const VB y = b[i];
    const double2 r = cmul(make_double2(double(y.x), -double(y.y)), make_double2(double(x.x), double(x.y)));
    acc[0] += r.x;
    acc[1] += r.y;
  }
  __shared__ double sh[2][kRedThreads];
  sh[0][threadIdx.x] = acc[0];
  sh[1][threadIdx.x] = acc[1];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partials[blockIdx.x * 4 + threadIdx.x] = threadIdx.x < 2 ? sh[threadIdx.x][0] : 0.0;
}

// Sums nblocks x 4 partials in a fixed order into result[0..4).
__global__ void __launch_bounds__(kRedThreads)
    k_finish(const double* __restrict__ partials, int nblocks, double* __restrict__ result,
             const uint8_t* pred) {
  if (pred != nullptr && *pred == 0) return;
  __shared__ double sh[4][kRedThreads];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblocks; b += kRedThreads)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c] += partials[b * 4 + c];
#pragma unroll
  for (int c = 0; c < 4; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int c = 0; c < 4; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 4) result[threadIdx.x] = sh[threadIdx.x][0];
}

// outcome = u < p1; surviving = outcome ? p1 : 1 - p1;
// scale = surviving > 0 ? 1/sqrt(surviving) : 0   (measure.rs:29-38).
__global__ void k_decide(const double* __restrict__ result, double u_host,
                         const double* __restrict__ u_dev, uint32_t* __restrict__ counter,
                         double* __restrict__ meas, uint8_t* __restrict__ outcome_dev,
                         const uint8_t* pred) {
  if (pred != nullptr && *pred == 0) return;
  const double p1 = result[0];
  double u = u_host;
  if (u_dev != nullptr) u = u_dev[counter[0]++];
  const bool outcome = u < p1;
  const double surviving = outcome ? p1 : __dadd_rn(1.0, -p1);
  const double scale = surviving > 0.0 ? __ddiv_rn(1.0, __dsqrt_rn(surviving)) : 0.0;
  meas[0] = p1;
  meas[1] = scale;
  meas[2] = outcome ? 1.0 : 0.0;
  meas[3] = u;
  if (outcome_dev != nullptr) *outcome_dev = outcome ? 1 : 0;
}

// Rescaling by an f64 factor: complex128 multiplies in f64 (Complex64 * f64,
// complex.rs:127-133).  complex64 applies the factor as a float pair
// s ~ sh + sl: x*sh is taken exactly inside an FMA with x*sl added, so each
// amplitude is rounded once from (nearly) x*s -- no systematic bias from a
// rounded factor, and the FP64 pipe stays idle.
template <typename V>
__device__ __forceinline__ V scale_amp(V a, double s) {
  if constexpr (sizeof(V) == 16) {
    return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s));
  } else {
    const float sh = float(s);
    const float sl = float(s - double(sh));
    return make_float2(__fmaf_rn(a.x, sh, __fmul_rn(a.x, sl)), __fmaf_rn(a.y, sh, __fmul_rn(a.y, sl)));
  }
}

// Pass 2 of measure_qubit (measure.rs:40-48).
template <typename V>
__global__ void __launch_bounds__(256)
    k_collapse(V* __restrict__ a, uint64_t npairs, int k, const double* __restrict__ meas,
               const uint8_t* pred) {
  if (pred != nullptr && *pred == 0) return;
  const double scale = meas[1];
  const bool one = meas[2] != 0.0;
  const uint64_t bit = uint64_t(1) << k;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  V zero;
  zero.x = 0;
  zero.y = 0;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < npairs; i += stride) {
    const uint64_t j0 = insert0(i, k), j1 = j0 | bit;
    const uint64_t keep = one ? j1 : j0, drop = one ? j0 : j1;
    a[keep] = scale_amp(a[keep], scale);
    a[drop] = zero;
  }
}

// State::normalize (state.rs:103-111): norm = sqrt(norm_sqr); inv = 1/norm.
template <typename V>
__global__ void __launch_bounds__(256)
    k_normalize(V* __restrict__ a, uint64_t len, const double* __restrict__ result) {
  const double norm = __dsqrt_rn(result[0]);
  if (!(norm > 0.0)) return;
  const double inv = __ddiv_rn(1.0, norm);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < len; j += stride)
    a[j] = scale_amp(a[j], inv);
}

__global__ void k_pred_and(const uint8_t* __restrict__ classical, const uint64_t* bits, int nbits,
                           uint8_t* out) {
  uint8_t v = 1;
  for (int i = 0; i < nbits; ++i) v = v && classical[bits[i]];
  *out = v;
}

// ---- sampling tree --------------------------------------------------------
// mass level q (2^q entries) lives at offset 2^q, so every level starts on a
// 2^q x 8-byte boundary and a warp's run of entries covers whole 32-byte
// sectors (entry 0 of the 2^n-double buffer is unused).  mass[n-1][r] =
// |a_r|^2 + |a_{r+2^(n-1)}|^2 and mass[q][r] = mass[q+1][r] + mass[q+1][r+2^q].

// complex128 leaves use the oracle's arithmetic (nsq + nsq, f64; the plain
// product inside nsq formed on the integer pipes), so shots match its tree
// exactly; complex64 leaves are the double-float sum of the four exact float
// squares, rounded to f64 once (~1e-14 relative) on the integer pipes.
// nsq(a) = fma(x, x, y*y) with the plain product y*y formed on the integer
// pipes when y is in the integer product's range (the same bits).
__device__ __forceinline__ double nsq_soft(double2 a) {
  const softfp::Unpacked uy = softfp::unpack(a.y);
  const double yy = uy.ok ? softfp::mul(uy, uy) : __dmul_rn(a.y, a.y);
  return __fma_rn(a.x, a.x, yy);
}
__device__ __forceinline__ double leaf_mass(double2 u, double2 v) {
  return __dadd_rn(nsq_soft(u), nsq_soft(v));
}
__device__ __forceinline__ double leaf_mass(float2 u, float2 v) {
  FF f;
  f.add_prod(u.x, u.x);
  f.add_prod(u.y, u.y);
  f.add_prod(v.x, v.x);
  f.add_prod(v.y, v.y);
  return ff_to_f64(f.hi, f.lo);  // = f.value(), with the final add on the integer pipes
}

template <typename V>
__global__ void __launch_bounds__(256)
    k_mass_leaf(const V* __restrict__ a, uint64_t half, double* __restrict__ out) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < half; r += stride)
    out[r] = leaf_mass(a[r], a[r + half]);
}

__global__ void __launch_bounds__(256)
    k_mass_level(const double* __restrict__ in, uint64_t w, double* __restrict__ out) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < w; r += stride)
    out[r] = __dadd_rn(in[r], in[r + w]);
}

// Several levels per pass.  Level q holds 2^q sums at mass + 2^q, entry
// e = level q+1 entry e + level q+1 entry e + 2^q.  The entries of L
// consecutive levels that end in entry r of the lowest of them form a
// subtree over the 2^L source entries r + j S of the level above them
// (S = the lowest level's width), so one thread reads those 2^L values once,
// forms the subtree with the same sums in the same order as level by level,
// and writes every level of it: each level is written once and no level but
// the source is read.

// Levels n-1 (leaves) .. n-L from the amplitudes.  Each thread takes two
// neighbouring source columns r, r + 1 (r even): its amplitude loads and its
// tree stores move 16 bytes each (two complex64 amplitudes; two f64 entries,
// aligned because every level starts at 2^q), half the memory instructions
// of one column per thread.  The sums are the same, in the same order.
template <typename V>
struct Amp2;  // two consecutive amplitudes as one vector access
template <>
struct Amp2<float2> {
  using T = float4;
  __device__ static void split(const float4& v, float2& a, float2& b) {
    a = make_float2(v.x, v.y);
    b = make_float2(v.z, v.w);
  }
};
template <>
struct Amp2<double2> {
  struct T {
    double2 a, b;
  };
  __device__ static void split(const T& v, double2& a, double2& b) {
    a = v.a;
    b = v.b;
  }
};

template <typename V, int L>
__global__ void __launch_bounds__(256)
    k_mass_leaf_fused(const V* __restrict__ a, int n, double* __restrict__ mass) {
  constexpr int C = 1 << (L - 1);  // leaves per column
  using A2 = Amp2<V>;
  const uint64_t S = uint64_t(1) << (n - L);
  const uint64_t half = uint64_t(1) << (n - 1);
  const uint64_t stride = 2 * uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t r = 2 * (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x); r < S; r += stride) {
    V lo0[C], lo1[C], hi0[C], hi1[C];
#pragma unroll
    for (int j = 0; j < C; ++j) {
      if constexpr (sizeof(V) == 8) {
        A2::split(*reinterpret_cast<const float4*>(a + r + uint64_t(j) * S), lo0[j], lo1[j]);
        A2::split(*reinterpret_cast<const float4*>(a + r + uint64_t(j) * S + half), hi0[j], hi1[j]);
      } else {
        lo0[j] = a[r + uint64_t(j) * S];
        lo1[j] = a[r + 1 + uint64_t(j) * S];
        hi0[j] = a[r + uint64_t(j) * S + half];
        hi1[j] = a[r + 1 + uint64_t(j) * S + half];
      }
    }
    double m0[C], m1[C];
#pragma unroll
    for (int j = 0; j < C; ++j) {
      m0[j] = leaf_mass(lo0[j], hi0[j]);
      m1[j] = leaf_mass(lo1[j], hi1[j]);
      *reinterpret_cast<double2*>(mass + half + r + uint64_t(j) * S) = make_double2(m0[j], m1[j]);
    }
#pragma unroll
    for (int lev = 1; lev < L; ++lev) {
      const int cnt = C >> lev;
      const uint64_t w = uint64_t(cnt) * S;
#pragma unroll
      for (int j = 0; j < cnt; ++j) {
        m0[j] = __dadd_rn(m0[j], m0[j + cnt]);
        m1[j] = __dadd_rn(m1[j], m1[j + cnt]);
        *reinterpret_cast<double2*>(mass + w + r + uint64_t(j) * S) = make_double2(m0[j], m1[j]);
      }
    }
  }
}

// Levels qsrc-1 .. qsrc-L from level qsrc, two columns per thread as above.
template <int L>
__global__ void __launch_bounds__(256) k_mass_level_fused(double* __restrict__ mass, int qsrc) {
  constexpr int C = 1 << L;  // source entries per column
  const uint64_t S = uint64_t(1) << (qsrc - L);
  const double* __restrict__ src = mass + (uint64_t(1) << qsrc);
  const uint64_t stride = 2 * uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t r = 2 * (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x); r < S; r += stride) {
    double m0[C], m1[C];
#pragma unroll
    for (int j = 0; j < C; ++j) {
      const double2 v = *reinterpret_cast<const double2*>(src + r + uint64_t(j) * S);
      m0[j] = v.x;
      m1[j] = v.y;
    }
#pragma unroll
    for (int lev = 1; lev <= L; ++lev) {
      const int cnt = C >> lev;
      const uint64_t w = uint64_t(cnt) * S;
#pragma unroll
      for (int j = 0; j < cnt; ++j) {
        m0[j] = __dadd_rn(m0[j], m0[j + cnt]);
        m1[j] = __dadd_rn(m1[j], m1[j + cnt]);
        *reinterpret_cast<double2*>(mass + w + r + uint64_t(j) * S) = make_double2(m0[j], m1[j]);
      }
    }
  }
}

// Levels top..0 of the tree in one block (level top already built).
__global__ void __launch_bounds__(1024) k_mass_top(double* __restrict__ mass, int top) {
  for (int q = top - 1; q >= 0; --q) {
    const uint64_t w = uint64_t(1) << q;
    const double* in = mass + 2 * w;
    double* out = mass + w;
    for (uint64_t r = threadIdx.x; r < w; r += blockDim.x) out[r] = __dadd_rn(in[r], in[r + w]);
    __syncthreads();
  }
}

// One thread per shot: descend the tree with n uniforms (qubits 0..n-1).
template <typename V>
__global__ void __launch_bounds__(256)
    k_descend(const double* __restrict__ mass, const V* __restrict__ a, int n,
              const double* __restrict__ uni, uint64_t shots, uint64_t* __restrict__ out) {
  const uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= shots) return;
  uint64_t r = 0;
  for (int q = 0; q < n; ++q) {
    const uint64_t w = uint64_t(1) << q;
    const double m = mass[w + r];
    const double m1 = (q + 1 < n) ? mass[2 * w + r + w] : nsq(a[r + w]);
    const double p1 = __ddiv_rn(m1, m);
    if (uni[s * uint64_t(n) + q] < p1) r |= w;
  }
  out[s] = r;
}

// ---- host ------------------------------------------------------------------

// Blocks and the (even) per-block term range of a reduction over count terms:
// one block per 4096 terms, at most per_sm blocks on each SM.
static void red_grid(uint64_t count, int sms, int per_sm, int max_blocks, int* nb_out,
                     uint64_t* chunk_out) {
  const uint64_t want = (count + 4095) / 4096;
  int nb = int(want < 1 ? 1 : want);
  int cap = sms * per_sm < kMaxRedBlocks ? sms * per_sm : kMaxRedBlocks;
  if (cap > max_blocks) cap = max_blocks;
  if (nb > cap) nb = cap;
  uint64_t chunk = (count + nb - 1) / nb;
  chunk = (chunk + 1) & ~uint64_t(1);
  *nb_out = nb;
  *chunk_out = chunk;
}

template <int OP>
static int reduce(const ev_state* s, const ev_state* other, uint64_t count, int k,
                  const uint8_t* pred) {
  int nb = 0;
  uint64_t chunk = 0;
  const bool c128 = s->dtype == EV_C128;
  if constexpr (OP == R_NORM || OP == R_P1) {
    if (c128) {
      red_grid(count, s->num_sms, resident_blocks<k_reduce_sq<OP, double2>>(), kMaxRedBlocks, &nb,
               &chunk);
      k_reduce_sq<OP, double2><<<nb, kRedThreads, 0, s->stream>>>(
          static_cast<const double2*>(s->amps), count, chunk, k, s->scratch.partials, pred);
    } else {
      red_grid(count, s->num_sms, resident_blocks<k_reduce_sq<OP, float2>>(), kMaxRedBlocks, &nb,
               &chunk);
      k_reduce_sq<OP, float2><<<nb, kRedThreads, 0, s->stream>>>(
          static_cast<const float2*>(s->amps), count, chunk, k, s->scratch.partials, pred);
    }
  } else if (OP == R_OVERLAP && !c128) {
    red_grid(count, s->num_sms, resident_blocks<k_overlap_c64>(), kMaxRedBlocks, &nb, &chunk);
    k_overlap_c64<<<nb, kRedThreads, 0, s->stream>>>(static_cast<const float2*>(s->amps),
                                                    static_cast<const float2*>(other->amps), count,
                                                    chunk, s->scratch.partials);
  } else if (OP == R_OVERLAP) {
    red_grid(count, s->num_sms, resident_blocks<k_overlap_c128>(), kMaxRedBlocks, &nb, &chunk);
    k_overlap_c128<<<nb, kRedThreads, 0, s->stream>>>(static_cast<const double2*>(s->amps),
                                                     static_cast<const double2*>(other->amps), count,
                                                     chunk, s->scratch.partials);
  } else if (c128) {
    red_grid(count, s->num_sms, resident_blocks<k_reduce<OP, double2>>(), kMaxRedBlocks, &nb,
             &chunk);
    k_reduce<OP, double2><<<nb, kRedThreads, 0, s->stream>>>(
        static_cast<const double2*>(s->amps),
        other ? static_cast<const double2*>(other->amps) : nullptr, count, chunk, k,
        s->scratch.partials, pred);
  } else {
    red_grid(count, s->num_sms, resident_blocks<k_reduce<OP, float2>>(), kMaxRedBlocks, &nb,
             &chunk);
    k_reduce<OP, float2><<<nb, kRedThreads, 0, s->stream>>>(
        static_cast<const float2*>(s->amps),
        other ? static_cast<const float2*>(other->amps) : nullptr, count, chunk, k,
        s->scratch.partials, pred);
  }
  k_finish<<<1, kRedThreads, 0, s->stream>>>(s->scratch.partials, nb, s->scratch.result, pred);
  s->launches += 2;
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

static unsigned grid_for(const ev_state* s, uint64_t work, int per_sm = 8) {
  const uint64_t want = (work + 255) / 256;
  const uint64_t cap = uint64_t(s->num_sms) * uint64_t(per_sm);
  return unsigned(want < 1 ? 1 : (want < cap ? want : cap));
}

int launch_measure(ev_state* s, uint64_t k, double u_host, const double* u_dev,
                   uint8_t* outcome_dev, const uint8_t* pred) {
  // pass 1 reads the bit-k half; pass 2 reads the kept half and writes all
  ProfScope prof(s, P_MEASURE, 2.0 * double(s->len()) * double(s->amp_bytes()));
  s->launches += 2;
  EV_TRY(reduce<R_P1>(s, nullptr, s->len() / 2, int(k), pred));
  k_decide<<<1, 1, 0, s->stream>>>(s->scratch.result, u_host, u_dev, s->scratch.counter,
                                   s->scratch.meas, outcome_dev, pred);
  const uint64_t np = s->len() / 2;
  if (s->dtype == EV_C128)
    k_collapse<double2><<<grid_for(s, np), 256, 0, s->stream>>>(
        static_cast<double2*>(s->amps), np, int(k), s->scratch.meas, pred);
  else
    k_collapse<float2><<<grid_for(s, np), 256, 0, s->stream>>>(
        static_cast<float2*>(s->amps), np, int(k), s->scratch.meas, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int launch_pred_and(ev_state* s, const uint8_t* classical, const uint64_t* bits, int nbits,
                    uint8_t* pred_out) {
  k_pred_and<<<1, 1, 0, s->stream>>>(classical, bits, nbits, pred_out);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

static int fetch_result(const ev_state* s, double* out, int count) {
  EV_CUDA(cudaMemcpyAsync(out, s->scratch.result, sizeof(double) * count, cudaMemcpyDeviceToHost,
                          s->stream));
  EV_CUDA(cudaStreamSynchronize(s->stream));
  return EV_OK;
}

int reduce_norm(const ev_state* s, double* out_host) {
  EV_TRY(reduce<R_NORM>(s, nullptr, s->len(), 0, nullptr));
  return fetch_result(s, out_host, 1);
}

static int ensure_mass(ev_state* s) {
  const uint64_t need = s->len();
  if (s->mass && s->mass_len >= need) return EV_OK;
  if (s->mass) cudaFreeAsync(s->mass, s->stream);
  s->mass = nullptr;
  s->mass_len = 0;
  void* p = nullptr;
  EV_CUDA(cudaMallocAsync(&p, need * sizeof(double), s->stream));
  s->mass = static_cast<double*>(p);
  s->mass_len = need;
  return EV_OK;
}

static int build_mass(ev_state* s) {
  const int n = int(s->n);
  // the amplitudes read once, the 2^n - 1 tree entries written once
  ProfScope prof(s, P_SAMPLE, double(s->len()) * double(s->amp_bytes()) + 8.0 * double(s->len()));
  constexpr int L = 4;   // levels per pass
  constexpr int LL = 4;  // levels of the leaf pass (three measured slower at 30 qubits)
  double* mass = s->mass;
  const uint64_t half = s->len() / 2;
  int q;  // highest level still to build
  if (n - LL >= 12) {
    const uint64_t S = uint64_t(1) << (n - LL);  // columns, two per thread
    // (the complex128 instance holds ~150 registers, one block per SM at a
    // time; a 3-block budget spills and measured slower: 6.31 vs 5.43 ms)
    if (s->dtype == EV_C128)
      k_mass_leaf_fused<double2, LL>
          <<<grid_for(s, S / 2, resident_blocks<k_mass_leaf_fused<double2, LL>>()), 256, 0,
             s->stream>>>(static_cast<const double2*>(s->amps), n, mass);
    else
      k_mass_leaf_fused<float2, LL>
          <<<grid_for(s, S / 2, resident_blocks<k_mass_leaf_fused<float2, LL>>()), 256, 0,
             s->stream>>>(static_cast<const float2*>(s->amps), n, mass);
    s->launches += 1;
    q = n - 1 - LL;
  } else {
    double* top = mass + half;  // level n-1
    if (s->dtype == EV_C128)
      k_mass_leaf<double2><<<grid_for(s, half), 256, 0, s->stream>>>(
          static_cast<const double2*>(s->amps), half, top);
    else
      k_mass_leaf<float2><<<grid_for(s, half), 256, 0, s->stream>>>(
          static_cast<const float2*>(s->amps), half, top);
    s->launches += 1;
    q = n - 2;
  }
  for (; q - (L - 1) >= 12; q -= L) {
    k_mass_level_fused<L><<<grid_for(s, uint64_t(1) << (q - L)), 256, 0, s->stream>>>(mass,
                                                                                      q + 1);
    s->launches += 1;
  }
  for (; q >= 12; --q) {
    const uint64_t w = uint64_t(1) << q;
    k_mass_level<<<grid_for(s, w), 256, 0, s->stream>>>(mass + 2 * w, w, mass + w);
    s->launches += 1;
  }
  if (q >= 0) {
    k_mass_top<<<1, 1024, 0, s->stream>>>(mass, q + 1);
    s->launches += 1;
  }
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

}  // namespace ev

using namespace ev;

extern "C" int ev_measure_qubit(ev_state* s, uint64_t k, double u, int32_t* outcome) {
  clear_error();
  if (!s || !outcome) return fail(EV_ERR_INVALID_ARGUMENT, "ev_measure_qubit: null argument");
  if (k >= s->n)
    return fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                (unsigned long long)k, (unsigned long long)s->n);
  EV_CUDA(cudaSetDevice(s->device));
  EV_TRY(launch_measure(s, k, u, nullptr, nullptr, nullptr));
  double meas[4];
  EV_CUDA(cudaMemcpyAsync(meas, s->scratch.meas, sizeof(meas), cudaMemcpyDeviceToHost, s->stream));
  EV_CUDA(cudaStreamSynchronize(s->stream));
  *outcome = meas[2] != 0.0 ? 1 : 0;
  return EV_OK;
}

extern "C" int ev_norm_sqr(const ev_state* s, double* out) {
  clear_error();
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_norm_sqr: null argument");
  EV_CUDA(cudaSetDevice(s->device));
  return reduce_norm(s, out);
}

int ev::launch_normalize(ev_state* s) {
  ProfScope prof(s, P_OTHER, 3.0 * double(s->len()) * double(s->amp_bytes()));
  EV_TRY(reduce<R_NORM>(s, nullptr, s->len(), 0, nullptr));
  s->launches += 1;
  if (s->dtype == EV_C128)
    k_normalize<double2><<<grid_for(s, s->len()), 256, 0, s->stream>>>(
        static_cast<double2*>(s->amps), s->len(), s->scratch.result);
  else
    k_normalize<float2><<<grid_for(s, s->len()), 256, 0, s->stream>>>(
        static_cast<float2*>(s->amps), s->len(), s->scratch.result);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

extern "C" int ev_normalize(ev_state* s) {
  clear_error();
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "ev_normalize: null argument");
  EV_CUDA(cudaSetDevice(s->device));
  EV_TRY(launch_normalize(s));
  EV_CUDA(cudaStreamSynchronize(s->stream));
  return EV_OK;
}

// Marginal distribution of the low m qubits: out[c] = sum over the high bits
// t of norm_sqr(a[t * 2^m + c]), each sum taken in increasing t from 0.0 --
// the order of the basis loop in phase_estimation.rs:97-110
// (most_probable_phase).  One thread per c; the loads of a warp are
// consecutive amplitudes.
template <typename V>
__global__ void __launch_bounds__(256)
    k_marginal_low(const V* __restrict__ s, uint32_t m, uint64_t iters, double* __restrict__ out) {
  const uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= (uint64_t(1) << m)) return;
  double acc = 0.0;
  for (uint64_t t = 0; t < iters; ++t) acc = __dadd_rn(acc, nsq(s[(t << m) | c]));
  out[c] = acc;
}

extern "C" int ev_marginal_low(const ev_state* s, uint64_t m, double* out) {
  clear_error();
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_marginal_low: null argument");
  if (m > s->n || m > 28)
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_marginal_low: %llu low qubits of a %llu-qubit state",
                (unsigned long long)m, (unsigned long long)s->n);
  EV_CUDA(cudaSetDevice(s->device));
  const uint64_t count = uint64_t(1) << m;
  double* d = nullptr;
  EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), count * sizeof(double), s->stream));
  const unsigned grid = unsigned((count + 255) / 256);
  const uint64_t iters = s->len() >> m;
  if (s->dtype == EV_C128)
    k_marginal_low<<<grid, 256, 0, s->stream>>>(static_cast<const double2*>(s->amps), uint32_t(m),
                                                iters, d);
  else
    k_marginal_low<<<grid, 256, 0, s->stream>>>(static_cast<const float2*>(s->amps), uint32_t(m),
                                                iters, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d, count * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(d, s->stream);
  const cudaError_t e2 = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess || e2 != cudaSuccess)
    return fail(EV_ERR_CUDA, "ev_marginal_low: %s",
                cudaGetErrorString(e != cudaSuccess ? e : e2));
  return EV_OK;
}

// State::probability: one amplitude, norm_sqr on the host with std::fma
// (state.rs:119-122).
extern "C" int ev_probability(const ev_state* s, uint64_t basis, double* out) {
  clear_error();
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_probability: null argument");
  if (basis >= s->len())
    return fail(EV_ERR_INVALID_ARGUMENT, "basis state %llu out of range", (unsigned long long)basis);
  EV_CUDA(cudaSetDevice(s->device));
  double re, im;
  if (s->dtype == EV_C128) {
    double v[2];
    EV_CUDA(cudaMemcpyAsync(v, static_cast<const double2*>(s->amps) + basis, 16,
                            cudaMemcpyDeviceToHost, s->stream));
    EV_CUDA(cudaStreamSynchronize(s->stream));
    re = v[0];
    im = v[1];
  } else {
    float v[2];
    EV_CUDA(cudaMemcpyAsync(v, static_cast<const float2*>(s->amps) + basis, 8,
                            cudaMemcpyDeviceToHost, s->stream));
    EV_CUDA(cudaStreamSynchronize(s->stream));
    re = v[0];
    im = v[1];
  }
  *out = std::fma(re, re, im * im);
  return EV_OK;
}

extern "C" int ev_amplitude(const ev_state* s, uint64_t basis, double out[2]) {
  clear_error();
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_amplitude: null argument");
  if (basis >= s->len())
    return fail(EV_ERR_INVALID_ARGUMENT, "basis state %llu out of range", (unsigned long long)basis);
  EV_CUDA(cudaSetDevice(s->device));
  if (s->dtype == EV_C128) {
    EV_CUDA(cudaMemcpyAsync(out, static_cast<const double2*>(s->amps) + basis, 16,
                            cudaMemcpyDeviceToHost, s->stream));
    EV_CUDA(cudaStreamSynchronize(s->stream));
  } else {
    float v[2];
    EV_CUDA(cudaMemcpyAsync(v, static_cast<const float2*>(s->amps) + basis, 8,
                            cudaMemcpyDeviceToHost, s->stream));
    EV_CUDA(cudaStreamSynchronize(s->stream));
    out[0] = v[0];
    out[1] = v[1];
  }
  return EV_OK;
}

extern "C" int ev_overlap(const ev_state* self, const ev_state* other, double out[2]) {
  clear_error();
  if (!self || !other || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_overlap: null argument");
  if (self->n != other->n)
    return fail(EV_ERR_DIMENSION_MISMATCH, "states must have equal qubit counts (%llu vs %llu)",
                (unsigned long long)self->n, (unsigned long long)other->n);
  EV_CUDA(cudaSetDevice(self->device));
  // other's pending work must be complete before self's stream reads it
  EV_CUDA(cudaStreamSynchronize(other->stream));
  if (self->dtype != other->dtype) {
    const uint64_t count = self->len();
    const uint64_t want = (count + 4095) / 4096;
    int nb = int(want < 1 ? 1 : want);
    const int cap = self->num_sms * 4 < kMaxRedBlocks ? self->num_sms * 4 : kMaxRedBlocks;
    if (nb > cap) nb = cap;
    const uint64_t chunk = (count + nb - 1) / nb;
    if (self->dtype == EV_C64)
      k_overlap_mixed<float2, double2><<<nb, kRedThreads, 0, self->stream>>>(
          static_cast<const float2*>(self->amps), static_cast<const double2*>(other->amps), count,
          chunk, self->scratch.partials);
    else
      k_overlap_mixed<double2, float2><<<nb, kRedThreads, 0, self->stream>>>(
          static_cast<const double2*>(self->amps), static_cast<const float2*>(other->amps), count,
          chunk, self->scratch.partials);
    k_finish<<<1, kRedThreads, 0, self->stream>>>(self->scratch.partials, nb, self->scratch.result,
                                                 nullptr);
    self->launches += 2;
    EV_CUDA(cudaGetLastError());
  } else {
    EV_TRY(reduce<R_OVERLAP>(self, other, self->len(), 0, nullptr));
  }
  double r[2];
  EV_TRY(fetch_result(self, r, 2));
  out[0] = r[0];
  out[1] = r[1];
  return EV_OK;
}

// State::fidelity = |<other|self>|^2 with the FMA-form norm (state.rs:149-151).
extern "C" int ev_fidelity(const ev_state* self, const ev_state* other, double* out) {
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_fidelity: null argument");
  double ov[2];
  EV_TRY(ev_overlap(self, other, ov));
  *out = std::fma(ov[0], ov[0], ov[1] * ov[1]);
  return EV_OK;
}

// max_j |self_j - other_j| (modulus in f64; a max, so the order of the
// reduction does not change the result).  The two states may hold different
// amplitude types: the error of a complex64 run against complex128.
template <typename VA, typename VB>
__global__ void __launch_bounds__(kRedThreads)
    k_maxdiff(const VA* __restrict__ a, const VB* __restrict__ b, uint64_t count, uint64_t chunk,
              double* __restrict__ partials) {
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  double m = 0.0;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += kRedThreads) {
    const double dx = double(a[i].x) - double(b[i].x), dy = double(a[i].y) - double(b[i].y);
    m = fmax(m, hypot(dx, dy));
  }
  __shared__ double sh[kRedThreads];
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void k_finish_max(const double* __restrict__ partials, int nblocks, double* result) {
  __shared__ double sh[kRedThreads];
  double m = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kRedThreads) m = fmax(m, partials[b]);
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) result[0] = sh[0];
}

extern "C" int ev_max_abs_diff(const ev_state* self, const ev_state* other, double* out) {
  clear_error();
  if (!self || !other || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_max_abs_diff: null argument");
  if (self->n != other->n)
    return fail(EV_ERR_DIMENSION_MISMATCH, "states must have equal qubit counts (%llu vs %llu)",
                (unsigned long long)self->n, (unsigned long long)other->n);
  EV_CUDA(cudaSetDevice(self->device));
  EV_CUDA(cudaStreamSynchronize(other->stream));
  int nb = 0;
  uint64_t chunk = 0;
  red_grid(self->len(), self->num_sms, 8, kMaxRedBlocks, &nb, &chunk);  // a maximum: any grid
  const bool a128 = self->dtype == EV_C128, b128 = other->dtype == EV_C128;
  double* part = self->scratch.partials;
  if (a128 && b128)
    k_maxdiff<double2, double2><<<nb, kRedThreads, 0, self->stream>>>(
        static_cast<const double2*>(self->amps), static_cast<const double2*>(other->amps),
        self->len(), chunk, part);
  else if (a128)
    k_maxdiff<double2, float2><<<nb, kRedThreads, 0, self->stream>>>(
        static_cast<const double2*>(self->amps), static_cast<const float2*>(other->amps),
        self->len(), chunk, part);
  else if (b128)
    k_maxdiff<float2, double2><<<nb, kRedThreads, 0, self->stream>>>(
        static_cast<const float2*>(self->amps), static_cast<const double2*>(other->amps),
        self->len(), chunk, part);
  else
    k_maxdiff<float2, float2><<<nb, kRedThreads, 0, self->stream>>>(
        static_cast<const float2*>(self->amps), static_cast<const float2*>(other->amps),
        self->len(), chunk, part);
  k_finish_max<<<1, kRedThreads, 0, self->stream>>>(part, nb, self->scratch.result);
  self->launches += 2;
  EV_CUDA(cudaGetLastError());
  return fetch_result(self, out, 1);
}

extern "C" int ev_bloch_vector(const ev_state* s, uint64_t qubit, double out[3]) {
  clear_error();
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_bloch_vector: null argument");
  if (qubit >= s->n)
    return fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                (unsigned long long)qubit, (unsigned long long)s->n);
  EV_CUDA(cudaSetDevice(s->device));
  EV_TRY(reduce<R_BLOCH>(s, nullptr, s->len() / 2, int(qubit), nullptr));
  double r[4];
  EV_TRY(fetch_result(s, r, 4));
  out[0] = 2.0 * r[2];
  out[1] = 2.0 * r[3];
  out[2] = r[0] - r[1];
  return EV_OK;
}

// ---- Pauli-string expectations (PauliString::expectation,
// src/backend/stabilizer.rs:79-125) ------------------------------------------
// The reference applies P to a copy of the state and takes Re <psi|P psi>.
// Here terms that share an X mask x are summed in one pass without a copy:
//   x == 0:  <P> = sign * sum_j s_j |a_j|^2
//   x != 0:  pairs (j, j ^ x) with the highest bit of x clear in j, and
//            w = conj(a_{j^x}) a_j;  with y = popc(x & z) (the Y count),
//            y even: <P> = sign * (-1)^(y/2) * 2 sum s_j Re w
//            y odd:  <P> = sign * (y % 4 == 1 ? -1 : 1) * 2 sum s_j Im w
// where s_j = (-1)^popc(j & z).  Each pair is read once for all its terms.
constexpr int kPauliTerms = 8;
struct PauliPass {
  uint64_t z[kPauliTerms];
  int nterms;
  int part;  // 0: |a_j|^2 (x == 0), 1: Re w, 2: Im w
};

template <typename V>
__global__ void __launch_bounds__(kRedThreads)
    k_pauli(const V* __restrict__ a, uint64_t count, uint64_t chunk, uint64_t xmask, int hbit,
            PauliPass pp, double* __restrict__ partials) {
  constexpr int kPG = 4;  // iterations whose loads are in flight together
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < count ? lo + chunk : count;
  double acc[kPauliTerms];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) acc[t] = 0.0;
  for (uint64_t base = lo + threadIdx.x; base < hi; base += uint64_t(kFlush) * kRedThreads) {
    FF f[kPauliTerms];
    for (int g0 = 0; g0 < kFlush; g0 += kPG) {
      V xs[kPG], ys[kPG];
      uint64_t js[kPG];
#pragma unroll
      for (int r = 0; r < kPG; ++r) {
        const uint64_t i = base + uint64_t(g0 + r) * kRedThreads;
        js[r] = pp.part == 0 ? i : insert0(i, hbit);
        if (i < hi) {
          xs[r] = a[js[r]];
          ys[r] = pp.part != 0 ? a[js[r] ^ xmask] : xs[r];
        }
      }
#pragma unroll
      for (int r = 0; r < kPG; ++r) {
        if (base + uint64_t(g0 + r) * kRedThreads >= hi) break;
        const uint64_t j = js[r];
        const V x = xs[r], y = ys[r];
        if constexpr (sizeof(V) == 8) {
          FF v;  // the term, exactly split: hi + lo
          if (pp.part == 0) {
            v.add_prod(x.x, x.x);
            v.add_prod(x.y, x.y);
          } else if (pp.part == 1) {
            v.add_prod(y.x, x.x);
            v.add_prod(y.y, x.y);
          } else {
            v.add_prod(y.x, x.y);
            v.add_prod(-y.y, x.x);
          }
#pragma unroll
          for (int t = 0; t < kPauliTerms; ++t)
            if (t < pp.nterms) {
              const bool neg = __popcll(j & pp.z[t]) & 1;
              f[t].lo = __fadd_rn(f[t].lo, neg ? -v.lo : v.lo);
              f[t].add(neg ? -v.hi : v.hi);
            }
        } else {
          double v;
          if (pp.part == 0)
            v = __fma_rn(x.x, x.x, __dmul_rn(x.y, x.y));
          else if (pp.part == 1)
            v = __fma_rn(y.x, x.x, __dmul_rn(y.y, x.y));
          else
            v = __fma_rn(y.x, x.y, -__dmul_rn(y.y, x.x));
#pragma unroll
          for (int t = 0; t < kPauliTerms; ++t)
            if (t < pp.nterms) acc[t] += (__popcll(j & pp.z[t]) & 1) ? -v : v;
        }
      }
    }
    if constexpr (sizeof(V) == 8) {
#pragma unroll
      for (int t = 0; t < kPauliTerms; ++t) acc[t] += f[t].value();
    }
  }
  __shared__ double sh[kPauliTerms][kRedThreads];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] = acc[t];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] += sh[t][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < kPauliTerms) partials[blockIdx.x * kPauliTerms + threadIdx.x] = sh[threadIdx.x][0];
}

// The same sums over aligned blocks of 8 indices (complex64).  The parity of
// j & z is the parity of the block's first index j0 xor that of
// (j mod 8) & (z mod 8), so a term's sum over the block is
//     (-1)^popc(j0 & z) * W[z mod 8],  W[m] = sum_r (-1)^popc(r & m) v_r,
// the Walsh-Hadamard transform of the block's 8 values v_r.  One 3-level
// transform serves every term of the pass: 3 butterflies and one term
// update per index for 8 terms, where adding each value to each term took
// 8 updates.  When x == 0 or the highest bit h of x is 3 or more, the 8
// indices of a block are 8 consecutive j (bit h clear), and their partners
// j ^ x the aligned block of j0 ^ x in the order r ^ (x mod 8).  When h < 3
// the partner lies in the same block: the blocks then cover all 2^n indices
// and the values of the indices with bit h set are zero, so each pair
// (j, j ^ x) counts once, from the index with bit h clear.
//
// Values are unnormalised double-float pairs (hi + lo): every hi sum is
// split exactly by two-sum and its error moves into lo, which carries the
// exact product errors as well, so a pair holds its value to ~2^-48 of the
// magnitudes summed into it.  A term's pair covers kPauliRun blocks and is
// then added to its f64 sum.
constexpr int kPauliRun = 16;  // blocks per double-float run

struct F2 {
  float hi, lo;
};

// a b + c d with the products split exactly
__device__ __forceinline__ F2 f2_dot2(float a, float b, float c, float d) {
  const float p = __fmul_rn(a, b), q = __fmul_rn(c, d);
  const float pe = __fmaf_rn(a, b, -p), qe = __fmaf_rn(c, d, -q);
  const float s = __fadd_rn(p, q);
  const float bp = __fsub_rn(s, p);
  const float e = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bp)), __fsub_rn(q, bp));
  return {s, __fadd_rn(__fadd_rn(pe, qe), e)};
}

// (a, b) <- (a + b, a - b)
__device__ __forceinline__ void f2_butterfly(F2& a, F2& b) {
  const float s = __fadd_rn(a.hi, b.hi), d = __fsub_rn(a.hi, b.hi);
  const float sb = __fsub_rn(s, a.hi), db = __fsub_rn(d, a.hi);
  const float se = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, sb)), __fsub_rn(b.hi, sb));
  const float de = __fsub_rn(__fsub_rn(a.hi, __fsub_rn(d, db)), __fadd_rn(b.hi, db));
  const float ls = __fadd_rn(a.lo, b.lo), ld = __fsub_rn(a.lo, b.lo);
  a = {s, __fadd_rn(ls, se)};
  b = {d, __fadd_rn(ld, de)};
}

// acc += w
__device__ __forceinline__ void f2_add(F2& acc, float whi, float wlo) {
  const float s = __fadd_rn(acc.hi, whi);
  const float bp = __fsub_rn(s, acc.hi);
  const float e = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bp)), __fsub_rn(whi, bp));
  acc = {s, __fadd_rn(__fadd_rn(acc.lo, wlo), e)};
}

// 3 blocks per SM: 80 registers, no spills (4 spill)
__global__ void __launch_bounds__(kRedThreads, 3)
    k_pauli_blk(const float2* __restrict__ a, uint64_t nblk, uint64_t chunk, uint64_t xmask,
                int hbit, PauliPass pp, double* __restrict__ partials) {
  __shared__ float2 shw[8][kRedThreads];  // this thread's W, read back at index z mod 8
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < nblk ? lo + chunk : nblk;
  const uint64_t xr = xmask & 7;
  double acc[kPauliTerms];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) acc[t] = 0.0;
  for (uint64_t base = lo + threadIdx.x; base < hi; base += uint64_t(kPauliRun) * kRedThreads) {
    F2 f[kPauliTerms];
#pragma unroll
    for (int t = 0; t < kPauliTerms; ++t) f[t] = {0.f, 0.f};
    for (int g = 0; g < kPauliRun; ++g) {
      const uint64_t blk = base + uint64_t(g) * kRedThreads;
      if (blk >= hi) break;
      const uint64_t j0 = (pp.part == 0 || hbit < 3) ? blk * 8 : insert0(blk * 8, hbit);
      // j0 is a multiple of 8: the block is 64 aligned bytes
      const float4* xp = reinterpret_cast<const float4*>(a + j0);
      float4 xq[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) xq[q] = xp[q];
      F2 w[8];
      if (pp.part == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          w[2 * q] = f2_dot2(xq[q].x, xq[q].x, xq[q].y, xq[q].y);
          w[2 * q + 1] = f2_dot2(xq[q].z, xq[q].z, xq[q].w, xq[q].w);
        }
      } else {
        const uint64_t p0 = (j0 ^ xmask) & ~uint64_t(7);
        float2 y[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) y[r] = a[p0 + (uint64_t(r) ^ xr)];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float2 x0 = make_float2(xq[q].x, xq[q].y), x1 = make_float2(xq[q].z, xq[q].w);
          const float2 y0 = y[2 * q], y1 = y[2 * q + 1];
          if (pp.part == 1) {  // Re(conj(y) x)
            w[2 * q] = f2_dot2(y0.x, x0.x, y0.y, x0.y);
            w[2 * q + 1] = f2_dot2(y1.x, x1.x, y1.y, x1.y);
          } else {  // Im(conj(y) x)
            w[2 * q] = f2_dot2(y0.x, x0.y, -y0.y, x0.x);
            w[2 * q + 1] = f2_dot2(y1.x, x1.y, -y1.y, x1.x);
          }
        }
        if (hbit < 3)  // partner in the block: count each pair once
#pragma unroll
          for (int r = 0; r < 8; ++r)
            if ((r >> hbit) & 1) w[r] = {0.f, 0.f};
      }
#pragma unroll
      for (int h = 1; h < 8; h <<= 1)
#pragma unroll
        for (int r = 0; r < 8; ++r)
          if (!(r & h)) f2_butterfly(w[r], w[r + h]);
#pragma unroll
      for (int m = 0; m < 8; ++m) shw[m][threadIdx.x] = make_float2(w[m].hi, w[m].lo);
#pragma unroll
      for (int t = 0; t < kPauliTerms; ++t)
        if (t < pp.nterms) {
          const float2 v = shw[pp.z[t] & 7][threadIdx.x];
          const uint32_t flip = uint32_t(__popcll(j0 & pp.z[t]) & 1) << 31;
          f2_add(f[t], __uint_as_float(__float_as_uint(v.x) ^ flip),
                 __uint_as_float(__float_as_uint(v.y) ^ flip));
        }
    }
#pragma unroll
    for (int t = 0; t < kPauliTerms; ++t) acc[t] += f2d_exact(f[t].hi) + f2d_exact(f[t].lo);
  }
  __shared__ double sh[kPauliTerms][kRedThreads];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] = acc[t];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] += sh[t][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < kPauliTerms) partials[blockIdx.x * kPauliTerms + threadIdx.x] = sh[threadIdx.x][0];
}

// The block transform in complex128, on the FP64 pipe: per block of 8
// indices 8 values (2 FP64 instructions each), 24 butterfly adds and one add
// per term, 6 FP64 instructions per index for 8 terms where adding each
// value to each term took 10.  3 blocks per SM: 80 registers, no spills.
__global__ void __launch_bounds__(kRedThreads, 3)
    k_pauli_blk_f64(const double2* __restrict__ a, uint64_t nblk, uint64_t chunk, uint64_t xmask,
                    int hbit, PauliPass pp, double* __restrict__ partials) {
  __shared__ double shw[8][kRedThreads];  // this thread's W, read back at index z mod 8
  const uint64_t lo = uint64_t(blockIdx.x) * chunk;
  const uint64_t hi = lo + chunk < nblk ? lo + chunk : nblk;
  const uint64_t xr = xmask & 7;
  double acc[kPauliTerms];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) acc[t] = 0.0;
  for (uint64_t blk = lo + threadIdx.x; blk < hi; blk += kRedThreads) {
    const uint64_t j0 = (pp.part == 0 || hbit < 3) ? blk * 8 : insert0(blk * 8, hbit);
    double w[8];
    if (pp.part == 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const double2 x = a[j0 + r];
        w[r] = __fma_rn(x.x, x.x, __dmul_rn(x.y, x.y));
      }
    } else {
      const uint64_t p0 = (j0 ^ xmask) & ~uint64_t(7);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const double2 x = a[j0 + r], y = a[p0 + (uint64_t(r) ^ xr)];
        w[r] = pp.part == 1 ? __fma_rn(y.x, x.x, __dmul_rn(y.y, x.y))
                            : __fma_rn(y.x, x.y, -__dmul_rn(y.y, x.x));
      }
      if (hbit < 3)  // partner in the block: count each pair once
#pragma unroll
        for (int r = 0; r < 8; ++r)
          if ((r >> hbit) & 1) w[r] = 0.0;
    }
#pragma unroll
    for (int h = 1; h < 8; h <<= 1)
#pragma unroll
      for (int r = 0; r < 8; ++r)
        if (!(r & h)) {
          const double u = w[r], v = w[r + h];
          w[r] = __dadd_rn(u, v);
          w[r + h] = __dsub_rn(u, v);
        }
#pragma unroll
    for (int m = 0; m < 8; ++m) shw[m][threadIdx.x] = w[m];
#pragma unroll
    for (int t = 0; t < kPauliTerms; ++t)
      if (t < pp.nterms) {
        const uint64_t flip = uint64_t(__popcll(j0 & pp.z[t]) & 1) << 63;
        const double v = __longlong_as_double(
            (long long)(uint64_t(__double_as_longlong(shw[pp.z[t] & 7][threadIdx.x])) ^ flip));
        acc[t] = __dadd_rn(acc[t], v);
      }
  }
  __shared__ double sh[kPauliTerms][kRedThreads];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] = acc[t];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] += sh[t][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < kPauliTerms) partials[blockIdx.x * kPauliTerms + threadIdx.x] = sh[threadIdx.x][0];
}

// result[t] = sum over blocks of partials[b][t], fixed order.
__global__ void __launch_bounds__(kRedThreads)
    k_finish_terms(const double* __restrict__ partials, int nblocks, double* __restrict__ result) {
  __shared__ double sh[kPauliTerms][kRedThreads];
  double acc[kPauliTerms] = {};
  for (int b = threadIdx.x; b < nblocks; b += kRedThreads)
#pragma unroll
    for (int t = 0; t < kPauliTerms; ++t) acc[t] += partials[b * kPauliTerms + t];
#pragma unroll
  for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] = acc[t];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int t = 0; t < kPauliTerms; ++t) sh[t][threadIdx.x] += sh[t][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < kPauliTerms) result[threadIdx.x] = sh[threadIdx.x][0];
}

extern "C" int ev_pauli_expectation(const ev_state* s, const uint64_t* x_masks,
                                    const uint64_t* z_masks, const uint8_t* negative,
                                    uint64_t count, double* out) {
  clear_error();
  if (!s || (count && (!x_masks || !z_masks || !out)))
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_pauli_expectation: null argument");
  const uint64_t valid = s->n >= 64 ? ~uint64_t(0) : (uint64_t(1) << s->n) - 1;
  for (uint64_t t = 0; t < count; ++t)
    if ((x_masks[t] | z_masks[t]) & ~valid)
      return fail(EV_ERR_QUBIT_OUT_OF_RANGE,
                  "Pauli string %llu acts on a qubit outside the %llu-qubit register",
                  (unsigned long long)t, (unsigned long long)s->n);
  if (count == 0) return EV_OK;
  EV_CUDA(cudaSetDevice(s->device));
  // group terms by (X mask, parity of the Y count), first appearance first:
  // one group shares its pairs and whether Re w or Im w is summed
  auto key_par = [&](uint64_t t) {
    return x_masks[t] ? (__builtin_popcountll(x_masks[t] & z_masks[t]) & 1) : 0;
  };
  std::vector<uint64_t> order;
  order.reserve(count);
  std::vector<char> used(count, 0);
  for (uint64_t t = 0; t < count; ++t) {
    if (used[t]) continue;
    for (uint64_t u = t; u < count; ++u)
      if (!used[u] && x_masks[u] == x_masks[t] && key_par(u) == key_par(t)) {
        used[u] = 1;
        order.push_back(u);
      }
  }
  size_t at = 0;
  while (at < order.size()) {
    const uint64_t first = order[at];
    const uint64_t x = x_masks[first];
    const int par = key_par(first);
    PauliPass pp{};
    uint64_t terms[kPauliTerms];
    while (at < order.size() && pp.nterms < kPauliTerms && x_masks[order[at]] == x &&
           key_par(order[at]) == par) {
      terms[pp.nterms] = order[at];
      pp.z[pp.nterms] = z_masks[order[at]];
      ++pp.nterms;
      ++at;
    }
    pp.part = x == 0 ? 0 : (par ? 2 : 1);
    const int hbit = x == 0 ? -1 : 63 - __builtin_clzll(x);
    const uint64_t work = x == 0 ? s->len() : s->len() / 2;
    int nb = 0;
    uint64_t chunk = 0;
    if (s->len() >= 8) {
      // aligned blocks of 8 indices, one Walsh-Hadamard transform each; an X
      // mask below bit 3 pairs indices inside a block, whose blocks then
      // cover every index
      const uint64_t nblk = (x != 0 && hbit >= 3 ? work : s->len()) / 8;
      if (s->dtype == EV_C128) {
        red_grid(nblk, s->num_sms, resident_blocks<k_pauli_blk_f64>(),
                 kMaxRedBlocks * 4 / kPauliTerms, &nb, &chunk);
        k_pauli_blk_f64<<<nb, kRedThreads, 0, s->stream>>>(static_cast<const double2*>(s->amps),
                                                            nblk, chunk, x, hbit, pp,
                                                            s->scratch.partials);
      } else {
        red_grid(nblk, s->num_sms, resident_blocks<k_pauli_blk>(),
                 kMaxRedBlocks * 4 / kPauliTerms, &nb, &chunk);
        k_pauli_blk<<<nb, kRedThreads, 0, s->stream>>>(static_cast<const float2*>(s->amps),
                                                        nblk, chunk, x, hbit, pp,
                                                        s->scratch.partials);
      }
    } else {  // fewer than 8 amplitudes
      red_grid(work, s->num_sms,
               s->dtype == EV_C128 ? resident_blocks<k_pauli<double2>>()
                                   : resident_blocks<k_pauli<float2>>(),
               kMaxRedBlocks * 4 / kPauliTerms, &nb, &chunk);
      if (s->dtype == EV_C128)
        k_pauli<double2><<<nb, kRedThreads, 0, s->stream>>>(static_cast<const double2*>(s->amps),
                                                             work, chunk, x, hbit, pp,
                                                             s->scratch.partials);
      else
        k_pauli<float2><<<nb, kRedThreads, 0, s->stream>>>(static_cast<const float2*>(s->amps),
                                                           work, chunk, x, hbit, pp,
                                                           s->scratch.partials);
    }
    k_finish_terms<<<1, kRedThreads, 0, s->stream>>>(s->scratch.partials, nb, s->scratch.result);
    s->launches += 2;
    EV_CUDA(cudaGetLastError());
    double r[kPauliTerms];
    EV_TRY(fetch_result(s, r, kPauliTerms));
    for (int t = 0; t < pp.nterms; ++t) {
      const uint64_t id = terms[t];
      const double sign = (negative && negative[id]) ? -1.0 : 1.0;
      if (x == 0) {
        out[id] = sign * r[t];
      } else {
        const int y = __builtin_popcountll(x & pp.z[t]);
        const double f = (y & 1) ? ((y % 4 == 1) ? -1.0 : 1.0) : ((y % 4 == 0) ? 1.0 : -1.0);
        out[id] = sign * f * 2.0 * r[t];
      }
    }
  }
  return EV_OK;
}

extern "C" int ev_sample(ev_state* s, uint64_t seed, uint64_t shots, uint64_t* out) {
  clear_error();
  if (!s || (shots && !out)) return fail(EV_ERR_INVALID_ARGUMENT, "ev_sample: null argument");
  if (s->n > 63) return fail(EV_ERR_INVALID_ARGUMENT, "ev_sample: at most 63 qubits");
  if (shots == 0) return EV_OK;
  if (s->n == 0) {
    std::memset(out, 0, shots * sizeof(uint64_t));
    return EV_OK;
  }
  EV_CUDA(cudaSetDevice(s->device));
  EV_TRY(ensure_mass(s));
  EV_TRY(build_mass(s));
  const uint64_t nu = shots * s->n;
  std::vector<double> uni(nu);
  Rng rng(seed);
  for (uint64_t j = 0; j < nu; ++j) uni[j] = rng.next_f64();
  void* du = nullptr;
  void* dout = nullptr;
  EV_CUDA(cudaMallocAsync(&du, nu * sizeof(double), s->stream));
  int rc = EV_OK;
  if (cudaMallocAsync(&dout, shots * sizeof(uint64_t), s->stream) != cudaSuccess) {
    cudaGetLastError();
    cudaFreeAsync(du, s->stream);
    return fail(EV_ERR_OOM, "ev_sample: cannot allocate %llu shots", (unsigned long long)shots);
  }
  cudaError_t e = cudaMemcpyAsync(du, uni.data(), nu * sizeof(double), cudaMemcpyHostToDevice,
                                  s->stream);
  if (e == cudaSuccess) {
    const unsigned g = unsigned((shots + 255) / 256);
    s->launches += 1;
    if (s->dtype == EV_C128)
      k_descend<double2><<<g, 256, 0, s->stream>>>(s->mass, static_cast<const double2*>(s->amps),
                                                   int(s->n), static_cast<const double*>(du),
                                                   shots, static_cast<uint64_t*>(dout));
    else
      k_descend<float2><<<g, 256, 0, s->stream>>>(s->mass, static_cast<const float2*>(s->amps),
                                                  int(s->n), static_cast<const double*>(du), shots,
                                                  static_cast<uint64_t*>(dout));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, dout, shots * sizeof(uint64_t), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "ev_sample: %s", cudaGetErrorString(e));
  cudaFreeAsync(du, s->stream);
  cudaFreeAsync(dout, s->stream);
  return rc;
}

// ---- measurement without allocation ----------------------------------------
//
// ev_measure_qubit_noalloc measures a complex128 statevector that lives in a
// device buffer the caller owns, and allocates nothing: its reduction
// partials and measurement words live in one file-scope __device__ array.
// It is for callers that cannot call cudaMalloc: a serving process that hands
// all of HBM to its own allocator up front, or a host framework (a Rust or
// C++ runtime with its own device pool) that must not see a foreign
// allocation or the device-wide synchronisation cudaMalloc/cudaFree imply.
//
// The array is 2048 reduction blocks x 4 partials plus 12 words
// (8204 doubles, ~64 KiB); every GPU that loads the library holds it until
// the process exits.  Host code must not pass the array's name to a kernel
// (on the host it is only a stand-in, not a device address), so the first
// call in each CUDA context (the device's primary context, or a context the
// caller made current with the driver API), with that context current,
// resolves the address with cudaGetSymbolAddress and caches it under the
// (device, context) pair; make that first call before any stream capture.
// All calls share the array and each overwrites what the previous one left,
// so calls that overlap on the GPU (different streams, no ordering between
// them) race; calls on one stream, or otherwise ordered, are safe.  Each call
// returns once its measurement has completed on the caller's stream.
namespace {
constexpr int kNoAllocBlocks = 2048;
constexpr uint64_t kNoAllocMaxQubits = 40;
__device__ __align__(256) double g_noalloc_scratch[kNoAllocBlocks * 4 + 12];

struct NoAllocSlot {
  int device;
  void* context;
  double* addr;
};
constexpr int kNoAllocSlots = 64;
std::mutex g_noalloc_mu;
NoAllocSlot g_noalloc_slot[kNoAllocSlots];
int g_noalloc_used = 0;

// Driver functions reached through the runtime (the library links no driver
// library, so it still loads where no driver is installed).
using CtxGetCurrentFn = int (*)(void**);
using MemGetAddressRangeFn = int (*)(unsigned long long*, size_t*, unsigned long long);
template <typename Fn>
Fn driver_fn(const char* name) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return reinterpret_cast<Fn>(p);
}

int current_context(void** ctx) {
  static const CtxGetCurrentFn fn = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
  if (!fn) return fail(EV_ERR_CUDA, "ev_measure_qubit_noalloc: cuCtxGetCurrent unavailable");
  *ctx = nullptr;
  if (fn(ctx) != 0) return fail(EV_ERR_CUDA, "ev_measure_qubit_noalloc: cuCtxGetCurrent failed");
  return EV_OK;
}

// The scratch array's device address in the current context.
int noalloc_scratch(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  void* ctx = nullptr;
  EV_TRY(current_context(&ctx));
  if (ctx == nullptr) {
    // No context is current on this thread yet: the runtime binds the
    // device's primary context on its next call, this one.
    void* p = nullptr;
    EV_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    EV_TRY(current_context(&ctx));
  }
  for (int i = 0; i < g_noalloc_used; ++i)
    if (g_noalloc_slot[i].device == device && g_noalloc_slot[i].context == ctx) {
      *out = g_noalloc_slot[i].addr;
      return EV_OK;
    }
  if (g_noalloc_used == kNoAllocSlots)
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_measure_qubit_noalloc: more than %d contexts",
                kNoAllocSlots);
  void* p = nullptr;
  EV_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  g_noalloc_slot[g_noalloc_used++] = NoAllocSlot{device, ctx, static_cast<double*>(p)};
  *out = static_cast<double*>(p);
  return EV_OK;
}

// Refuses, before any launch, a buffer the kernels could not use: not
// 16-byte aligned (they move whole complex128 values), not device or managed
// memory of the current device, or shorter than 2^n amplitudes.
int check_caller_buffer(const double* amps, uint64_t n, int device) {
  if (reinterpret_cast<uintptr_t>(amps) % 16 != 0)
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: amplitude buffer is not 16-byte aligned");
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, amps) != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: amplitude buffer is not CUDA memory");
  }
  if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: amplitude buffer is not device memory");
  if (attr.type == cudaMemoryTypeDevice && attr.device != device)
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: amplitude buffer is on device %d, current is %d",
                attr.device, device);
  static const MemGetAddressRangeFn range = driver_fn<MemGetAddressRangeFn>("cuMemGetAddressRange");
  unsigned long long base = 0;
  size_t size = 0;
  const unsigned long long at = reinterpret_cast<unsigned long long>(amps);
  if (!range || range(&base, &size, at) != 0)
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: cannot find the allocation of the amplitude buffer");
  const unsigned long long need = (unsigned long long)(uint64_t(16) << n);
  if (at < base || at - base > size || size - (at - base) < need)
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: the allocation holds fewer than 2^%llu amplitudes "
                "from the given address",
                (unsigned long long)n);
  return EV_OK;
}
}  // namespace

extern "C" int ev_measure_qubit_noalloc(double* amps, uint64_t n, uint64_t k, double u,
                                        void* stream, int32_t* outcome) {
  clear_error();
  if (!amps || !outcome) return fail(EV_ERR_INVALID_ARGUMENT, "ev_measure_qubit_noalloc: null argument");
  if (n > kNoAllocMaxQubits)
    return fail(EV_ERR_INVALID_ARGUMENT,
                "ev_measure_qubit_noalloc: %llu qubits exceeds the maximum of %llu",
                (unsigned long long)n, (unsigned long long)kNoAllocMaxQubits);
  if (k >= n)
    return fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                (unsigned long long)k, (unsigned long long)n);
  int device = 0, sms = 0;
  EV_CUDA(cudaGetDevice(&device));
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  EV_TRY(check_caller_buffer(amps, n, device));
  double* scratch = nullptr;
  EV_TRY(noalloc_scratch(device, &scratch));
  double* partials = scratch;
  double* result = scratch + kNoAllocBlocks * 4;
  double* meas = result + 8;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2* a = reinterpret_cast<double2*>(amps);
  // same kernel and grid as the state-owned path, so the sums (and results)
  // agree
  const uint64_t count = (uint64_t(1) << n) / 2;
  int nb = 0;
  uint64_t chunk = 0;
  red_grid(count, sms, resident_blocks<k_reduce_sq<R_P1, double2>>(), kNoAllocBlocks, &nb, &chunk);
  k_reduce_sq<R_P1, double2><<<nb, kRedThreads, 0, st>>>(a, count, chunk, int(k), partials, nullptr);
  k_finish<<<1, kRedThreads, 0, st>>>(partials, nb, result, nullptr);
  k_decide<<<1, 1, 0, st>>>(result, u, nullptr, nullptr, meas, nullptr, nullptr);
  const uint64_t gw = (count + 255) / 256, gcap = uint64_t(sms) * 8;
  k_collapse<double2><<<unsigned(gw < 1 ? 1 : (gw < gcap ? gw : gcap)), 256, 0, st>>>(
      a, count, int(k), meas, nullptr);
  EV_CUDA(cudaGetLastError());
  double words[4];
  EV_CUDA(cudaMemcpyAsync(words, meas, sizeof(words), cudaMemcpyDeviceToHost, st));
  EV_CUDA(cudaStreamSynchronize(st));
  *outcome = words[2] != 0.0 ? 1 : 0;
  return EV_OK;
}
