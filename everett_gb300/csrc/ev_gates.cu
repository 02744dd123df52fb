// ev_gates.cu -- streaming gate kernels, one HBM pass per gate.
//
// Each kernel restates one loop of src/kernel.rs on the GPU:
//   apply_1q              kernel.rs:76-119   -> k_pair / k_diag
//   apply_2q (+ cnot/cz/swap dispatch)
//                         kernel.rs:192-289  -> k_quad
//   apply_controlled_1q   kernel.rs:299-358  -> k_ctrl
// The per-amplitude arithmetic is the reference's (ev_device.cuh); what
// changes is the iteration: grid-stride loops over pair/quad indices with
// 16-byte (complex128) or 8-byte (complex64) vector accesses, and the
// controlled gate enumerates only its active subspace (fixed 1 bits inserted
// into the counter) instead of testing every pair.
//
// Matrix-structure specialisations keep the reference's results: a zero
// entry contributes an exact +-0 to the FMA-form sum and a real entry r
// reduces fma(r, x, -(0*y)) to the rounded product r*x, so dropping those
// terms changes no value (only, at most, the sign of a zero).  In the same
// way an anti-diagonal complex128 gate with entries in {1, i, -1, -i} (X, Y)
// is applied as a permutation with sign flips.
#include <cstdio>
#include <cstdlib>

#include <type_traits>

#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_softpair.cuh"

namespace ev {

template <typename V>
struct M1 {
  V m0, m1, m2, m3;
};
template <typename V>
struct M2 {
  V m[16];
};
struct Positions {
  int np;
  int p[64];  // ascending bit positions that get a 0 inserted
};

template <typename V>
M1<V> to_m1(const double m[8]);
template <>
M1<double2> to_m1<double2>(const double m[8]) {
  return {make_double2(m[0], m[1]), make_double2(m[2], m[3]), make_double2(m[4], m[5]),
          make_double2(m[6], m[7])};
}
template <>
M1<float2> to_m1<float2>(const double m[8]) {
  return {make_float2(float(m[0]), float(m[1])), make_float2(float(m[2]), float(m[3])),
          make_float2(float(m[4]), float(m[5])), make_float2(float(m[6]), float(m[7]))};
}

__device__ __forceinline__ bool skip(const uint8_t* pred) { return pred != nullptr && *pred == 0; }

// Applies the 2x2 update to one index pair in the reference's order
// (kernel.rs:113-116): new0 = m0*a0 + m1*a1, new1 = m2*a0 + m3*a1.
template <int KIND, typename V>
__device__ __forceinline__ void pair_update(V* __restrict__ s, uint64_t i0, uint64_t i1,
                                            const M1<V>& m) {
  if constexpr (KIND == K1_PHASE) {
    s[i1] = cmul(m.m3, s[i1]);
  } else {
    const V a0 = s[i0], a1 = s[i1];
    if constexpr (KIND == K1_DENSE) {
      s[i0] = cadd(cmul(m.m0, a0), cmul(m.m1, a1));
      s[i1] = cadd(cmul(m.m2, a0), cmul(m.m3, a1));
    } else if constexpr (KIND == K1_REAL) {
      s[i0] = cadd(rmul(m.m0.x, a0), rmul(m.m1.x, a1));
      s[i1] = cadd(rmul(m.m2.x, a0), rmul(m.m3.x, a1));
    } else if constexpr (KIND == K1_DIAG) {
      s[i0] = cmul(m.m0, a0);
      s[i1] = cmul(m.m3, a1);
    } else {  // K1_ANTI
      s[i0] = cmul(m.m1, a1);
      s[i1] = cmul(m.m2, a0);
    }
  }
}

// pair_update with the complex128 products of both outputs on the integer
// pipes (ev_softpair.cuh); same results.
template <int KIND>
__device__ __forceinline__ void pair_update_soft(double2* __restrict__ s, uint64_t i0, uint64_t i1,
                                                 const SoftM1& f) {
  if constexpr (KIND == K1_PHASE) {
    double2 a0 = make_double2(0.0, 0.0), a1 = s[i1];
    soft_pair<KIND>(a0, a1, f, true);
    s[i1] = a1;
  } else {
    double2 a0 = s[i0], a1 = s[i1];
    soft_pair<KIND>(a0, a1, f, true);
    s[i0] = a0;
    s[i1] = a1;
  }
}

// An entry in {1, i, -1, -i} as its power of i (0..3), else -1.
__device__ __forceinline__ int unit_power(double2 m) {
  if (m.y == 0.0) return m.x == 1.0 ? 0 : (m.x == -1.0 ? 2 : -1);
  if (m.x == 0.0) return m.y == 1.0 ? 1 : (m.y == -1.0 ? 3 : -1);
  return -1;
}
__device__ __forceinline__ double neg_if(double v, uint64_t flip) {
  return __longlong_as_double((long long)(uint64_t(__double_as_longlong(v)) ^ flip));
}
// i^p a by moving parts and flipping sign bits: the FMA-form product with a
// unit entry, whose products with the entry's zero part only add +-0, so
// the two agree up to the sign of a zero (the latitude the zero-entry
// specialisations above already take).
__device__ __forceinline__ double2 unit_mul(int p, double2 a) {
  constexpr uint64_t kSign = 0x8000000000000000ull;
  const double x = (p & 1) ? a.y : a.x, y = (p & 1) ? a.x : a.y;
  return make_double2(neg_if(x, (p == 1 || p == 2) ? kSign : 0u), neg_if(y, p >= 2 ? kSign : 0u));
}

// apply_1q over all 2^(n-1) pairs (kernel.rs:100-119).
template <int KIND, typename V>
__global__ void __launch_bounds__(256) k_pair(V* __restrict__ s, uint64_t npairs, int k, M1<V> m,
                                              const uint8_t* pred) {
  if (skip(pred)) return;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  const uint64_t bit = uint64_t(1) << k;
  if constexpr (std::is_same<V, double2>::value) {
    if constexpr (KIND == K1_ANTI) {  // X, Y and their sign variants: a permutation
      const int p1 = unit_power(m.m1), p2 = unit_power(m.m2);
      if ((p1 | p2) >= 0) {
        for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < npairs;
             i += stride) {
          const uint64_t i0 = insert0(i, k), i1 = i0 | bit;
          const double2 a0 = s[i0], a1 = s[i1];
          s[i0] = unit_mul(p1, a1);
          s[i1] = unit_mul(p2, a0);
        }
        return;
      }
    }
    const SoftM1 f = soft_matrix<KIND>(m.m0, m.m1, m.m2, m.m3);
    if (f.ok) {
      for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < npairs; i += stride) {
        const uint64_t i0 = insert0(i, k);
        pair_update_soft<KIND>(s, i0, i0 | bit, f);
      }
      return;
    }
  }
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < npairs; i += stride) {
    const uint64_t i0 = insert0(i, k);
    pair_update<KIND>(s, i0, i0 | bit, m);
  }
}

// apply_1q on one of the lowest five qubits, resolved within a warp: each
// lane loads one amplitude (a warp moves 32 consecutive amplitudes, 512
// contiguous bytes in complex128, with 16-byte accesses), takes its partner
// j ^ 2^k from lane ^ 2^k by __shfl_xor_sync, and computes its own output
// of the pair -- new0 = m0*a0 + m1*a1 on the lane whose bit k is 0, new1 =
// m2*a0 + m3*a1 on the other -- with the pair form's operations in the
// pair form's order, so the results are the same bits.  Each amplitude is
// read and written once by one lane, in whole 128-byte lines.  Needs 2^n a
// multiple of 32 (n >= 5) so that every warp is full.
template <typename V>
__device__ __forceinline__ V shfl_xor_amp(V a, int mask) {
  V r;
  r.x = __shfl_xor_sync(0xFFFFFFFFu, a.x, mask);
  r.y = __shfl_xor_sync(0xFFFFFFFFu, a.y, mask);
  return r;
}

// Instantiated for complex128 dense and anti-diagonal gates (see
// low_shuffle_enabled for the measurements behind that choice).
template <int KIND, typename V>
__global__ void __launch_bounds__(256) k_pair_shfl(V* __restrict__ s, uint64_t len, int k, M1<V> m,
                                                   const uint8_t* pred) {
  if (skip(pred)) return;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  const int lane = int(threadIdx.x & 31), mask = 1 << k;
  const bool hi = ((lane >> k) & 1) != 0;  // this lane holds a1 of its pair
  // the lane's matrix row: (m0, m1) for new0, (m2, m3) for new1
  const V r0 = hi ? m.m2 : m.m0, r1 = hi ? m.m3 : m.m1;
  if constexpr (std::is_same<V, double2>::value && (KIND == K1_DENSE || KIND == K1_REAL)) {
    const SoftM1 f = soft_matrix<KIND>(m.m0, m.m1, m.m2, m.m3);
    if (f.ok) {  // uniform: the row's factors on the integer pipes
      const softfp::Unpacked u0 = hi ? f.u2 : f.u0, u1 = hi ? f.u3 : f.u1;
      for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < len; j += stride) {
        const double2 own = s[j], other = shfl_xor_amp(own, mask);
        const double2 a0 = hi ? other : own, a1 = hi ? own : other;
        const SoftAmp s0 = sunpack(a0), s1 = sunpack(a1);
        double2 out;
        if (sok(s0) & sok(s1)) {
          if constexpr (KIND == K1_REAL)
            out = cadd(srmul(u0, s0), srmul(u1, s1));
          else
            out = cadd(scmul(r0, u0, a0, s0), scmul(r1, u1, a1, s1));
        } else if constexpr (KIND == K1_REAL) {
          out = cadd(rmul(r0.x, a0), rmul(r1.x, a1));
        } else {
          out = cadd(cmul(r0, a0), cmul(r1, a1));
        }
        s[j] = out;
      }
      return;
    }
  }
  if constexpr (std::is_same<V, double2>::value && KIND == K1_ANTI) {
    const int p1 = unit_power(m.m1), p2 = unit_power(m.m2);
    if ((p1 | p2) >= 0) {  // X, Y and their sign variants: a permutation
      const int p = hi ? p2 : p1;
      for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < len; j += stride)
        s[j] = unit_mul(p, shfl_xor_amp(s[j], mask));
      return;
    }
  }
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < len; j += stride) {
    const V own = s[j], other = shfl_xor_amp(own, mask);
    const V a0 = hi ? other : own, a1 = hi ? own : other;
    if constexpr (KIND == K1_DENSE)
      s[j] = cadd(cmul(r0, a0), cmul(r1, a1));
    else if constexpr (KIND == K1_REAL)
      s[j] = cadd(rmul(r0.x, a0), rmul(r1.x, a1));
    else  // K1_ANTI: new0 = m1*a1, new1 = m2*a0
      s[j] = cmul(hi ? m.m2 : m.m1, other);
  }
}

// Diagonal 1-qubit gate as a flat pass: a_j *= (bit k of j ? m3 : m0).
// Coalesced for every k; same products as the pair form.
template <typename V>
__global__ void __launch_bounds__(256) k_diag(V* __restrict__ s, uint64_t len, int k, V d0, V d1,
                                              const uint8_t* pred) {
  if (skip(pred)) return;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  if constexpr (std::is_same<V, double2>::value) {
    const softfp::Unpacked u0 = softfp::unpack(d0.y), u1 = softfp::unpack(d1.y);
    if (u0.ok & u1.ok) {  // products on the integer pipes, as ev_softpair.cuh
      for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < len; j += stride) {
        const bool one = (j >> k) & 1;
        s[j] = soft_diag(one ? d1 : d0, one ? u1 : u0, s[j]);
      }
      return;
    }
  }
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < len; j += stride)
    s[j] = cmul(((j >> k) & 1) ? d1 : d0, s[j]);
}

// apply_controlled_1q on the active subspace only (kernel.rs:332-358 tests
// i0 & mask == mask on every pair; here the fixed bits are inserted).
template <int KIND, typename V>
__global__ void __launch_bounds__(256) k_ctrl(V* __restrict__ s, uint64_t count, Positions pos,
                                              uint64_t ctrl_mask, int target, M1<V> m,
                                              const uint8_t* pred) {
  if (skip(pred)) return;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  const uint64_t tbit = uint64_t(1) << target;
  if constexpr (std::is_same<V, double2>::value) {
    if constexpr (KIND == K1_ANTI) {  // controlled X, Y and sign variants: a permutation
      const int p1 = unit_power(m.m1), p2 = unit_power(m.m2);
      if ((p1 | p2) >= 0) {
        for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count;
             i += stride) {
          uint64_t j = i;
          for (int q = 0; q < pos.np; ++q) j = insert0(j, pos.p[q]);
          const uint64_t i0 = j | ctrl_mask, i1 = i0 | tbit;
          const double2 a0 = s[i0], a1 = s[i1];
          s[i0] = unit_mul(p1, a1);
          s[i1] = unit_mul(p2, a0);
        }
        return;
      }
    }
    const SoftM1 f = soft_matrix<KIND>(m.m0, m.m1, m.m2, m.m3);
    if (f.ok) {
      for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        uint64_t j = i;
        for (int q = 0; q < pos.np; ++q) j = insert0(j, pos.p[q]);
        const uint64_t i0 = j | ctrl_mask;
        pair_update_soft<KIND>(s, i0, i0 | tbit, f);
      }
      return;
    }
  }
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
    uint64_t j = i;
    for (int q = 0; q < pos.np; ++q) j = insert0(j, pos.p[q]);
    const uint64_t i0 = j | ctrl_mask;
    pair_update<KIND>(s, i0, i0 | tbit, m);
  }
}

// apply_2q over 2^(n-2) quads; idx = [base, base|b, base|a, base|a|b]
// (kernel.rs:54-66).  Row r of the dense form is summed left to right
// (kernel.rs:234-237).
template <int KIND, typename V>
__global__ void __launch_bounds__(256) k_quad(V* __restrict__ s, uint64_t nquads, int lo, int hi,
                                              uint64_t bit_a, uint64_t bit_b, M2<V> m,
                                              const uint8_t* pred) {
  if (skip(pred)) return;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nquads; i += stride) {
    const uint64_t base = insert0(insert0(i, lo), hi);
    const uint64_t i1 = base | bit_b, i2 = base | bit_a, i3 = base | bit_a | bit_b;
    if constexpr (KIND == K2_CNOT) {  // swap i10 <-> i11 (kernel.rs:248-260)
      const V t = s[i2];
      s[i2] = s[i3];
      s[i3] = t;
    } else if constexpr (KIND == K2_CZ) {  // negate i11 (kernel.rs:263-274)
      s[i3] = cneg(s[i3]);
    } else if constexpr (KIND == K2_SWAP) {  // swap i01 <-> i10 (kernel.rs:277-289)
      const V t = s[i1];
      s[i1] = s[i2];
      s[i2] = t;
    } else if constexpr (KIND == K2_DIAG) {
      s[base] = cmul(m.m[0], s[base]);
      s[i1] = cmul(m.m[5], s[i1]);
      s[i2] = cmul(m.m[10], s[i2]);
      s[i3] = cmul(m.m[15], s[i3]);
    } else {  // dense 4x4 (kernel.rs:214-243)
      const V a0 = s[base], a1 = s[i1], a2 = s[i2], a3 = s[i3];
      const uint64_t out[4] = {base, i1, i2, i3};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        V acc = cmul(m.m[4 * r + 0], a0);
        acc = cadd(acc, cmul(m.m[4 * r + 1], a1));
        acc = cadd(acc, cmul(m.m[4 * r + 2], a2));
        acc = cadd(acc, cmul(m.m[4 * r + 3], a3));
        s[out[r]] = acc;
      }
    }
  }
}

// The imaginary parts of a 4x4 matrix, unpacked on the host for the
// integer-pipe products (the factors of the plain multiplications of the
// FMA-form complex multiply).
struct SoftM2 {
  softfp::Unpacked u[16];
};

// Dense (K2_DENSE) and diagonal (K2_DIAG) 4x4 updates on complex128 with the
// plain products on the integer pipes (ev_softpair.cuh), bit-identical to
// k_quad: the FMAs and adds stay on the FP64 pipe.  A quad holding an
// amplitude outside softfp's domain takes the FP64 pipe for that quad.
template <int KIND>
__global__ void __launch_bounds__(256)
    k_quad_soft(double2* __restrict__ s, uint64_t nquads, int lo, int hi, uint64_t bit_a,
                uint64_t bit_b, M2<double2> m, SoftM2 sm, const uint8_t* pred) {
  if (skip(pred)) return;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nquads; i += stride) {
    const uint64_t base = insert0(insert0(i, lo), hi);
    const uint64_t out[4] = {base, base | bit_b, base | bit_a, base | bit_a | bit_b};
    double2 a[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) a[c] = s[out[c]];
    if constexpr (KIND == K2_DIAG) {
#pragma unroll
      for (int c = 0; c < 4; ++c) s[out[c]] = soft_diag(m.m[5 * c], sm.u[5 * c], a[c]);
    } else {
      SoftAmp ua[4];
      uint32_t ok = 1u;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        ua[c] = sunpack(a[c]);
        ok &= sok(ua[c]);
      }
      if (ok) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          double2 acc = scmul(m.m[4 * r + 0], sm.u[4 * r + 0], a[0], ua[0]);
          acc = cadd(acc, scmul(m.m[4 * r + 1], sm.u[4 * r + 1], a[1], ua[1]));
          acc = cadd(acc, scmul(m.m[4 * r + 2], sm.u[4 * r + 2], a[2], ua[2]));
          acc = cadd(acc, scmul(m.m[4 * r + 3], sm.u[4 * r + 3], a[3], ua[3]));
          s[out[r]] = acc;
        }
      } else {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          double2 acc = cmul(m.m[4 * r + 0], a[0]);
          acc = cadd(acc, cmul(m.m[4 * r + 1], a[1]));
          acc = cadd(acc, cmul(m.m[4 * r + 2], a[2]));
          acc = cadd(acc, cmul(m.m[4 * r + 3], a[3]));
          s[out[r]] = acc;
        }
      }
    }
  }
}

// ---- host side ---------------------------------------------------------

static bool is0(const double* z) { return z[0] == 0.0 && z[1] == 0.0; }
static bool is1(const double* z) { return z[0] == 1.0 && z[1] == 0.0; }

Kind1 classify1(const double m[8]) {
  if (is0(m + 2) && is0(m + 4)) {
    if (is1(m) && is1(m + 6)) return K1_IDENT;
    if (is1(m)) return K1_PHASE;
    return K1_DIAG;
  }
  if (is0(m) && is0(m + 6)) return K1_ANTI;
  if (m[1] == 0.0 && m[3] == 0.0 && m[5] == 0.0 && m[7] == 0.0) return K1_REAL;
  return K1_DENSE;
}

// Exact-equality dispatch as in kernel.rs:201-212 (the constant matrices
// hold only 0, 1 and -1, so f64 == is the right test), plus a diagonal case.
Kind2 classify2(const double m[32]) {
  auto entry_is = [&](int r, int c, double re) { return m[2 * (4 * r + c)] == re && m[2 * (4 * r + c) + 1] == 0.0; };
  auto perm = [&](const int cols[4], double last) {
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c)
        if (!entry_is(r, c, c == cols[r] ? (r == 3 ? last : 1.0) : 0.0)) return false;
    return true;
  };
  static const int cnot[4] = {0, 1, 3, 2}, id[4] = {0, 1, 2, 3}, swp[4] = {0, 2, 1, 3};
  if (perm(cnot, 1.0)) return K2_CNOT;
  if (perm(id, -1.0)) return K2_CZ;
  if (perm(swp, 1.0)) return K2_SWAP;
  bool diag = true;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c)
      if (r != c && !is0(m + 2 * (4 * r + c))) diag = false;
  return diag ? K2_DIAG : K2_DENSE;
}

static unsigned grid_for(const ev_state* s, uint64_t work, int per_sm = 8) {
  const uint64_t want = (work + 255) / 256;
  const uint64_t cap = uint64_t(s->num_sms) * uint64_t(per_sm);
  return unsigned(want < 1 ? 1 : (want < cap ? want : cap));
}

// complex128 dense and anti-diagonal gates on qubits 0-4 take the
// warp-shuffle kernel unless EV_LOW_SHUFFLE=0 (the pair kernel; the same
// results).  Measured at 30 qubits (ms, shuffle vs pair): complex128 dense
// on qubit 0 11.73 vs 12.42, X on qubit 1 5.26 vs 5.48, but H on qubit 2
// 8.21 vs 6.41 (each lane unpacks both amplitudes of its pair for the
// integer-pipe products, twice the pair form's work) and every complex64
// gate 2.93-2.95 vs 2.63 (8 bytes in flight per lane and load instead of
// 16) -- so those keep the pair kernel.
static bool low_shuffle_enabled() {
  const char* e = getenv("EV_LOW_SHUFFLE");
  return e == nullptr || e[0] != '0';
}

template <typename V>
static void go_apply1(ev_state* s, Kind1 kind, uint64_t k, const double m[8], const uint8_t* pred) {
  V* a = static_cast<V*>(s->amps);
  const M1<V> mm = to_m1<V>(m);
  const uint64_t npairs = s->len() / 2;
  const unsigned g = grid_for(s, npairs);
  if constexpr (std::is_same<V, double2>::value) {
    static const bool shfl = low_shuffle_enabled();
    if (shfl && k < 5 && s->n >= 5 && (kind == K1_DENSE || kind == K1_ANTI)) {
      const uint64_t len = s->len();
      const unsigned gl = grid_for(s, len);
      if (kind == K1_DENSE)
        k_pair_shfl<K1_DENSE><<<gl, 256, 0, s->stream>>>(a, len, int(k), mm, pred);
      else
        k_pair_shfl<K1_ANTI><<<gl, 256, 0, s->stream>>>(a, len, int(k), mm, pred);
      return;
    }
  }
  switch (kind) {
    case K1_DENSE: k_pair<K1_DENSE><<<g, 256, 0, s->stream>>>(a, npairs, int(k), mm, pred); break;
    case K1_REAL: k_pair<K1_REAL><<<g, 256, 0, s->stream>>>(a, npairs, int(k), mm, pred); break;
    case K1_ANTI: k_pair<K1_ANTI><<<g, 256, 0, s->stream>>>(a, npairs, int(k), mm, pred); break;
    case K1_PHASE: k_pair<K1_PHASE><<<g, 256, 0, s->stream>>>(a, npairs, int(k), mm, pred); break;
    case K1_DIAG:
      k_diag<<<grid_for(s, s->len()), 256, 0, s->stream>>>(a, s->len(), int(k), mm.m0, mm.m3, pred);
      break;
    case K1_IDENT: break;
  }
}

int launch_apply1(ev_state* s, uint64_t k, const double m[8], const uint8_t* pred) {
  const Kind1 kind = classify1(m);
  if (kind == K1_IDENT) return EV_OK;
  const double nt = kind == K1_PHASE ? double(s->len() / 2) : double(s->len());
  ProfScope prof(s, P_GATE, 2.0 * nt * double(s->amp_bytes()));
  s->launches += 1;
  if (s->dtype == EV_C128)
    go_apply1<double2>(s, kind, k, m, pred);
  else
    go_apply1<float2>(s, kind, k, m, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

template <typename V>
static void go_ctrl(ev_state* s, Kind1 kind, const Positions& pos, uint64_t mask, uint64_t t,
                    const double m[8], const uint8_t* pred) {
  V* a = static_cast<V*>(s->amps);
  const M1<V> mm = to_m1<V>(m);
  const uint64_t count = s->len() >> pos.np;
  const unsigned g = grid_for(s, count);
  switch (kind) {
    case K1_DENSE: k_ctrl<K1_DENSE><<<g, 256, 0, s->stream>>>(a, count, pos, mask, int(t), mm, pred); break;
    case K1_REAL: k_ctrl<K1_REAL><<<g, 256, 0, s->stream>>>(a, count, pos, mask, int(t), mm, pred); break;
    case K1_ANTI: k_ctrl<K1_ANTI><<<g, 256, 0, s->stream>>>(a, count, pos, mask, int(t), mm, pred); break;
    case K1_PHASE: k_ctrl<K1_PHASE><<<g, 256, 0, s->stream>>>(a, count, pos, mask, int(t), mm, pred); break;
    case K1_DIAG: k_ctrl<K1_DIAG><<<g, 256, 0, s->stream>>>(a, count, pos, mask, int(t), mm, pred); break;
    case K1_IDENT: break;
  }
}

int launch_controlled(ev_state* s, uint64_t ctrl_mask, uint64_t target, const double m[8],
                      const uint8_t* pred) {
  Positions pos{};
  const uint64_t all = ctrl_mask | (uint64_t(1) << target);
  for (int q = 0; q < 64; ++q)
    if ((all >> q) & 1) pos.p[pos.np++] = q;
  const Kind1 kind = classify1(m);
  if (kind == K1_IDENT) return EV_OK;
  const double nt = double(s->len() >> (pos.np - (kind == K1_PHASE ? 0 : 1)));
  ProfScope prof(s, P_GATE, 2.0 * nt * double(s->amp_bytes()));
  s->launches += 1;
  if (s->dtype == EV_C128)
    go_ctrl<double2>(s, kind, pos, ctrl_mask, target, m, pred);
  else
    go_ctrl<float2>(s, kind, pos, ctrl_mask, target, m, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

template <typename V>
static M2<V> to_m2(const double m[32]) {
  M2<V> r;
  for (int i = 0; i < 16; ++i) {
    if constexpr (sizeof(V) == 16)
      r.m[i] = make_double2(m[2 * i], m[2 * i + 1]);
    else
      r.m[i] = make_float2(float(m[2 * i]), float(m[2 * i + 1]));
  }
  return r;
}

template <typename V>
static void go_apply2_fp64(ev_state* s, Kind2 kind, uint64_t a, uint64_t b, const double m[32],
                           const uint8_t* pred) {
  V* st = static_cast<V*>(s->amps);
  const M2<V> mm = to_m2<V>(m);
  const uint64_t nq = s->len() / 4;
  const int lo = int(a < b ? a : b), hi = int(a < b ? b : a);
  const uint64_t ba = uint64_t(1) << a, bb = uint64_t(1) << b;
  const unsigned g = grid_for(s, nq);
  switch (kind) {
    case K2_CNOT: k_quad<K2_CNOT><<<g, 256, 0, s->stream>>>(st, nq, lo, hi, ba, bb, mm, pred); break;
    case K2_CZ: k_quad<K2_CZ><<<g, 256, 0, s->stream>>>(st, nq, lo, hi, ba, bb, mm, pred); break;
    case K2_SWAP: k_quad<K2_SWAP><<<g, 256, 0, s->stream>>>(st, nq, lo, hi, ba, bb, mm, pred); break;
    case K2_DIAG: k_quad<K2_DIAG><<<g, 256, 0, s->stream>>>(st, nq, lo, hi, ba, bb, mm, pred); break;
    case K2_DENSE: k_quad<K2_DENSE><<<g, 256, 0, s->stream>>>(st, nq, lo, hi, ba, bb, mm, pred); break;
  }
}

template <typename V>
static void go_apply2(ev_state* s, Kind2 kind, uint64_t a, uint64_t b, const double m[32],
                      const uint8_t* pred) {
  go_apply2_fp64<V>(s, kind, a, b, m, pred);
}

// complex128 dense and diagonal 4x4: the integer-pipe products when every
// imaginary part the kind multiplies by is in softfp's domain.
template <>
void go_apply2<double2>(ev_state* s, Kind2 kind, uint64_t a, uint64_t b, const double m[32],
                        const uint8_t* pred) {
  if (kind == K2_DENSE || kind == K2_DIAG) {
    SoftM2 sm;
    uint32_t ok = 1u;
    for (int e = 0; e < 16; ++e) {
      sm.u[e] = softfp::unpack(m[2 * e + 1]);
      if (kind == K2_DENSE || e % 5 == 0) ok &= sm.u[e].ok;
    }
    if (ok) {
      double2* st = static_cast<double2*>(s->amps);
      const M2<double2> mm = to_m2<double2>(m);
      const uint64_t nq = s->len() / 4;
      const int lo = int(a < b ? a : b), hi = int(a < b ? b : a);
      const uint64_t ba = uint64_t(1) << a, bb = uint64_t(1) << b;
      if (kind == K2_DENSE)
        k_quad_soft<K2_DENSE>
            <<<grid_for(s, nq, resident_blocks<k_quad_soft<K2_DENSE>>()), 256, 0, s->stream>>>(
                st, nq, lo, hi, ba, bb, mm, sm, pred);
      else
        k_quad_soft<K2_DIAG>
            <<<grid_for(s, nq, resident_blocks<k_quad_soft<K2_DIAG>>()), 256, 0, s->stream>>>(
                st, nq, lo, hi, ba, bb, mm, sm, pred);
      return;
    }
  }
  go_apply2_fp64<double2>(s, kind, a, b, m, pred);
}

int launch_apply2(ev_state* s, uint64_t a, uint64_t b, const double m[32], const uint8_t* pred) {
  const Kind2 kind = classify2(m);
  const double nt = kind == K2_CZ ? double(s->len() / 4)
                    : (kind == K2_CNOT || kind == K2_SWAP) ? double(s->len() / 2)
                                                            : double(s->len());
  ProfScope prof(s, P_GATE, 2.0 * nt * double(s->amp_bytes()));
  s->launches += 1;
  if (s->dtype == EV_C128)
    go_apply2<double2>(s, kind, a, b, m, pred);
  else
    go_apply2<float2>(s, kind, a, b, m, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

}  // namespace ev

// ---- C ABI: gate kernels --------------------------------------------------

extern "C" int ev_apply_1q(ev_state* s, uint64_t k, const double m[8]) {
  ev::clear_error();
  if (!s || !m) return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_apply_1q: null argument");
  if (k >= s->n)
    return ev::fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                    (unsigned long long)k, (unsigned long long)s->n);
  EV_CUDA(cudaSetDevice(s->device));
  return ev::launch_apply1(s, k, m, nullptr);
}

extern "C" int ev_apply_2q(ev_state* s, uint64_t a, uint64_t b, const double m[32]) {
  ev::clear_error();
  if (!s || !m) return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_apply_2q: null argument");
  if (s->n < 2 || a >= s->n || b >= s->n)
    return ev::fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit out of range for %llu-qubit register",
                    (unsigned long long)s->n);
  if (a == b)
    return ev::fail(EV_ERR_DUPLICATE_QUBIT, "qubit q%llu used more than once in a single gate",
                    (unsigned long long)a);
  EV_CUDA(cudaSetDevice(s->device));
  return ev::launch_apply2(s, a, b, m, nullptr);
}

extern "C" int ev_apply_controlled_1q(ev_state* s, const uint64_t* controls, uint64_t ncontrols,
                                      uint64_t target, const double m[8]) {
  ev::clear_error();
  if (!s || !m || (ncontrols && !controls))
    return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_apply_controlled_1q: null argument");
  if (target >= s->n)
    return ev::fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                    (unsigned long long)target, (unsigned long long)s->n);
  uint64_t mask = 0;
  for (uint64_t j = 0; j < ncontrols; ++j) {
    if (controls[j] >= s->n)
      return ev::fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                      (unsigned long long)controls[j], (unsigned long long)s->n);
    if (controls[j] == target)
      return ev::fail(EV_ERR_DUPLICATE_QUBIT, "qubit q%llu used more than once in a single gate",
                      (unsigned long long)target);
    mask |= uint64_t(1) << controls[j];
  }
  EV_CUDA(cudaSetDevice(s->device));
  return ev::launch_controlled(s, mask, target, m, nullptr);
}
