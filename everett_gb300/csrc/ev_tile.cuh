// ev_tile.cuh -- gate records applied to shared-memory tiles, shared by
// the tile pass (ev_tile.cu) and the batched runner (ev_batch.cu).
//
// A tile is the 2^k amplitudes whose indices agree outside a qubit set T;
// local index bit i is the i-th lowest qubit of T.  Each record is applied
// with the per-amplitude arithmetic of the per-gate kernels (ev_gates.cu,
// the reference's kernel.rs:100-289), so tiling changes no value.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_softpair.cuh"

namespace ev {


enum TileKind : uint8_t {
  T_1Q = 0,  // (possibly controlled) 1-qubit gate; sub-kind in k1
  T_CNOT,
  T_CZ,
  T_SWAP,
  T_DIAG2,
  T_DENSE2
};

struct __align__(16) TileOp {
  uint8_t kind;
  uint8_t k1;      // Kind1 for T_1Q
  uint8_t p0, p1;  // local positions: target / (a, b)
  uint8_t lo, hi;  // T_*2: sorted local positions
  uint8_t nins;    // T_1Q: number of sorted positions in ins[]
  uint8_t soft;    // complex128 T_1Q: products on the integer pipes
                   // (ev_softfp.cuh): 0 none, 1 first amplitude of each
                   // pair, 2 both; real-matrix records 3..6: both, and the
                   // adds of the first soft - 2 output parts too
  uint32_t lmask;  // local control mask
  uint8_t run;     // records from this one on that form a chain (ctype:
                   // pair, quad or diagonal, applied in registers); 0 or 1:
                   // none
  uint8_t sok;     // complex128 T_1Q: the factors in m[8..15] are in the
                   // integer-pipe product's domain (SoftM1::ok)
  uint8_t ctype;   // first record of a chain (run > 1): ChainKind
  uint8_t pad2;
  uint64_t emask;  // controls outside the tile (global bit mask)
  uint64_t ins;    // T_1Q: sorted local positions of (local controls + target),
                   // 4 bits each, lowest position in the low nibble
  uint64_t pad3[2];
  double m[32];    // T_1Q: the 2x2 matrix in m[0..7], then its product
                   // factors unpacked (4 softfp::Unpacked, soft_factors)
};

static_assert(sizeof(TileOp) % 16 == 0, "op records are staged with 16-byte copies");

// What a chain of records (TileOp::run > 1 on its first record) is:
// CH_PAIR  1-qubit records on one target with the same controls, applied to
//          pairs held in registers;
// CH_QUAD  uncontrolled 1-qubit records on two targets, applied to quads;
// CH_DIAG  diagonal records (uncontrolled diagonal and phase 1-qubit
//          records, diagonal 2-qubit records; the chain code also applies
//          CZ), applied to each amplitude in turn: a diagonal record
//          multiplies every amplitude by the entry its index selects,
//          independently of the others.
enum ChainKind : uint8_t { CH_PAIR = 0, CH_QUAD = 1, CH_DIAG = 2 };

// The matrix and integer-pipe flag of a record; records kept elsewhere (the
// batched runner's, whose matrices sit in a shared pool) overload these.
__host__ __device__ __forceinline__ const double* rec_m(const TileOp& op, const double*) {
  return op.m;
}
__host__ __device__ __forceinline__ uint32_t rec_sok(const TileOp& op) { return op.sok; }

struct TilePlan {
  int k, L;
  int nH;
  uint8_t H[40];     // local positions L..k-1 map to global qubits H[0..nH)
  int ncomp;
  uint8_t comp[64];  // global qubits outside T, ascending
};

// Entry i of a record's matrix.  complex128 records hold f64 [re, im]
// pairs; complex64 records hold f32 pairs, rounded once on the host
// (pack_f32_matrix) because GB300 runs f64 -> f32 conversions at its FP64
// rate: converting a 2x2 matrix per record and thread cost more than the
// record's complex64 arithmetic on a 2^13-amplitude tile.
template <typename V>
__device__ __forceinline__ V ldm(const double* m, int i);
template <>
__device__ __forceinline__ double2 ldm<double2>(const double* m, int i) {
  return make_double2(m[2 * i], m[2 * i + 1]);
}
template <>
__device__ __forceinline__ float2 ldm<float2>(const double* m, int i) {
  return reinterpret_cast<const float2*>(m)[i];
}

// Rewrites the first nd doubles of m as nd floats (round to nearest even,
// the device's f64 -> f32 conversion) in its first nd * 4 bytes and zeroes
// the rest of those nd doubles: the complex64 form of a record's matrix.
inline void pack_f32_matrix(double* m, int nd) {
  float f[32];
  for (int j = 0; j < nd; ++j) f[j] = static_cast<float>(m[j]);
  std::memset(m, 0, size_t(nd) * sizeof(double));
  std::memcpy(m, f, size_t(nd) * sizeof(float));
}

__device__ __forceinline__ uint32_t ins0(uint32_t i, int p) {
  return ((i >> p) << (p + 1)) | (i & ((1u << p) - 1));
}

template <int K1, typename V, typename Op>
__device__ __forceinline__ void tile_1q_fp64(V* t, uint32_t count, const Op& op, const double* mm);

// The pair loop of tile_1q with the complex128 products of one (op.soft ==
// 1) or both amplitudes of each pair on the integer pipes (ev_softpair.cuh).
template <int K1, typename Op>
__device__ __forceinline__ void tile_1q_soft(double2* t, uint32_t count, const Op& op,
                                             const double* mm) {
  const SoftM1 f = soft_matrix<K1>(ldm<double2>(mm, 0), ldm<double2>(mm, 1), ldm<double2>(mm, 2),
                                   ldm<double2>(mm, 3));
  if (!f.ok) {  // uniform across the block
    tile_1q_fp64<K1>(t, count, op, mm);
    return;
  }
  const bool both = op.soft >= 2;
  const int nadd = op.soft > 2 ? op.soft - 2 : 0;
  const uint32_t tbit = 1u << op.p0, lmask = op.lmask;
  const int nins = op.nins;
  const uint64_t ins = op.ins;
  const int ins_first = int(ins & 15);
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    uint32_t j = ins0(i, ins_first);
    for (int q = 1; q < nins; ++q) j = ins0(j, int((ins >> (4 * q)) & 15));
    const uint32_t i0 = j | lmask, i1 = i0 | tbit;
    if constexpr (K1 == K1_PHASE) {
      double2 a0 = make_double2(0.0, 0.0), a1 = t[i1];
      soft_pair<K1>(a0, a1, f, both, nadd);
      t[i1] = a1;
    } else {
      double2 a0 = t[i0], a1 = t[i1];
      soft_pair<K1>(a0, a1, f, both, nadd);
      t[i0] = a0;
      t[i1] = a1;
    }
  }
}

// One (possibly controlled) 1-qubit record over the tile: the pair loop is
// specialised per matrix kind, with the matrix held in registers.
template <int K1, typename V, typename Op>
__device__ __forceinline__ void tile_1q(V* t, uint32_t count, const Op& op, const double* mm) {
  if constexpr (std::is_same<V, double2>::value && K1 != K1_ANTI) {
    if (op.soft) {
      tile_1q_soft<K1>(t, count, op, mm);
      return;
    }
  }
  tile_1q_fp64<K1>(t, count, op, mm);
}

template <int K1, typename V, typename Op>
__device__ __forceinline__ void tile_1q_fp64(V* t, uint32_t count, const Op& op, const double* mm) {
  const V m0 = ldm<V>(mm, 0), m1 = ldm<V>(mm, 1), m2 = ldm<V>(mm, 2), m3 = ldm<V>(mm, 3);
  using R = typename Real<V>::T;
  const uint32_t tbit = 1u << op.p0, lmask = op.lmask;
  const int nins = op.nins;
  const uint64_t ins = op.ins;
  const int ins_first = int(ins & 15);
  if constexpr (K1 == K1_DENSE && std::is_same<V, float2>::value) {
    // complex64 records with a real diagonal and an imaginary off-diagonal
    // (Rx, the TFIM's transverse field): 2 FP32 instructions per output part
    // instead of the complex product's 5 (one rounding fewer per part; the
    // complex64 bar is fidelity, not bits)
    if (m0.y == 0.f && m3.y == 0.f && m1.x == 0.f && m2.x == 0.f) {  // uniform
      const float c0 = m0.x, c3 = m3.x, s1 = m1.y, s2 = m2.y;
      for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
        uint32_t j = ins0(i, ins_first);
        for (int q = 1; q < nins; ++q) j = ins0(j, int((ins >> (4 * q)) & 15));
        const uint32_t i0 = j | lmask, i1 = i0 | tbit;
        const float2 a0 = t[i0], a1 = t[i1];
        t[i0] = make_float2(__fmaf_rn(c0, a0.x, -(s1 * a1.y)), __fmaf_rn(c0, a0.y, s1 * a1.x));
        t[i1] = make_float2(__fmaf_rn(c3, a1.x, -(s2 * a0.y)), __fmaf_rn(c3, a1.y, s2 * a0.x));
      }
      return;
    }
  }
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    uint32_t j = ins0(i, ins_first);
    for (int q = 1; q < nins; ++q) j = ins0(j, int((ins >> (4 * q)) & 15));
    const uint32_t i0 = j | lmask, i1 = i0 | tbit;
    if constexpr (K1 == K1_DENSE) {
      const V a0 = t[i0], a1 = t[i1];
      t[i0] = cadd(cmul(m0, a0), cmul(m1, a1));
      t[i1] = cadd(cmul(m2, a0), cmul(m3, a1));
    } else if constexpr (K1 == K1_REAL) {
      const V a0 = t[i0], a1 = t[i1];
      t[i0] = cadd(rmul(R(m0.x), a0), rmul(R(m1.x), a1));
      t[i1] = cadd(rmul(R(m2.x), a0), rmul(R(m3.x), a1));
    } else if constexpr (K1 == K1_DIAG) {
      t[i0] = cmul(m0, t[i0]);
      t[i1] = cmul(m3, t[i1]);
    } else if constexpr (K1 == K1_PHASE) {
      t[i1] = cmul(m3, t[i1]);
    } else if constexpr (K1 == K1_ANTI) {
      const V a0 = t[i0], a1 = t[i1];
      t[i0] = cmul(m1, a1);
      t[i1] = cmul(m2, a0);
    }
  }
}

template <int KIND, typename V, typename Op>
__device__ __forceinline__ void tile_2q(V* t, uint32_t count, const Op& op, const double* mm) {
  const uint32_t ba = 1u << op.p0, bb = 1u << op.p1;
  const int lo = op.lo, hi = op.hi;
  if constexpr (KIND == T_DIAG2 && !std::is_same<V, double2>::value) {
    // complex64: the f64 -> f32 conversions of the four entries run at the
    // FP64 rate on GB300, so they are made once, not per quad
    const V d0 = ldm<V>(mm, 0), d1 = ldm<V>(mm, 5), d2 = ldm<V>(mm, 10), d3 = ldm<V>(mm, 15);
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
      const uint32_t base = ins0(ins0(i, lo), hi);
      const uint32_t i1 = base | bb, i2 = base | ba, i3 = base | ba | bb;
      t[base] = cmul(d0, t[base]);
      t[i1] = cmul(d1, t[i1]);
      t[i2] = cmul(d2, t[i2]);
      t[i3] = cmul(d3, t[i3]);
    }
    return;
  }
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    const uint32_t base = ins0(ins0(i, lo), hi);
    const uint32_t i1 = base | bb, i2 = base | ba, i3 = base | ba | bb;
    if constexpr (KIND == T_CNOT) {
      const V x = t[i2];
      t[i2] = t[i3];
      t[i3] = x;
    } else if constexpr (KIND == T_CZ) {
      t[i3] = cneg(t[i3]);
    } else if constexpr (KIND == T_SWAP) {
      const V x = t[i1];
      t[i1] = t[i2];
      t[i2] = x;
    } else if constexpr (KIND == T_DIAG2) {
      t[base] = cmul(ldm<V>(mm, 0), t[base]);
      t[i1] = cmul(ldm<V>(mm, 5), t[i1]);
      t[i2] = cmul(ldm<V>(mm, 10), t[i2]);
      t[i3] = cmul(ldm<V>(mm, 15), t[i3]);
    } else {  // dense 4x4, rows summed left to right
      const V a[4] = {t[base], t[i1], t[i2], t[i3]};
      const uint32_t out[4] = {base, i1, i2, i3};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        V acc = cmul(ldm<V>(mm, 4 * r + 0), a[0]);
        acc = cadd(acc, cmul(ldm<V>(mm, 4 * r + 1), a[1]));
        acc = cadd(acc, cmul(ldm<V>(mm, 4 * r + 2), a[2]));
        acc = cadd(acc, cmul(ldm<V>(mm, 4 * r + 3), a[3]));
        t[out[r]] = acc;
      }
    }
  }
}

// One 1-qubit record on one pair in registers, with the arithmetic of
// tile_1q_fp64 (FP64 or FP32 pipe).
template <int K1, typename V>
__device__ __forceinline__ void pair_fp(const double* mm, V& a0, V& a1) {
  using R = typename Real<V>::T;
  if constexpr (K1 == K1_DENSE) {
    const V m0 = ldm<V>(mm, 0), m1 = ldm<V>(mm, 1), m2 = ldm<V>(mm, 2), m3 = ldm<V>(mm, 3);
    if constexpr (std::is_same<V, float2>::value) {
      // Rx-like complex64 records, as in tile_1q_fp64
      if (m0.y == 0.f && m3.y == 0.f && m1.x == 0.f && m2.x == 0.f) {
        const float2 n0 = make_float2(__fmaf_rn(m0.x, a0.x, -(m1.y * a1.y)),
                                      __fmaf_rn(m0.x, a0.y, m1.y * a1.x));
        a1 = make_float2(__fmaf_rn(m3.x, a1.x, -(m2.y * a0.y)), __fmaf_rn(m3.x, a1.y, m2.y * a0.x));
        a0 = n0;
        return;
      }
    }
    const V n0 = cadd(cmul(m0, a0), cmul(m1, a1));
    a1 = cadd(cmul(m2, a0), cmul(m3, a1));
    a0 = n0;
  } else if constexpr (K1 == K1_REAL) {
    const R r0 = ldm<V>(mm, 0).x, r1 = ldm<V>(mm, 1).x, r2 = ldm<V>(mm, 2).x, r3 = ldm<V>(mm, 3).x;
    const V n0 = cadd(rmul(r0, a0), rmul(r1, a1));
    a1 = cadd(rmul(r2, a0), rmul(r3, a1));
    a0 = n0;
  } else if constexpr (K1 == K1_DIAG) {
    a0 = cmul(ldm<V>(mm, 0), a0);
    a1 = cmul(ldm<V>(mm, 3), a1);
  } else if constexpr (K1 == K1_PHASE) {
    a1 = cmul(ldm<V>(mm, 3), a1);
  } else if constexpr (K1 == K1_ANTI) {
    const V n0 = cmul(ldm<V>(mm, 1), a1);
    a1 = cmul(ldm<V>(mm, 2), a0);
    a0 = n0;
  }
}

// One record of a chain on two pairs held in registers: complex128 records
// with their factors in range take the integer-pipe products, the rest the
// plain arithmetic.  The two pairs are updated one after the other: a
// straight-line block over both needs more registers than a 64-register
// thread has, and its spills cost more than its extra overlap gains.
template <int K1, typename V, typename Op>
__device__ __forceinline__ void chain_rec(const Op& op, const double* mats, V& a0, V& a1, V& b0,
                                          V& b1) {
  const double* mm = rec_m(op, mats);
  if constexpr (std::is_same<V, double2>::value && K1 != K1_ANTI && K1 != K1_IDENT) {
    if (op.soft && rec_sok(op)) {  // uniform across the block
      SoftM1 f;
      f.m0 = ldm<double2>(mm, 0);
      f.m1 = ldm<double2>(mm, 1);
      f.m2 = ldm<double2>(mm, 2);
      f.m3 = ldm<double2>(mm, 3);
      const softfp::Unpacked* u = reinterpret_cast<const softfp::Unpacked*>(mm + 8);
      f.u0 = u[0];
      f.u1 = u[1];
      f.u2 = u[2];
      f.u3 = u[3];
      f.ok = 1;
      const bool both = op.soft >= 2;
      const int nadd = op.soft > 2 ? op.soft - 2 : 0;
      soft_pair<K1>(a0, a1, f, both, nadd);
      soft_pair<K1>(b0, b1, f, both, nadd);
      return;
    }
  }
  pair_fp<K1>(mm, a0, a1);
  pair_fp<K1>(mm, b0, b1);
}

template <typename V, typename Op>
__device__ __forceinline__ void chain_rec_any(const Op& op, const double* mats, V& a0, V& a1,
                                              V& b0, V& b1);

// A chain of `run` 1-qubit records that share their target and controls:
// each thread loads two pairs, applies every record of the chain to them in
// circuit order and stores them once.  Every amplitude sees the same
// operations in the same order as record-by-record application.
template <typename V, typename Op>
__device__ void tile_chain(V* t, uint32_t count, const Op* ops, int run, const double* mats) {
  const Op& op0 = ops[0];
  const uint32_t tbit = 1u << op0.p0, lmask = op0.lmask;
  const int nins = op0.nins;
  const uint64_t ins = op0.ins;
  const int ins_first = int(ins & 15);
  const uint32_t stride = blockDim.x;
  for (uint32_t i = threadIdx.x; i < count; i += 2 * stride) {
    const uint32_t i2 = i + stride;
    const bool two = i2 < count;
    uint32_t ja = ins0(i, ins_first), jb = ins0(two ? i2 : i, ins_first);
    for (int q = 1; q < nins; ++q) {
      const int p = int((ins >> (4 * q)) & 15);
      ja = ins0(ja, p);
      jb = ins0(jb, p);
    }
    ja |= lmask;
    jb |= lmask;
    V a0 = t[ja], a1 = t[ja | tbit], b0 = t[jb], b1 = t[jb | tbit];
    for (int r = 0; r < run; ++r) chain_rec_any(ops[r], mats, a0, a1, b0, b1);
    t[ja] = a0;
    t[ja | tbit] = a1;
    if (two) {
      t[jb] = b0;
      t[jb | tbit] = b1;
    }
  }
}

// chain_rec for the record's kind.
template <typename V, typename Op>
__device__ __forceinline__ void chain_rec_any(const Op& op, const double* mats, V& a0, V& a1,
                                              V& b0, V& b1) {
  switch (op.k1) {
    case K1_DENSE: chain_rec<K1_DENSE>(op, mats, a0, a1, b0, b1); break;
    case K1_REAL: chain_rec<K1_REAL>(op, mats, a0, a1, b0, b1); break;
    case K1_DIAG: chain_rec<K1_DIAG>(op, mats, a0, a1, b0, b1); break;
    case K1_PHASE: chain_rec<K1_PHASE>(op, mats, a0, a1, b0, b1); break;
    case K1_ANTI: chain_rec<K1_ANTI>(op, mats, a0, a1, b0, b1); break;
    default: break;  // identity
  }
}

// A chain of `run` uncontrolled 1-qubit records whose targets are two local
// positions lo < hi (TileOp::lo/hi of the first record): each thread holds
// the four amplitudes of a quad in registers; a record on lo updates the
// pairs (q0, q1) and (q2, q3), one on hi the pairs (q0, q2) and (q1, q3).
// The pairs of a record are disjoint and each amplitude sees its records in
// circuit order, so the results equal record-by-record application.
template <typename V, typename Op>
__device__ void tile_quad_chain(V* t, uint32_t size, const Op* ops, int run, const double* mats) {
  const int lo = ops[0].lo, hi = ops[0].hi;
  const uint32_t lob = 1u << lo, hib = 1u << hi;
  const uint32_t count = size >> 2;
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    const uint32_t base = ins0(ins0(i, lo), hi);
    V q0 = t[base], q1 = t[base | lob], q2 = t[base | hib], q3 = t[base | lob | hib];
    for (int r = 0; r < run; ++r) {
      const Op& op = ops[r];
      if (op.p0 == lo)
        chain_rec_any(op, mats, q0, q1, q2, q3);
      else
        chain_rec_any(op, mats, q0, q2, q1, q3);
    }
    t[base] = q0;
    t[base | lob] = q1;
    t[base | hib] = q2;
    t[base | lob | hib] = q3;
  }
}

// A chain of `run` diagonal records (CH_DIAG): each thread holds a few
// amplitudes (local indices l0 + j * blockDim.x) in registers, reads each
// record once and applies it to all of them, in circuit order.  Records act
// on each amplitude alone, so this equals record-by-record application.
template <typename V, typename Op>
__device__ void tile_diag_chain(V* t, uint32_t size, const Op* ops, int run, const double* mats) {
  // one amplitude at a time for complex128: more live registers spill the
  // 64-register tile pass
  constexpr int CH = sizeof(V) == 16 ? 1 : 4;
  const uint32_t nb = blockDim.x;
  for (uint32_t l0 = threadIdx.x; l0 < size; l0 += CH * nb) {
    V a[CH];
#pragma unroll
    for (int j = 0; j < CH; ++j)
      if (l0 + j * nb < size) a[j] = t[l0 + j * nb];
    // not unrolled: with the compiler's unrolling this loop ran no iteration
    // for a 2-record chain of the batched runner (its records in shared
    // memory or in global memory alike; found by device printf, fixed by this
    // pragma or by ptxas -O0)
#pragma unroll 1
    for (int r = 0; r < run; ++r) {
      const Op& op = ops[r];
      const double* mm = rec_m(op, mats);
      const int kind = op.kind;
      const uint32_t b0 = 1u << op.p0;
      if (kind == T_1Q) {
        const int k1 = op.k1;
        const uint32_t lmask = op.lmask;
        const V e0 = ldm<V>(mm, 0), e3 = ldm<V>(mm, 3);
        bool soft0 = false, soft1 = false;
        if constexpr (std::is_same<V, double2>::value) {
          soft0 = op.soft && rec_sok(op);
          soft1 = soft0 && op.soft >= 2;
        }
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const uint32_t l = l0 + j * nb;
          const bool one = (l & b0) != 0;
          // identity records, amplitudes with a local control at 0 and the
          // 0 row of a phase record keep their value
          if (k1 != K1_IDENT && (l & lmask) == lmask && (one || k1 != K1_PHASE)) {
            bool done = false;
            if constexpr (std::is_same<V, double2>::value) {
              if (one ? soft1 : soft0) {
                const softfp::Unpacked* u = reinterpret_cast<const softfp::Unpacked*>(mm + 8);
                a[j] = soft_diag(one ? e3 : e0, u[one ? 3 : 0], a[j]);
                done = true;
              }
            }
            if (!done) a[j] = cmul(one ? e3 : e0, a[j]);
          }
        }
      } else if (kind == T_CZ) {
        const uint32_t b1 = 1u << op.p1;
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const uint32_t l = l0 + j * nb;
          if ((l & b0) && (l & b1)) a[j] = cneg(a[j]);
        }
      } else if (op.k1 == 1) {  // parity-diagonal T_DIAG2: entry 0 or 5 by the bits' parity
        const uint32_t p0 = op.p0, p1 = op.p1;
        const V d0 = ldm<V>(mm, 0), d1 = ldm<V>(mm, 5);
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const uint32_t l = l0 + j * nb;
          a[j] = cmul((((l >> p0) ^ (l >> p1)) & 1u) ? d1 : d0, a[j]);
        }
      } else {  // T_DIAG2: entry 5c with c = 2 * bit(p0) + bit(p1), as tile_2q maps them
        const uint32_t b1 = 1u << op.p1;
        const V d0 = ldm<V>(mm, 0), d1 = ldm<V>(mm, 5), d2 = ldm<V>(mm, 10), d3 = ldm<V>(mm, 15);
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const uint32_t l = l0 + j * nb;
          const V d = (l & b0) ? ((l & b1) ? d3 : d2) : ((l & b1) ? d1 : d0);
          a[j] = cmul(d, a[j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < CH; ++j)
      if (l0 + j * nb < size) t[l0 + j * nb] = a[j];
  }
}

template <typename V, typename Op>
__device__ void apply_tile_op(V* t, int k, const Op& op, const double* mm) {
  const uint32_t size = 1u << k;
  if (op.kind == T_1Q) {
    const uint32_t count = size >> op.nins;
    switch (op.k1) {
      case K1_DENSE: tile_1q<K1_DENSE>(t, count, op, mm); break;
      case K1_REAL: tile_1q<K1_REAL>(t, count, op, mm); break;
      case K1_DIAG: tile_1q<K1_DIAG>(t, count, op, mm); break;
      case K1_PHASE: tile_1q<K1_PHASE>(t, count, op, mm); break;
      case K1_ANTI: tile_1q<K1_ANTI>(t, count, op, mm); break;
      default: break;
    }
    return;
  }
  const uint32_t count = size >> 2;
  switch (op.kind) {
    case T_CNOT: tile_2q<T_CNOT>(t, count, op, mm); break;
    case T_CZ: tile_2q<T_CZ>(t, count, op, mm); break;
    case T_SWAP: tile_2q<T_SWAP>(t, count, op, mm); break;
    case T_DIAG2: tile_2q<T_DIAG2>(t, count, op, mm); break;
    default: tile_2q<T_DENSE2>(t, count, op, mm); break;
  }
}

// ---- host planning ---------------------------------------------------------

struct Pass {
  std::vector<uint64_t> ops;  // op indices in application order
  uint64_t tset;              // global qubits of the tile
};

inline uint64_t data_qubits(const ev_op& op) {
  switch (op.kind) {
    case EV_OP_APPLY1:
    case EV_OP_CONTROLLED:
      return uint64_t(1) << op.q0;
    case EV_OP_APPLY2:
      return (uint64_t(1) << op.q0) | (uint64_t(1) << op.q1);
    default:
      return 0;
  }
}

inline int popc(uint64_t x) { return __builtin_popcountll(x); }

// Greedy: extend the current pass while the union of data qubits (plus the
// L lowest qubits) fits in k, then fill T with the lowest unused qubits.
// Every qubit an op reads or writes (data qubits and controls).
inline uint64_t all_qubits(const ev_circuit* c, const ev_op& op) {
  uint64_t m = data_qubits(op);
  if (op.kind == EV_OP_CONTROLLED)
    for (uint32_t j = 0; j < op.nctrl; ++j) m |= uint64_t(1) << c->ctrl_pool[op.ctrl_off + j];
  return m;
}

// Greedy pass planning over ops [first, last).  In order (reorder = false)
// a pass is the longest run of consecutive ops whose data qubits, with the
// L lowest qubits, fit in k; this keeps every amplitude's sequence of
// roundings, so complex128 results stay bit-identical.  With reorder = true
// a pass also takes later ops that touch no qubit of an op left behind
// (they commute with everything they jump), which packs many more gates per
// pass at the cost of a different rounding order.  T is filled up to k with
// the lowest unused qubits.
inline std::vector<Pass> plan_passes(const ev_circuit* c, uint64_t first, uint64_t last, int n,
                                     int k, int L, uint64_t max_ops = 48, bool reorder = false) {
  std::vector<Pass> passes;
  const uint64_t low = (L >= 64) ? ~0ull : ((uint64_t(1) << L) - 1);
  const uint64_t everything = n >= 64 ? ~0ull : ((uint64_t(1) << n) - 1);
  std::vector<uint64_t> pending;
  for (uint64_t j = first; j < last; ++j) pending.push_back(j);
  size_t head = 0;  // in-order mode consumes pending from the front
  while (head < pending.size()) {
    Pass p;
    uint64_t set = low, blocked = 0;
    if (!reorder) {
      while (head < pending.size() && p.ops.size() < max_ops) {
        const uint64_t want = set | data_qubits(c->ops[pending[head]]);
        if (popc(want) > k) break;
        set = want;
        p.ops.push_back(pending[head++]);
      }
    } else {
      std::vector<uint64_t> rest;
      for (size_t i = head; i < pending.size(); ++i) {
        const ev_op& op = c->ops[pending[i]];
        const uint64_t aq = all_qubits(c, op), dq = data_qubits(op);
        if ((aq & blocked) == 0 && popc(set | dq) <= k && p.ops.size() < max_ops &&
            blocked != everything) {
          set |= dq;
          p.ops.push_back(pending[i]);
        } else {
          blocked |= aq;
          rest.push_back(pending[i]);
        }
      }
      pending.swap(rest);
      head = 0;
    }
    for (int q = 0; q < n && popc(set) < k; ++q) set |= uint64_t(1) << q;
    p.tset = set;
    passes.push_back(std::move(p));
  }
  return passes;
}

inline void encode_op(const ev_circuit* c, const ev_op& op, uint64_t tset, const int* local,
                      TileOp* out) {
  std::memset(out, 0, sizeof(*out));
  std::memcpy(out->m, op.m, sizeof(op.m));
  if (op.kind == EV_OP_APPLY2) {
    switch (classify2(op.m)) {
      case K2_CNOT: out->kind = T_CNOT; break;
      case K2_CZ: out->kind = T_CZ; break;
      case K2_SWAP: out->kind = T_SWAP; break;
      case K2_DIAG: {
        out->kind = T_DIAG2;
        // k1 = 1 marks a parity-diagonal record (entries 0 and 15 equal, 5
        // and 10 equal: Rzz and its kin), whose entry is picked by the
        // parity of the two bits alone
        const double* m = op.m;
        out->k1 = uint8_t(m[0] == m[30] && m[1] == m[31] && m[10] == m[20] && m[11] == m[21] &&
                          std::signbit(m[0]) == std::signbit(m[30]) &&
                          std::signbit(m[1]) == std::signbit(m[31]) &&
                          std::signbit(m[10]) == std::signbit(m[20]) &&
                          std::signbit(m[11]) == std::signbit(m[21]));
        break;
      }
      default: out->kind = T_DENSE2; break;
    }
    out->p0 = uint8_t(local[op.q0]);
    out->p1 = uint8_t(local[op.q1]);
    out->lo = std::min(out->p0, out->p1);
    out->hi = std::max(out->p0, out->p1);
    return;
  }
  out->kind = T_1Q;
  out->k1 = uint8_t(classify1(op.m));
  out->sok = uint8_t(soft_factors(out->k1, op.m, reinterpret_cast<softfp::Unpacked*>(out->m + 8)));
  out->p0 = uint8_t(local[op.q0]);
  uint32_t lmask = 0;
  uint64_t emask = 0;
  if (op.kind == EV_OP_CONTROLLED)
    for (uint32_t j = 0; j < op.nctrl; ++j) {
      const uint64_t q = c->ctrl_pool[op.ctrl_off + j];
      if ((tset >> q) & 1)
        lmask |= 1u << local[q];
      else
        emask |= uint64_t(1) << q;
    }
  out->lmask = lmask;
  out->emask = emask;
  const uint32_t all = lmask | (1u << out->p0);
  int ni = 0;
  uint64_t packed = 0;
  for (int p = 0; p < 16; ++p)
    if ((all >> p) & 1) packed |= uint64_t(p) << (4 * ni++);
  out->ins = packed;
  out->nins = uint8_t(ni);
}

// Which chains a pass forms (TileOp::run): pair chains, quad chains,
// diagonal chains.  All give the same results.
struct ChainSet {
  bool pairs, quads, diag;
};

// A ChainSet from an environment variable: "0" none, otherwise letters p
// (pair), q (quad), d (diagonal), or the levels 1 (p), 2 (pq), 3 (pqd).
// EV_TILE_CHAIN sets the tile pass's (default pqd), EV_BATCH_CHAIN the
// batched runner's.
inline ChainSet chain_set(const char* var, ChainSet dflt) {
  const char* e = getenv(var);
  if (e == nullptr || e[0] == 0) return dflt;
  if (e[1] == 0 && e[0] >= '0' && e[0] <= '3') {
    const int l = e[0] - '0';
    return ChainSet{l >= 1, l >= 2, l >= 3};
  }
  ChainSet c{false, false, false};
  for (const char* x = e; *x; ++x) {
    if (*x == 'p') c.pairs = true;
    else if (*x == 'q') c.quads = true;
    else if (*x == 'd') c.diag = true;
    else return dflt;
  }
  return c;
}

// Records a diagonal chain takes: diagonal 2-qubit records, and diagonal,
// phase and identity 1-qubit records without local controls.  A CZ or a
// locally controlled record touches a fraction of the tile on its own, which
// a chain would test amplitude by amplitude: the 30-qubit QFT, whose
// controlled phases would chain, 1.59 -> 1.93 s with them in; 28-qubit Haar
// layers with CZ bricks 3.79 -> 4.11 s with the CZs in.
inline bool is_diag_rec(const TileOp& o) {
  if (o.kind == T_DIAG2) return true;
  return o.kind == T_1Q && o.lmask == 0 &&
         (o.k1 == K1_DIAG || o.k1 == K1_PHASE || o.k1 == K1_IDENT);
}

// Marks the chains of a pass's records (TileOp::run, TileOp::ctype).  A run
// of consecutive uncontrolled 1-qubit records with the same outside controls
// whose targets are two local positions becomes a quad chain (lo/hi set on
// its first record); a run on one target with the same controls becomes a
// pair chain; a longer run of diagonal records with the same outside
// controls becomes a diagonal chain instead.  Only the kinds in cs form, and
// no chain is longer than maxrun records.
inline void mark_chains(TileOp* ops, size_t nops, ChainSet cs, size_t maxrun = 255) {
  const bool quads = cs.quads, diag = cs.diag;
  for (size_t j = 0; j < nops;) {
    TileOp& h = ops[j];
    size_t d = j;
    if (diag)
      while (d < nops && d - j < maxrun && is_diag_rec(ops[d]) && ops[d].emask == h.emask) ++d;
    size_t e = j + 1;
    int t2 = -1;
    if (h.kind == T_1Q && h.lmask == 0 && quads) {
      while (e < nops && e - j < maxrun && ops[e].kind == T_1Q && ops[e].lmask == 0 &&
             ops[e].emask == h.emask) {
        const int p = ops[e].p0;
        if (p != h.p0 && p != t2) {
          if (t2 >= 0) break;
          t2 = p;
        }
        ++e;
      }
    } else if (h.kind == T_1Q && cs.pairs) {
      while (e < nops && e - j < maxrun && ops[e].kind == T_1Q && ops[e].p0 == h.p0 &&
             ops[e].lmask == h.lmask && ops[e].emask == h.emask)
        ++e;
    }
    if (d - j >= 2 && d > e) {
      h.run = uint8_t(d - j);
      h.ctype = CH_DIAG;
      for (size_t r = j + 1; r < d; ++r) ops[r].run = 0;
      j = d;
      continue;
    }
    h.run = uint8_t(e - j);
    h.ctype = CH_PAIR;
    if (t2 >= 0) {
      h.lo = uint8_t(std::min<int>(h.p0, t2));
      h.hi = uint8_t(std::max<int>(h.p0, t2));
      h.ctype = CH_QUAD;
    }
    for (size_t r = j + 1; r < e; ++r) ops[r].run = 0;
    j = e;
  }
}

}  // namespace ev
