// ev_softpair.cuh -- the complex128 pair update of a 1-qubit record with its
// products formed on the integer pipes (ev_softfp.cuh).
//
// The FP64 pipe bounds the complex128 gate passes.  A correctly rounded
// product formed by softfp::mul is bit-identical to the FP64 pipe's, so the
// pair update below returns exactly what the FP64-only form returns
// (pair_update in ev_gates.cu, tile_1q in ev_tile.cuh, the reference's
// kernel.rs:113-116): the FMAs and adds stay on the FP64 pipe, the plain
// products move.  A pair with an operand outside the fast path (a zero, a
// subnormal, a magnitude far from 1) takes the FP64 pipe for that pair.
#pragma once

#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_softfp.cuh"

namespace ev {

struct SoftAmp {
  softfp::Unpacked x, y;
};
__device__ __forceinline__ SoftAmp sunpack(double2 a) {
  return SoftAmp{softfp::unpack(a.x), softfp::unpack(a.y)};
}
__device__ __forceinline__ uint32_t sok(const SoftAmp& a) { return a.x.ok & a.y.ok; }
// r * a for a real r, as rmul
__device__ __forceinline__ double2 srmul(const softfp::Unpacked& r, const SoftAmp& a) {
  return make_double2(softfp::mul(r, a.x), softfp::mul(r, a.y));
}
// m * a in FMA form, as cmul; my is m.y unpacked
__device__ __forceinline__ double2 scmul(double2 m, const softfp::Unpacked& my, double2 a,
                                         const SoftAmp& ua) {
  return make_double2(__fma_rn(m.x, a.x, -softfp::mul(my, ua.y)),
                      __fma_rn(m.x, a.y, softfp::mul(my, ua.x)));
}

// The matrix of a record, unpacked once: the real parts for real matrices,
// the imaginary parts (the factors of the FMA-form product's plain
// multiplications) otherwise.  ok is set when every factor the kind uses is
// in the fast path's domain.
struct SoftM1 {
  double2 m0, m1, m2, m3;
  softfp::Unpacked u0, u1, u2, u3;
  uint32_t ok;
};

template <int K1>
__device__ __forceinline__ SoftM1 soft_matrix(double2 m0, double2 m1, double2 m2, double2 m3) {
  constexpr bool kReal = K1 == K1_REAL;
  SoftM1 f;
  f.m0 = m0;
  f.m1 = m1;
  f.m2 = m2;
  f.m3 = m3;
  f.u0 = softfp::unpack(kReal ? m0.x : m0.y);
  f.u1 = softfp::unpack(kReal ? m1.x : m1.y);
  f.u2 = softfp::unpack(kReal ? m2.x : m2.y);
  f.u3 = softfp::unpack(kReal ? m3.x : m3.y);
  if constexpr (K1 == K1_DIAG) f.ok = f.u0.ok & f.u3.ok;
  else if constexpr (K1 == K1_PHASE) f.ok = f.u3.ok;
  else if constexpr (K1 == K1_REAL || K1 == K1_DENSE) f.ok = f.u0.ok & f.u1.ok & f.u2.ok & f.u3.ok;
  else f.ok = 0;  // anti-diagonal and identity records stay on the FP64 pipe
  return f;
}

// The same factors for a matrix m (interleaved [re, im], row-major 2x2) of
// kind k1, formed once on the host for records whose matrices travel with
// them; the return value is SoftM1::ok.
__host__ __device__ inline uint32_t soft_factors(int k1, const double* m, softfp::Unpacked u[4]) {
  const int part = k1 == K1_REAL ? 0 : 1;
  for (int j = 0; j < 4; ++j) u[j] = softfp::unpack(m[2 * j + part]);
  switch (k1) {
    case K1_DIAG: return u[0].ok & u[3].ok;
    case K1_PHASE: return u[3].ok;
    case K1_REAL:
    case K1_DENSE: return u[0].ok & u[1].ok & u[2].ok & u[3].ok;
    default: return 0;
  }
}

// x + y, on the integer pipes (softfp::add) when soft is set and both
// operands are in its domain, else on the FP64 pipe: the same bits.
__device__ __forceinline__ double sadd(double x, double y, bool soft) {
  return (soft && softfp::add_ok(x, y)) ? softfp::add(x, y) : __dadd_rn(x, y);
}

// new0 = m0*a0 + m1*a1, new1 = m2*a0 + m3*a1 for a record of kind K1 (REAL,
// DENSE, DIAG or PHASE; PHASE reads and writes a1 only), with the products
// of new0 (both == false) or of both outputs on the integer pipes; for REAL
// records with both set, the first nadd of the four output parts' adds too.
template <int K1>
__device__ __forceinline__ void soft_pair(double2& a0, double2& a1, const SoftM1& f, bool both,
                                          int nadd = 0) {
  if constexpr (K1 == K1_REAL || K1 == K1_DENSE) {
    const SoftAmp s0 = sunpack(a0), s1 = sunpack(a1);
    double2 n0, n1;
    if (sok(s0) & sok(s1)) {
      if constexpr (K1 == K1_REAL) {
        if (both && nadd > 0) {  // uniform across the block
          const double2 p0 = srmul(f.u0, s0), q0 = srmul(f.u1, s1);
          const double2 p1 = srmul(f.u2, s0), q1 = srmul(f.u3, s1);
          a0 = make_double2(sadd(p0.x, q0.x, nadd >= 1), sadd(p0.y, q0.y, nadd >= 2));
          a1 = make_double2(sadd(p1.x, q1.x, nadd >= 3), sadd(p1.y, q1.y, nadd >= 4));
          return;
        }
        n0 = cadd(srmul(f.u0, s0), srmul(f.u1, s1));
        n1 = both ? cadd(srmul(f.u2, s0), srmul(f.u3, s1))
                  : cadd(rmul(f.m2.x, a0), rmul(f.m3.x, a1));
      } else {
        n0 = cadd(scmul(f.m0, f.u0, a0, s0), scmul(f.m1, f.u1, a1, s1));
        n1 = both ? cadd(scmul(f.m2, f.u2, a0, s0), scmul(f.m3, f.u3, a1, s1))
                  : cadd(cmul(f.m2, a0), cmul(f.m3, a1));
      }
    } else if constexpr (K1 == K1_REAL) {
      n0 = cadd(rmul(f.m0.x, a0), rmul(f.m1.x, a1));
      n1 = cadd(rmul(f.m2.x, a0), rmul(f.m3.x, a1));
    } else {
      n0 = cadd(cmul(f.m0, a0), cmul(f.m1, a1));
      n1 = cadd(cmul(f.m2, a0), cmul(f.m3, a1));
    }
    a0 = n0;
    a1 = n1;
  } else if constexpr (K1 == K1_DIAG) {
    const SoftAmp s0 = sunpack(a0);
    const double2 n0 = sok(s0) ? scmul(f.m0, f.u0, a0, s0) : cmul(f.m0, a0);
    if (both) {
      const SoftAmp s1 = sunpack(a1);
      a1 = sok(s1) ? scmul(f.m3, f.u3, a1, s1) : cmul(f.m3, a1);
    } else {
      a1 = cmul(f.m3, a1);
    }
    a0 = n0;
  } else if constexpr (K1 == K1_PHASE) {
    const SoftAmp s1 = sunpack(a1);
    a1 = sok(s1) ? scmul(f.m3, f.u3, a1, s1) : cmul(f.m3, a1);
  }
}

// One amplitude times a diagonal entry d (du = d.y unpacked), as cmul(d, a).
__device__ __forceinline__ double2 soft_diag(double2 d, const softfp::Unpacked& du, double2 a) {
  const SoftAmp s = sunpack(a);
  return sok(s) ? scmul(d, du, a, s) : cmul(d, a);
}

}  // namespace ev
