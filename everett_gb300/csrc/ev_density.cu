// ev_density.cu -- density matrices in HBM (src/density.rs, src/noise.rs,
// src/backend/density_matrix.rs).
//
// rho is 2^n x 2^n complex128, row-major: element (i, j) at i * 2^n + j, so
// the matrix is a 2n-qubit vector whose low n bits index the column and high
// n bits the row.  The reference applies a gate as two full passes with a
// scratch matrix (left_multiply: U rho, then right_multiply_adjoint:
// (U rho) U^dagger) and a controlled gate through a full 2^n x 2^n unitary.
// Here one kernel per gate takes a 2x2 (4x4 for two qubits) block of rows x
// columns into registers, does the left products column by column and then
// the right products row by row, and writes the block back: one HBM pass,
// the reference's products and sums in the reference's order (the right
// product keeps its operand order, x * conj(u), which the FMA-form
// imaginary part is not symmetric in).  Controls select rows (left) and
// columns (right) independently, which is what the full unitary's identity
// rows and columns do.  A channel sums K rho K^dagger over its Kraus
// operators per block in the same order, starting from the first term.
// Results equal the reference bit for bit, signed zeros aside, until a
// measurement, whose probability sums (and hence the renormalisation)
// agree to rounding.
#include <cmath>
#include <cstring>
#include <vector>

#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_softpair.cuh"

struct ev_dm {
  uint64_t n = 0;
  int device = 0;
  int num_sms = 0;
  double2* rho = nullptr;
  cudaStream_t stream = nullptr;
  void* scratch = nullptr;  // partials | result | meas | pred | counter
  double* partials = nullptr;
  double* result = nullptr;
  double* meas = nullptr;
  uint8_t* pred = nullptr;
  uint32_t* counter = nullptr;
  uint64_t dim() const { return uint64_t(1) << n; }
  uint64_t elems() const { return uint64_t(1) << (2 * n); }
};

namespace ev {
namespace {

constexpr int kDmThreads = 256;
constexpr int kDmRedBlocks = 1024;
constexpr uint64_t kDmMaxQubits = 16;  // 4^16 x 16 B = 64 GiB

__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ bool dm_skip(const uint8_t* pred) { return pred != nullptr && *pred == 0; }

struct U1 {
  double2 m[4];
};
struct U2 {
  double2 m[16];
};
struct KrausSet {
  double2 k[EV_MAX_KRAUS][4];
  int nops;
};

// left: (x_top, x_bot) of one column -> U (x_top, x_bot)
__device__ __forceinline__ void left2(const double2* u, double2& a, double2& b) {
  const double2 t = cadd(cmul(u[0], a), cmul(u[1], b));
  const double2 s = cadd(cmul(u[2], a), cmul(u[3], b));
  a = t;
  b = s;
}
// right: (y_left, y_right) of one row -> (y U^dagger): z_c = sum_k y_k conj(u[c][k])
__device__ __forceinline__ void right2(const double2* u, double2& a, double2& b) {
  const double2 t = cadd(cmul(a, cconj(u[0])), cmul(b, cconj(u[1])));
  const double2 s = cadd(cmul(a, cconj(u[2])), cmul(b, cconj(u[3])));
  a = t;
  b = s;
}

// The same left and right products with their multiplications formed on
// the integer pipes (ev_softfp.cuh: a correctly rounded product, bit-identical
// to the FP64 pipe's), for elements whose parts are normal and within the
// fast domain.  Each matrix entry is classified once per CTA:
//   FULL  both parts non-zero: the FMA form stays, its plain products move;
//   REAL  imaginary part +-0: u * x = (RN(u.x x.x), RN(u.x x.y)) exactly
//         (the FMA form adds a signed zero to a non-zero product);
//   IMAG  real part +-0: u * x = (-RN(u.y x.y), RN(u.y x.x)) exactly;
//   ZERO  both parts +-0: the term is a signed zero, and adding it to the
//         other term of its row (non-zero, or +0 from an exact cancellation)
//         returns that term unchanged, so it is skipped.
// A matrix with a row of two ZERO entries (whose sum's sign would need the
// signed-zero rules) or a part outside the fast domain takes the FP64 path,
// and so does a 2x2 block with an element outside the domain.  The right
// products x * conj(u) follow from the same classes.
enum : uint32_t { SK_FULL = 0, SK_REAL = 1, SK_IMAG = 2, SK_ZERO = 3 };
struct SoftU1 {
  softfp::Unpacked ux[4], uy[4], nuy[4];  // u.x, u.y, -u.y
  uint32_t kind[4];
  uint32_t ok;
};
__device__ __forceinline__ void soft_u1(const double2* u, SoftU1* f) {
  f->ok = 1;
  for (int j = 0; j < 4; ++j) {
    const bool zx = u[j].x == 0.0, zy = u[j].y == 0.0;
    f->ux[j] = softfp::unpack(u[j].x);
    f->uy[j] = softfp::unpack(u[j].y);
    f->nuy[j] = softfp::unpack(-u[j].y);
    f->kind[j] = zx && zy ? SK_ZERO : zy ? SK_REAL : zx ? SK_IMAG : SK_FULL;
    if (!zx && !f->ux[j].ok) f->ok = 0;
    if (!zy && !f->uy[j].ok) f->ok = 0;
  }
  if ((f->kind[0] == SK_ZERO && f->kind[1] == SK_ZERO) ||
      (f->kind[2] == SK_ZERO && f->kind[3] == SK_ZERO))
    f->ok = 0;
}
// u_j * x (cmul(u_j, x)) for an x whose parts are in the domain
__device__ __forceinline__ double2 soft_left(const SoftU1& f, int j, double2 u, double2 x,
                                             const SoftAmp& sx) {
  switch (f.kind[j]) {
    case SK_REAL: return make_double2(softfp::mul(f.ux[j], sx.x), softfp::mul(f.ux[j], sx.y));
    case SK_IMAG: return make_double2(-softfp::mul(f.uy[j], sx.y), softfp::mul(f.uy[j], sx.x));
    default: return scmul(u, f.uy[j], x, sx);  // FULL (ZERO is never used)
  }
}
// x * conj(u_j) (cmul(x, conj(u_j)))
__device__ __forceinline__ double2 soft_right(const SoftU1& f, int j, double2 u, double2 x,
                                              const SoftAmp& sx) {
  switch (f.kind[j]) {
    case SK_REAL: return make_double2(softfp::mul(sx.x, f.ux[j]), softfp::mul(sx.y, f.ux[j]));
    case SK_IMAG: return make_double2(softfp::mul(sx.y, f.uy[j]), -softfp::mul(sx.x, f.uy[j]));
    default:
      return make_double2(__fma_rn(x.x, u.x, -softfp::mul(sx.y, f.nuy[j])),
                          __fma_rn(x.x, -u.y, softfp::mul(sx.y, f.ux[j])));
  }
}
// one output of a row (j0, j1): the sum of its two terms, a ZERO term skipped
template <bool kLeft>
__device__ __forceinline__ double2 soft_row(const SoftU1& f, const double2* u, int j0, int j1,
                                            double2 a, const SoftAmp& sa, double2 b,
                                            const SoftAmp& sb) {
  if (f.kind[j0] == SK_ZERO)
    return kLeft ? soft_left(f, j1, u[j1], b, sb) : soft_right(f, j1, u[j1], b, sb);
  const double2 p = kLeft ? soft_left(f, j0, u[j0], a, sa) : soft_right(f, j0, u[j0], a, sa);
  if (f.kind[j1] == SK_ZERO) return p;
  return cadd(p, kLeft ? soft_left(f, j1, u[j1], b, sb) : soft_right(f, j1, u[j1], b, sb));
}
// left2 / right2 on the pair (a, b), soft when the matrix and both elements
// allow it
__device__ __forceinline__ void left2_any(const double2* u, const SoftU1& f, double2& a, double2& b) {
  const SoftAmp sa = sunpack(a), sb = sunpack(b);
  if (f.ok & sok(sa) & sok(sb)) {
    const double2 t = soft_row<true>(f, u, 0, 1, a, sa, b, sb);
    const double2 s2 = soft_row<true>(f, u, 2, 3, a, sa, b, sb);
    a = t;
    b = s2;
  } else {
    left2(u, a, b);
  }
}
__device__ __forceinline__ void right2_any(const double2* u, const SoftU1& f, double2& a,
                                           double2& b) {
  const SoftAmp sa = sunpack(a), sb = sunpack(b);
  if (f.ok & sok(sa) & sok(sb)) {
    const double2 t = soft_row<false>(f, u, 0, 1, a, sa, b, sb);
    const double2 s2 = soft_row<false>(f, u, 2, 3, a, sa, b, sb);
    a = t;
    b = s2;
  } else {
    right2(u, a, b);
  }
}

// rho -> U rho U^dagger on qubit t; with mask != 0 the left product applies
// to rows whose bits in mask are all set, the right product to such columns.
__global__ void __launch_bounds__(kDmThreads)
    k_dm_1q(double2* __restrict__ rho, int n, int t, U1 u, uint64_t mask, const uint8_t* pred) {
  if (dm_skip(pred)) return;
  __shared__ SoftU1 su;
  if (threadIdx.x == 0) soft_u1(u.m, &su);
  __syncthreads();
  const SoftU1& f = su;
  const uint64_t half = uint64_t(1) << (n - 1), blocks = half * half;
  const uint64_t dim = uint64_t(1) << n, bit = uint64_t(1) << t;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t b = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; b < blocks; b += stride) {
    const uint64_t r0 = insert0(b >> (n - 1), t), c0 = insert0(b & (half - 1), t);
    const uint64_t r1 = r0 | bit, c1 = c0 | bit;
    double2 e00 = rho[r0 * dim + c0], e01 = rho[r0 * dim + c1];
    double2 e10 = rho[r1 * dim + c0], e11 = rho[r1 * dim + c1];
    if ((r0 & mask) == mask) {
      left2_any(u.m, f, e00, e10);
      left2_any(u.m, f, e01, e11);
    }
    if ((c0 & mask) == mask) {
      right2_any(u.m, f, e00, e01);
      right2_any(u.m, f, e10, e11);
    }
    rho[r0 * dim + c0] = e00;
    rho[r0 * dim + c1] = e01;
    rho[r1 * dim + c0] = e10;
    rho[r1 * dim + c1] = e11;
  }
}

// rho -> U rho U^dagger for a dense 4x4 U on (a, b); group order
// [base, base|b, base|a, base|a|b] (index_group with targets [b, a]).
__global__ void __launch_bounds__(kDmThreads)
    k_dm_2q(double2* __restrict__ rho, int n, int a, int bq, U2 u, const uint8_t* pred) {
  if (dm_skip(pred)) return;
  const int lo = a < bq ? a : bq, hi = a < bq ? bq : a;
  const uint64_t q = uint64_t(1) << (n - 2), blocks = q * q;
  const uint64_t dim = uint64_t(1) << n, ba = uint64_t(1) << a, bb = uint64_t(1) << bq;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < blocks; g += stride) {
    const uint64_t rb = insert0(insert0(g >> (n - 2), lo), hi);
    const uint64_t cb = insert0(insert0(g & (q - 1), lo), hi);
    const uint64_t ri[4] = {rb, rb | bb, rb | ba, rb | ba | bb};
    const uint64_t ci[4] = {cb, cb | bb, cb | ba, cb | ba | bb};
    double2 e[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) e[r][c] = rho[ri[r] * dim + ci[c]];
#pragma unroll
    for (int c = 0; c < 4; ++c) {  // left_multiply, column by column
      double2 y[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double2 acc = cmul(u.m[4 * r], e[0][c]);
#pragma unroll
        for (int k = 1; k < 4; ++k) acc = cadd(acc, cmul(u.m[4 * r + k], e[k][c]));
        y[r] = acc;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) e[r][c] = y[r];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {  // right_multiply_adjoint, row by row
      double2 z[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double2 acc = cmul(e[r][0], cconj(u.m[4 * c]));
#pragma unroll
        for (int k = 1; k < 4; ++k) acc = cadd(acc, cmul(e[r][k], cconj(u.m[4 * c + k])));
        z[c] = acc;
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) rho[ri[r] * dim + ci[c]] = z[c];
    }
  }
}

// CNOT / CZ / SWAP: the dense products with 0, 1 and -1 entries are exact
// moves and negations, so rows and then columns are permuted (and signed)
// directly.  kind: 0 CNOT (swap 2<->3), 1 CZ (negate 3), 2 SWAP (swap 1<->2).
__global__ void __launch_bounds__(kDmThreads)
    k_dm_perm2(double2* __restrict__ rho, int n, int a, int bq, int kind, const uint8_t* pred) {
  if (dm_skip(pred)) return;
  const int lo = a < bq ? a : bq, hi = a < bq ? bq : a;
  const uint64_t q = uint64_t(1) << (n - 2), blocks = q * q;
  const uint64_t dim = uint64_t(1) << n, ba = uint64_t(1) << a, bb = uint64_t(1) << bq;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < blocks; g += stride) {
    const uint64_t rb = insert0(insert0(g >> (n - 2), lo), hi);
    const uint64_t cb = insert0(insert0(g & (q - 1), lo), hi);
    const uint64_t ri[4] = {rb, rb | bb, rb | ba, rb | ba | bb};
    const uint64_t ci[4] = {cb, cb | bb, cb | ba, cb | ba | bb};
    // the source of output index k under the permutation
    const int src[3][4] = {{0, 1, 3, 2}, {0, 1, 2, 3}, {0, 2, 1, 3}};
    double2 e[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) e[r][c] = rho[ri[r] * dim + ci[c]];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double2 v = e[src[kind][r]][src[kind][c]];
        if (kind == 1 && (r == 3) != (c == 3)) v = make_double2(-v.x, -v.y);
        rho[ri[r] * dim + ci[c]] = v;
      }
  }
}

// rho -> sum_k K_k rho K_k^dagger on qubit t, per 2x2 block.
__global__ void __launch_bounds__(kDmThreads)
    k_dm_channel(double2* __restrict__ rho, int n, int t, KrausSet ks, const uint8_t* pred) {
  if (dm_skip(pred)) return;
  __shared__ SoftU1 sk[EV_MAX_KRAUS];
  for (int k = threadIdx.x; k < ks.nops; k += blockDim.x) soft_u1(ks.k[k], &sk[k]);
  __syncthreads();
  const uint64_t half = uint64_t(1) << (n - 1), blocks = half * half;
  const uint64_t dim = uint64_t(1) << n, bit = uint64_t(1) << t;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t b = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; b < blocks; b += stride) {
    const uint64_t r0 = insert0(b >> (n - 1), t), c0 = insert0(b & (half - 1), t);
    const uint64_t r1 = r0 | bit, c1 = c0 | bit;
    const double2 x00 = rho[r0 * dim + c0], x01 = rho[r0 * dim + c1];
    const double2 x10 = rho[r1 * dim + c0], x11 = rho[r1 * dim + c1];
    double2 a00, a01, a10, a11;
    for (int k = 0; k < ks.nops; ++k) {
      double2 e00 = x00, e01 = x01, e10 = x10, e11 = x11;
      const SoftU1& f = sk[k];
      left2_any(ks.k[k], f, e00, e10);
      left2_any(ks.k[k], f, e01, e11);
      right2_any(ks.k[k], f, e00, e01);
      right2_any(ks.k[k], f, e10, e11);
      if (k == 0) {
        a00 = e00;
        a01 = e01;
        a10 = e10;
        a11 = e11;
      } else {
        a00 = cadd(a00, e00);
        a01 = cadd(a01, e01);
        a10 = cadd(a10, e10);
        a11 = cadd(a11, e11);
      }
    }
    rho[r0 * dim + c0] = a00;
    rho[r0 * dim + c1] = a01;
    rho[r1 * dim + c0] = a10;
    rho[r1 * dim + c1] = a11;
  }
}

// Fixed-order block partials of up to 8 sums; result[c] = sum over blocks.
__device__ __forceinline__ void dm_block_sum(double (&acc)[8], int ncol, double* partials) {
  __shared__ double sh[8][kDmThreads];
  for (int c = 0; c < ncol; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = kDmThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < ncol; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < ncol) partials[blockIdx.x * 8 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(kDmThreads)
    k_dm_finish(const double* __restrict__ partials, int nblocks, int ncol, double* result,
                const uint8_t* pred) {
  if (dm_skip(pred)) return;
  __shared__ double sh[8][kDmThreads];
  double acc[8] = {};
  for (int b = threadIdx.x; b < nblocks; b += kDmThreads)
    for (int c = 0; c < ncol; ++c) acc[c] += partials[b * 8 + c];
  for (int c = 0; c < ncol; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = kDmThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < ncol; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < ncol) result[threadIdx.x] = sh[threadIdx.x][0];
}

// Diagonal sums: [0] entries whose bit k is set, [1] the others
// (measure_probability, density_matrix.rs:165-176; trace, density.rs:117-120).
__global__ void __launch_bounds__(kDmThreads)
    k_dm_diag(const double2* __restrict__ rho, int n, int k, uint64_t chunk, double* partials,
              const uint8_t* pred) {
  if (dm_skip(pred)) return;
  const uint64_t dim = uint64_t(1) << n;
  const uint64_t lo = uint64_t(blockIdx.x) * chunk, hi = lo + chunk < dim ? lo + chunk : dim;
  double acc[8] = {};
  for (uint64_t j = lo + threadIdx.x; j < hi; j += kDmThreads) {
    const double d = rho[j * dim + j].x;
    if (k >= 0 && ((j >> k) & 1))
      acc[0] += d;
    else
      acc[1] += d;
  }
  dm_block_sum(acc, 2, partials);
}

// sum |rho_ij|^2 (purity, density.rs:126-136)
__global__ void __launch_bounds__(kDmThreads)
    k_dm_purity(const double2* __restrict__ rho, uint64_t count, uint64_t chunk, double* partials) {
  const uint64_t lo = uint64_t(blockIdx.x) * chunk, hi = lo + chunk < count ? lo + chunk : count;
  double acc[8] = {};
  for (uint64_t e = lo + threadIdx.x; e < hi; e += kDmThreads) {
    const double2 x = rho[e];
    acc[e & 1] = __fma_rn(x.x, x.x, acc[e & 1]);
    acc[e & 1] = __fma_rn(x.y, x.y, acc[e & 1]);
  }
  acc[0] += acc[1];
  dm_block_sum(acc, 1, partials);
}

// The reduced 2x2 matrix of qubit q (partial_trace_1q, density.rs:275-295):
// [r00, r01, r10, r11] as 8 doubles.
__global__ void __launch_bounds__(kDmThreads)
    k_dm_ptrace(const double2* __restrict__ rho, int n, int q, uint64_t chunk, double* partials) {
  const uint64_t dim = uint64_t(1) << n, count = dim / 2, bit = uint64_t(1) << q;
  const uint64_t lo = uint64_t(blockIdx.x) * chunk, hi = lo + chunk < count ? lo + chunk : count;
  double acc[8] = {};
  for (uint64_t o = lo + threadIdx.x; o < hi; o += kDmThreads) {
    const uint64_t i0 = insert0(o, q), i1 = i0 | bit;
    const double2 v[4] = {rho[i0 * dim + i0], rho[i0 * dim + i1], rho[i1 * dim + i0],
                          rho[i1 * dim + i1]};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      acc[2 * e] += v[e].x;
      acc[2 * e + 1] += v[e].y;
    }
  }
  dm_block_sum(acc, 8, partials);
}

// outcome = u < p1; trace after collapse = the kept diagonal sum; an extra
// uniform flips the reported bit with the readout probability
// (density_matrix.rs:136-158).  meas: [outcome, 1/trace, scale?].
__global__ void k_dm_decide(const double* __restrict__ result, const double* __restrict__ uni,
                            uint32_t* counter, double readout, double* meas, uint8_t* bit_out,
                            const uint8_t* pred) {
  if (dm_skip(pred)) return;
  const double p1 = result[0], p0 = result[1];
  const double u = uni[counter[0]++];
  const bool raw = u < p1;
  const double t = raw ? p1 : p0;
  meas[0] = raw ? 1.0 : 0.0;
  meas[1] = t > 0.0 ? __ddiv_rn(1.0, t) : 1.0;
  meas[2] = t > 0.0 ? 1.0 : 0.0;
  bool out = raw;
  if (readout > 0.0 && uni[counter[0]++] < readout) out = !raw;
  *bit_out = out ? 1 : 0;
}

// collapse (density_matrix.rs:178-193) then renormalize (density.rs:218-226)
__global__ void __launch_bounds__(kDmThreads)
    k_dm_collapse(double2* __restrict__ rho, int n, int k, const double* __restrict__ meas,
                  const uint8_t* pred) {
  if (dm_skip(pred)) return;
  const uint64_t count = uint64_t(1) << (2 * n);
  const bool raw = meas[0] != 0.0, scale = meas[2] != 0.0;
  const double inv = meas[1];
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < count; e += stride) {
    const bool im = ((e >> (n + k)) & 1) == uint64_t(raw), jm = ((e >> k) & 1) == uint64_t(raw);
    double2 x = make_double2(0.0, 0.0);
    if (im && jm) {
      x = rho[e];
      if (scale) x = make_double2(__dmul_rn(x.x, inv), __dmul_rn(x.y, inv));
    }
    rho[e] = x;
  }
}

__global__ void k_dm_pred_and(const uint8_t* classical, const uint64_t* bits, int nbits,
                              uint8_t* out) {
  uint8_t v = 1;
  for (int i = 0; i < nbits; ++i) v = v && classical[bits[i]];
  *out = v;
}

__global__ void k_dm_from_amps(double2* __restrict__ rho, const double2* __restrict__ a, int n) {
  const uint64_t dim = uint64_t(1) << n, count = dim * dim;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < count; e += stride)
    rho[e] = cmul(a[e >> n], cconj(a[e & (dim - 1)]));
}

__global__ void k_dm_one(double2* rho) { rho[0] = make_double2(1.0, 0.0); }

// ---- host ----------------------------------------------------------------------

unsigned dm_grid(const ev_dm* d, uint64_t work) {
  const uint64_t want = (work + kDmThreads - 1) / kDmThreads;
  const uint64_t cap = uint64_t(d->num_sms) * 8;
  return unsigned(want < 1 ? 1 : (want < cap ? want : cap));
}

void red_shape(const ev_dm* d, uint64_t count, int* nb, uint64_t* chunk) {
  uint64_t want = (count + 4095) / 4096;
  if (want < 1) want = 1;
  uint64_t cap = uint64_t(d->num_sms) * 4;
  if (cap > kDmRedBlocks) cap = kDmRedBlocks;
  *nb = int(want < cap ? want : cap);
  *chunk = (count + uint64_t(*nb) - 1) / uint64_t(*nb);
}

int dm_alloc(uint64_t n, ev_dm** out) {
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "null output");
  if (n > kDmMaxQubits)
    return fail(EV_ERR_OOM, "a %llu-qubit density matrix (4^n elements) cannot be stored",
                (unsigned long long)n);
  ev_dm* d = new ev_dm();
  d->n = n;
  cudaError_t e = cudaGetDevice(&d->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, d->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete d;
    return fail(EV_ERR_CUDA, "density matrix setup: %s", cudaGetErrorString(e));
  }
  const size_t bytes = size_t(d->elems()) * sizeof(double2);
  e = cudaMalloc(reinterpret_cast<void**>(&d->rho), bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaStreamDestroy(d->stream);
    delete d;
    return fail(EV_ERR_OOM, "cannot allocate %zu bytes for a %llu-qubit density matrix", bytes,
                (unsigned long long)n);
  }
  const size_t sb = kDmRedBlocks * 8 * sizeof(double) + 16 * sizeof(double) + 64 + 16;
  e = cudaMalloc(&d->scratch, sb);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d->rho);
    cudaStreamDestroy(d->stream);
    delete d;
    return fail(EV_ERR_OOM, "cannot allocate density-matrix scratch");
  }
  char* p = static_cast<char*>(d->scratch);
  d->partials = reinterpret_cast<double*>(p);
  p += kDmRedBlocks * 8 * sizeof(double);
  d->result = reinterpret_cast<double*>(p);
  p += 8 * sizeof(double);
  d->meas = reinterpret_cast<double*>(p);
  p += 8 * sizeof(double);
  d->pred = reinterpret_cast<uint8_t*>(p);
  p += 64;
  d->counter = reinterpret_cast<uint32_t*>(p);
  *out = d;
  return EV_OK;
}

int dm_zero(ev_dm* d) {
  EV_CUDA(cudaMemsetAsync(d->rho, 0, size_t(d->elems()) * sizeof(double2), d->stream));
  k_dm_one<<<1, 1, 0, d->stream>>>(d->rho);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int dm_fetch(const ev_dm* d, double* out, int count) {
  EV_CUDA(cudaMemcpyAsync(out, d->result, sizeof(double) * count, cudaMemcpyDeviceToHost, d->stream));
  EV_CUDA(cudaStreamSynchronize(d->stream));
  return EV_OK;
}

int dm_reduce_diag(const ev_dm* d, int k, const uint8_t* pred) {
  int nb = 0;
  uint64_t chunk = 0;
  red_shape(d, d->dim(), &nb, &chunk);
  k_dm_diag<<<nb, kDmThreads, 0, d->stream>>>(d->rho, int(d->n), k, chunk, d->partials, pred);
  k_dm_finish<<<1, kDmThreads, 0, d->stream>>>(d->partials, nb, 2, d->result, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int dm_unitary_1q(ev_dm* d, uint64_t t, const double m[8], uint64_t mask, const uint8_t* pred) {
  if (mask == 0 && classify1(m) == K1_IDENT) return EV_OK;  // U = I: exact no-op
  U1 u;
  for (int e = 0; e < 4; ++e) u.m[e] = make_double2(m[2 * e], m[2 * e + 1]);
  const uint64_t half = d->dim() / 2;
  k_dm_1q<<<dm_grid(d, half * half), kDmThreads, 0, d->stream>>>(d->rho, int(d->n), int(t), u,
                                                                   mask, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int dm_unitary_2q(ev_dm* d, uint64_t a, uint64_t b, const double m[32], const uint8_t* pred) {
  const uint64_t q = d->dim() / 4;
  const Kind2 kind = classify2(m);
  if (kind == K2_CNOT || kind == K2_CZ || kind == K2_SWAP) {
    const int pk = kind == K2_CNOT ? 0 : kind == K2_CZ ? 1 : 2;
    k_dm_perm2<<<dm_grid(d, q * q), kDmThreads, 0, d->stream>>>(d->rho, int(d->n), int(a), int(b),
                                                                 pk, pred);
  } else {
    U2 u;
    for (int e = 0; e < 16; ++e) u.m[e] = make_double2(m[2 * e], m[2 * e + 1]);
    k_dm_2q<<<dm_grid(d, q * q), kDmThreads, 0, d->stream>>>(d->rho, int(d->n), int(a), int(b), u,
                                                              pred);
  }
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int dm_channel(ev_dm* d, const ev_channel& ch, uint64_t t, const uint8_t* pred) {
  if (ch.nops == 0) return EV_OK;
  KrausSet ks;
  ks.nops = int(ch.nops);
  for (uint32_t k = 0; k < ch.nops; ++k)
    for (int e = 0; e < 4; ++e) ks.k[k][e] = make_double2(ch.k[k][2 * e], ch.k[k][2 * e + 1]);
  const uint64_t half = d->dim() / 2;
  k_dm_channel<<<dm_grid(d, half * half), kDmThreads, 0, d->stream>>>(d->rho, int(d->n), int(t),
                                                                       ks, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int dm_measure(ev_dm* d, uint64_t k, const double* uni, double readout, uint8_t* bit_out,
               const uint8_t* pred) {
  EV_TRY(dm_reduce_diag(d, int(k), pred));
  k_dm_decide<<<1, 1, 0, d->stream>>>(d->result, uni, d->counter, readout, d->meas, bit_out, pred);
  k_dm_collapse<<<dm_grid(d, d->elems()), kDmThreads, 0, d->stream>>>(d->rho, int(d->n), int(k),
                                                                       d->meas, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

struct DmBuffers {
  cudaStream_t stream = nullptr;
  uint8_t* classical = nullptr;
  double* uniforms = nullptr;
  uint64_t* ifbits = nullptr;
  ~DmBuffers() {
    if (classical) cudaFreeAsync(classical, stream);
    if (uniforms) cudaFreeAsync(uniforms, stream);
    if (ifbits) cudaFreeAsync(ifbits, stream);
  }
};

int dm_run_ops(ev_dm* d, const ev_circuit* c, const ev_noise_model* nz, uint64_t seed,
               uint8_t* classical_out) {
  static const ev_noise_model kIdeal = {};
  if (!nz) nz = &kIdeal;
  if (nz->after_1q.nops > EV_MAX_KRAUS || nz->after_2q.nops > EV_MAX_KRAUS)
    return fail(EV_ERR_INVALID_ARGUMENT, "at most %d Kraus operators per channel", EV_MAX_KRAUS);
  DmBuffers rb;
  rb.stream = d->stream;
  uint64_t nmeas = 0, nif = 0;
  for (uint64_t j = 0; j < c->nops; ++j) {
    if (c->ops[j].kind == EV_OP_MEASURE) ++nmeas;
    if (c->ops[j].kind == EV_OP_IF) ++nif;
  }
  const uint64_t per = nz->readout_error > 0.0 ? 2 : 1;
  std::vector<double> uni((nmeas ? nmeas : 1) * per, 0.0);
  Rng rng(seed);
  for (uint64_t j = 0; j < nmeas * per; ++j) uni[j] = rng.next_f64();
  const uint64_t ncl = c->num_classical ? c->num_classical : 1;
  EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&rb.classical), ncl, d->stream));
  EV_CUDA(cudaMemsetAsync(rb.classical, 0, ncl, d->stream));
  EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&rb.uniforms), uni.size() * sizeof(double), d->stream));
  EV_CUDA(cudaMemcpyAsync(rb.uniforms, uni.data(), uni.size() * sizeof(double),
                          cudaMemcpyHostToDevice, d->stream));
  EV_CUDA(cudaMemsetAsync(d->counter, 0, 2 * sizeof(uint32_t), d->stream));
  std::vector<uint64_t> host_ifbits(nif ? nif : 1);
  if (nif)
    EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&rb.ifbits), nif * sizeof(uint64_t), d->stream));
  uint64_t if_used = 0, pos = 0;
  while (pos < c->nops) {
    uint64_t chain[64];
    int nchain = 0;
    while (c->ops[pos].kind == EV_OP_IF) {
      if (nchain < 64) chain[nchain++] = c->ops[pos].q0;
      ++pos;
    }
    const uint8_t* pred = nullptr;
    if (nchain == 1) {
      pred = rb.classical + chain[0];
    } else if (nchain > 1) {
      std::memcpy(&host_ifbits[if_used], chain, nchain * sizeof(uint64_t));
      EV_CUDA(cudaMemcpyAsync(rb.ifbits + if_used, &host_ifbits[if_used], nchain * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, d->stream));
      k_dm_pred_and<<<1, 1, 0, d->stream>>>(rb.classical, rb.ifbits + if_used, nchain, d->pred);
      if_used += nchain;
      pred = d->pred;
    }
    const ev_op& op = c->ops[pos];
    switch (op.kind) {
      case EV_OP_APPLY1:  // density_matrix.rs:101-107
        EV_TRY(dm_unitary_1q(d, op.q0, op.m, 0, pred));
        EV_TRY(dm_channel(d, nz->after_1q, op.q0, pred));
        break;
      case EV_OP_APPLY2:  // density_matrix.rs:109-117
        EV_TRY(dm_unitary_2q(d, op.q0, op.q1, op.m, pred));
        EV_TRY(dm_channel(d, nz->after_2q, op.q0, pred));
        EV_TRY(dm_channel(d, nz->after_2q, op.q1, pred));
        break;
      case EV_OP_CONTROLLED: {  // density_matrix.rs:119-132
        uint64_t mask = 0;
        for (uint32_t j = 0; j < op.nctrl; ++j) mask |= uint64_t(1) << c->ctrl_pool[op.ctrl_off + j];
        EV_TRY(dm_unitary_1q(d, op.q0, op.m, mask, pred));
        EV_TRY(dm_channel(d, nz->after_1q, op.q0, pred));
        for (uint32_t j = 0; j < op.nctrl; ++j)
          EV_TRY(dm_channel(d, nz->after_1q, c->ctrl_pool[op.ctrl_off + j], pred));
        break;
      }
      case EV_OP_MEASURE:  // density_matrix.rs:134-158
        EV_TRY(dm_measure(d, op.q0, rb.uniforms, nz->readout_error, rb.classical + op.q1, pred));
        break;
    }
    ++pos;
  }
  if (c->num_classical)
    EV_CUDA(cudaMemcpyAsync(classical_out, rb.classical, c->num_classical, cudaMemcpyDeviceToHost,
                            d->stream));
  EV_CUDA(cudaStreamSynchronize(d->stream));
  return EV_OK;
}

}  // namespace
}  // namespace ev

using namespace ev;

extern "C" int ev_dm_create(uint64_t n, ev_dm** out) {
  clear_error();
  EV_TRY(dm_alloc(n, out));
  int rc = dm_zero(*out);
  if (rc == EV_OK && cudaStreamSynchronize((*out)->stream) != cudaSuccess)
    rc = fail(EV_ERR_CUDA, "density matrix init failed");
  if (rc != EV_OK) {
    ev_dm_destroy(*out);
    *out = nullptr;
  }
  return rc;
}

// Destroying never fails and leaves the last error message in place (a run
// that fails frees its own state before returning the error).
extern "C" int ev_dm_destroy(ev_dm* d) {
  if (!d) return EV_OK;
  cudaSetDevice(d->device);
  cudaStreamSynchronize(d->stream);
  cudaFree(d->rho);
  cudaFree(d->scratch);
  cudaStreamDestroy(d->stream);
  cudaGetLastError();
  delete d;
  return EV_OK;
}

extern "C" int ev_dm_num_qubits(const ev_dm* d, uint64_t* out) {
  clear_error();
  if (!d || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_num_qubits: null argument");
  *out = d->n;
  return EV_OK;
}

extern "C" int ev_dm_from_amplitudes(const double* amps, uint64_t len, ev_dm** out) {
  clear_error();
  if (!amps || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_from_amplitudes: null argument");
  if (len == 0 || (len & (len - 1))) {
    uint64_t next = 1;
    while (next < len) next <<= 1;
    return fail(EV_ERR_DIMENSION_MISMATCH, "amplitude buffer has length %llu, expected %llu",
                (unsigned long long)len, (unsigned long long)next);
  }
  uint64_t n = 0;
  while ((uint64_t(1) << n) < len) ++n;
  EV_TRY(dm_alloc(n, out));
  ev_dm* d = *out;
  double2* a = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&a), len * sizeof(double2), d->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(a, amps, len * sizeof(double2), cudaMemcpyHostToDevice, d->stream);
  if (e == cudaSuccess) {
    k_dm_from_amps<<<dm_grid(d, d->elems()), kDmThreads, 0, d->stream>>>(d->rho, a, int(n));
    e = cudaGetLastError();
  }
  if (a) cudaFreeAsync(a, d->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) {
    ev_dm_destroy(d);
    *out = nullptr;
    return fail(EV_ERR_CUDA, "ev_dm_from_amplitudes: %s", cudaGetErrorString(e));
  }
  return EV_OK;
}

extern "C" int ev_dm_download(const ev_dm* d, double* data, uint64_t len) {
  clear_error();
  if (!d || !data) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_download: null argument");
  if (len != d->elems())
    return fail(EV_ERR_DIMENSION_MISMATCH, "buffer of %llu elements, matrix has %llu",
                (unsigned long long)len, (unsigned long long)d->elems());
  EV_CUDA(cudaSetDevice(d->device));
  EV_CUDA(cudaMemcpyAsync(data, d->rho, len * sizeof(double2), cudaMemcpyDeviceToHost, d->stream));
  EV_CUDA(cudaStreamSynchronize(d->stream));
  return EV_OK;
}

extern "C" int ev_dm_get(const ev_dm* d, uint64_t i, uint64_t j, double out[2]) {
  clear_error();
  if (!d || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_get: null argument");
  if (i >= d->dim() || j >= d->dim())
    return fail(EV_ERR_INVALID_ARGUMENT, "element (%llu, %llu) outside a %llu x %llu matrix",
                (unsigned long long)i, (unsigned long long)j, (unsigned long long)d->dim(),
                (unsigned long long)d->dim());
  EV_CUDA(cudaSetDevice(d->device));
  EV_CUDA(cudaMemcpyAsync(out, d->rho + i * d->dim() + j, sizeof(double2), cudaMemcpyDeviceToHost,
                          d->stream));
  EV_CUDA(cudaStreamSynchronize(d->stream));
  return EV_OK;
}

extern "C" int ev_dm_trace(const ev_dm* d, double* out) {
  clear_error();
  if (!d || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_trace: null argument");
  EV_CUDA(cudaSetDevice(d->device));
  EV_TRY(dm_reduce_diag(d, -1, nullptr));
  double r[2];
  EV_TRY(dm_fetch(d, r, 2));
  *out = r[1];
  return EV_OK;
}

extern "C" int ev_dm_purity(const ev_dm* d, double* out) {
  clear_error();
  if (!d || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_purity: null argument");
  EV_CUDA(cudaSetDevice(d->device));
  int nb = 0;
  uint64_t chunk = 0;
  red_shape(d, d->elems(), &nb, &chunk);
  k_dm_purity<<<nb, kDmThreads, 0, d->stream>>>(d->rho, d->elems(), chunk, d->partials);
  k_dm_finish<<<1, kDmThreads, 0, d->stream>>>(d->partials, nb, 1, d->result, nullptr);
  EV_CUDA(cudaGetLastError());
  return dm_fetch(d, out, 1);
}

extern "C" int ev_dm_probability(const ev_dm* d, uint64_t basis, double* out) {
  clear_error();
  if (!d || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_probability: null argument");
  if (basis >= d->dim())
    return fail(EV_ERR_INVALID_ARGUMENT, "basis state %llu out of range for %llu-qubit register",
                (unsigned long long)basis, (unsigned long long)d->n);
  double v[2];
  EV_TRY(ev_dm_get(d, basis, basis, v));
  *out = v[0];
  return EV_OK;
}

extern "C" int ev_dm_partial_trace_1q(const ev_dm* d, uint64_t qubit, double out[8]) {
  clear_error();
  if (!d || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_partial_trace_1q: null argument");
  if (qubit >= d->n)
    return fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
                (unsigned long long)qubit, (unsigned long long)d->n);
  EV_CUDA(cudaSetDevice(d->device));
  int nb = 0;
  uint64_t chunk = 0;
  red_shape(d, d->dim() / 2, &nb, &chunk);
  k_dm_ptrace<<<nb, kDmThreads, 0, d->stream>>>(d->rho, int(d->n), int(qubit), chunk, d->partials);
  k_dm_finish<<<1, kDmThreads, 0, d->stream>>>(d->partials, nb, 8, d->result, nullptr);
  EV_CUDA(cudaGetLastError());
  return dm_fetch(d, out, 8);
}

// Tr(P rho) = Re(P00 r00 + P01 r10 + P10 r01 + P11 r11) from the reduced
// matrix of the qubit (density.rs:236-266 sums P_ij rho_ji over the same
// elements).
extern "C" int ev_dm_expectation_pauli(const ev_dm* d, uint64_t qubit, char observable,
                                       double* out) {
  clear_error();
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_expectation_pauli: null argument");
  if (observable != 'I' && observable != 'X' && observable != 'Y' && observable != 'Z')
    return fail(EV_ERR_INVALID_ARGUMENT, "unknown Pauli '%c'; expected I, X, Y, or Z", observable);
  double r[8];
  EV_TRY(ev_dm_partial_trace_1q(d, qubit, r));
  // r = [r00.re, r00.im, r01.re, r01.im, r10.re, r10.im, r11.re, r11.im]
  switch (observable) {
    case 'I': *out = r[0] + r[6]; break;
    case 'X': *out = r[4] + r[2]; break;
    case 'Y': *out = r[5] - r[3]; break;  // Re(-i r10 + i r01) = Im r10 - Im r01
    default: *out = r[0] - r[6]; break;
  }
  return EV_OK;
}

extern "C" int ev_validate(const ev_circuit* c);

extern "C" int ev_dm_run(const ev_circuit* c, const ev_noise_model* noise, uint64_t seed,
                         ev_dm** out, uint8_t* classical_out) {
  clear_error();
  EV_TRY(ev_validate(c));
  if (!out || (c->num_classical && !classical_out))
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_dm_run: null output");
  if (noise && !(noise->readout_error >= 0.0 && noise->readout_error <= 1.0))
    return fail(EV_ERR_INVALID_ARGUMENT, "readout error %g not in [0, 1]", noise->readout_error);
  EV_TRY(ev_dm_create(c->num_qubits, out));
  const int rc = dm_run_ops(*out, c, noise, seed, classical_out);
  if (rc != EV_OK) {
    ev_dm_destroy(*out);
    *out = nullptr;
  }
  return rc;
}
