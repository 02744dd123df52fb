// ev_fused.cu -- gate runs fused into dense k-qubit unitaries (complex64,
// and complex128 by digit slicing).
//
// The host groups consecutive gate records into blocks that act on at most
// k qubits (a record may move ahead of earlier records that share none of
// its qubits), multiplies each block's gates into one 2^k x 2^k unitary in
// f64, and applies each block to the state in one HBM pass.  A block on the
// qubit set F maps every group of 2^k amplitudes that agree outside F to
// U times that group: with rows = groups, the state is a (2^(n-k) x 2^k)
// complex matrix S and the pass computes S U^T.  In the real embedding each
// row is 2^(k+1) interleaved floats [re_0, im_0, re_1, ...] and
//     y = x W,  W[2f][2a] = Re U[a][f],  W[2f+1][2a] = -Im U[a][f],
//               W[2f][2a+1] = Im U[a][f], W[2f+1][2a+1] = Re U[a][f],
// a real GEMM with K = N = 2^(k+1).
//
// Four arithmetics:
//   EV_FUSED_TF32X3  complex64; tcgen05.mma kind::tf32, x = x_hi + x_lo and
//                    W = W_hi + W_lo split into TF32 parts, D accumulates
//                    x_hi W_hi + x_hi W_lo + x_lo W_hi in f32 (TMEM)
//   EV_FUSED_BF16X3  complex64; the same with BF16 parts (kind::f16)
//   EV_FUSED_FP32    complex64; CUDA cores, f32 complex multiply-add
//   EV_FUSED_OZAKI   complex128; k = 5, each f64 as seven 8-bit FP16 digits
//                    (kind::f16), exact digit-pair sums in TMEM, int64
//                    recombination (ev_ozaki.cuh, k_fused_oz below)
//   EV_FUSED_OZAKI6  the same with six digits (47 bits per value): a quarter
//                    fewer MMAs, one digit slice and one diagonal less
// The complex64 tensor-core kernel stages 128 rows per step: loads gather the rows
// (addresses contiguous for at least 128 amplitudes because the row qubits
// are the lowest qubits outside F), split into hi/lo and write the A operand
// in the 128-byte-swizzled K-major layout; one thread issues the MMAs and
// commits them to an mbarrier; the four warps read their 32 TMEM lanes back
// and scatter the rows to HBM.  Every mbarrier wait is bounded: on timeout
// the kernel records an error, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdio>
#include <cstdlib>

#include <algorithm>
#include <complex>
#include <cstring>
#include <vector>

#include "ev_bulk.cuh"
#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_ozaki.cuh"

namespace ev {

using cd = std::complex<double>;

constexpr int kRows = 128;  // rows per MMA step (UMMA M)

// Per-block index tables, built on the host.
struct FusedDesc {
  uint64_t ftab[64];   // global offset of local group index f (bits of F)
  uint64_t rtab[128];  // global offset of row r within a 128-row step (bits of R)
  uint64_t hitab[64];  // global offset of the T bits above the contiguous low run
  uint8_t rlo[128], flo[128];  // local index l: low 7 bits -> (r part, f part)
  uint8_t rhi[64], fhi[64];    // high bits of l -> (r part, f part)
  uint8_t comp_hi[64];         // qubits outside T, ascending (row-step index bits)
  uint16_t lrow[128];          // (r, f) -> local index: lrow[r] | lf[f]
  uint16_t lf[64];
  int32_t ncomp_hi;
  int32_t k;
  int32_t lowbits;  // T holds qubits 0..lowbits-1
  int32_t pad;
  uint64_t nsteps;  // 2^(n-k-7) row steps
};

// ---- host: fusion ----------------------------------------------------------

struct Block {
  std::vector<int> F;           // sorted qubits, |F| == k after padding
  std::vector<uint64_t> ops;    // op indices in application order
  std::vector<cd> U;            // 2^k x 2^k row-major
};

static void op_qubits(const ev_circuit* c, const ev_op& op, std::vector<int>* q) {
  q->clear();
  if (op.kind == EV_OP_APPLY2) {
    q->push_back(int(op.q0));
    q->push_back(int(op.q1));
    return;
  }
  q->push_back(int(op.q0));
  if (op.kind == EV_OP_CONTROLLED)
    for (uint32_t j = 0; j < op.nctrl; ++j) {
      const int cq = int(c->ctrl_pool[op.ctrl_off + j]);
      if (std::find(q->begin(), q->end(), cq) == q->end()) q->push_back(cq);
    }
}

// Left-multiplies U (d x d, local bit i <-> F[i]) by one gate record.
static void apply_to_unitary(const ev_circuit* c, const ev_op& op, const std::vector<int>& F,
                             std::vector<cd>* U) {
  const int d = int(1u << F.size());
  auto loc = [&](int q) { return int(std::find(F.begin(), F.end(), q) - F.begin()); };
  auto m = [&](int i) { return cd(op.m[2 * i], op.m[2 * i + 1]); };
  if (op.kind == EV_OP_APPLY2) {
    const int ba = 1 << loc(int(op.q0)), bb = 1 << loc(int(op.q1));
    for (int col = 0; col < d; ++col)
      for (int base = 0; base < d; ++base) {
        if (base & (ba | bb)) continue;
        const int idx[4] = {base, base | bb, base | ba, base | ba | bb};
        cd in[4], out[4];
        for (int r = 0; r < 4; ++r) in[r] = (*U)[idx[r] * d + col];
        for (int r = 0; r < 4; ++r) {
          out[r] = 0;
          for (int cc = 0; cc < 4; ++cc) out[r] += m(4 * r + cc) * in[cc];
        }
        for (int r = 0; r < 4; ++r) (*U)[idx[r] * d + col] = out[r];
      }
    return;
  }
  const int tb = 1 << loc(int(op.q0));
  int cmask = 0;
  if (op.kind == EV_OP_CONTROLLED)
    for (uint32_t j = 0; j < op.nctrl; ++j) cmask |= 1 << loc(int(c->ctrl_pool[op.ctrl_off + j]));
  for (int col = 0; col < d; ++col)
    for (int i0 = 0; i0 < d; ++i0) {
      if ((i0 & tb) || (i0 & cmask) != cmask) continue;
      const int i1 = i0 | tb;
      const cd a0 = (*U)[i0 * d + col], a1 = (*U)[i1 * d + col];
      (*U)[i0 * d + col] = m(0) * a0 + m(1) * a1;
      (*U)[i1 * d + col] = m(2) * a0 + m(3) * a1;
    }
}

// Greedy fusion: each block starts at the first pending record and takes
// every later pending record whose qubits fit (|F| <= k) and which does not
// touch a qubit of a record skipped before it.
std::vector<Block> fuse_ops(const ev_circuit* c, uint64_t first, uint64_t last, int n, int k) {
  std::vector<Block> blocks;
  std::vector<uint64_t> pending;
  for (uint64_t j = first; j < last; ++j) pending.push_back(j);
  std::vector<int> q;
  const size_t window = 4096;
  while (!pending.empty()) {
    Block b;
    uint64_t fset = 0, blocked = 0;
    std::vector<uint64_t> rest;
    size_t scanned = 0;
    for (size_t i = 0; i < pending.size(); ++i) {
      const ev_op& op = c->ops[pending[i]];
      op_qubits(c, op, &q);
      uint64_t qm = 0;
      for (int x : q) qm |= uint64_t(1) << x;
      const bool fits = __builtin_popcountll(fset | qm) <= k && (qm & blocked) == 0;
      if (fits && scanned < window) {
        fset |= qm;
        b.ops.push_back(pending[i]);
      } else {
        blocked |= qm;
        rest.push_back(pending[i]);
      }
      ++scanned;
    }
    // pad F to exactly k qubits with the lowest unused ones
    for (int x = 0; x < n && __builtin_popcountll(fset) < k; ++x) fset |= uint64_t(1) << x;
    for (int x = 0; x < n; ++x)
      if ((fset >> x) & 1) b.F.push_back(x);
    const int d = 1 << b.F.size();
    b.U.assign(size_t(d) * d, cd(0, 0));
    for (int i = 0; i < d; ++i) b.U[size_t(i) * d + i] = 1;
    for (uint64_t j : b.ops) apply_to_unitary(c, c->ops[j], b.F, &b.U);
    blocks.push_back(std::move(b));
    pending.swap(rest);
  }
  return blocks;
}

static uint64_t pdep(uint64_t x, const std::vector<int>& pos) {
  uint64_t r = 0;
  for (size_t i = 0; i < pos.size(); ++i)
    if ((x >> i) & 1) r |= uint64_t(1) << pos[i];
  return r;
}

static void build_desc(const Block& b, int n, FusedDesc* d) {
  std::memset(d, 0, sizeof(*d));
  const int k = int(b.F.size());
  uint64_t fmask = 0;
  for (int x : b.F) fmask |= uint64_t(1) << x;
  std::vector<int> R, comp;
  for (int x = 0; x < n; ++x)
    if (!((fmask >> x) & 1)) (R.size() < 7 ? R : comp).push_back(x);
  std::vector<int> T;  // sorted union of F and R
  for (int x = 0; x < n; ++x)
    if (((fmask >> x) & 1) || std::find(R.begin(), R.end(), x) != R.end()) T.push_back(x);
  int low = 0;
  while (low < int(T.size()) && T[low] == low) ++low;
  d->k = k;
  d->lowbits = low;
  for (int f = 0; f < (1 << k); ++f) d->ftab[f] = pdep(uint64_t(f), b.F);
  for (int r = 0; r < kRows; ++r) d->rtab[r] = pdep(uint64_t(r), R);
  std::vector<int> Thi(T.begin() + low, T.end());
  for (int h = 0; h < (1 << Thi.size()) && h < 64; ++h) d->hitab[h] = pdep(uint64_t(h), Thi);
  // local index l (bit i <-> T[i]) to (r, f)
  auto split = [&](uint64_t l, int* r, int* f) {
    *r = 0;
    *f = 0;
    int ri = 0, fi = 0;
    for (size_t i = 0; i < T.size(); ++i) {
      const bool inF = (fmask >> T[i]) & 1;
      if ((l >> i) & 1) {
        if (inF)
          *f |= 1 << fi;
        else
          *r |= 1 << ri;
      }
      inF ? ++fi : ++ri;
    }
  };
  for (int j = 0; j < 128; ++j) {
    int r, f;
    split(uint64_t(j), &r, &f);
    d->rlo[j] = uint8_t(r);
    d->flo[j] = uint8_t(f);
  }
  for (int j = 0; j < (1 << (int(T.size()) - 7)) && j < 64; ++j) {
    int r, f;
    split(uint64_t(j) << 7, &r, &f);
    d->rhi[j] = uint8_t(r);
    d->fhi[j] = uint8_t(f);
  }
  // inverse maps: local bit positions of R and F inside T
  {
    std::vector<int> rpos, fpos;
    for (size_t i = 0; i < T.size(); ++i) ((fmask >> T[i]) & 1 ? fpos : rpos).push_back(int(i));
    for (int r = 0; r < kRows; ++r) d->lrow[r] = uint16_t(pdep(uint64_t(r), rpos));
    for (int f = 0; f < (1 << k); ++f) d->lf[f] = uint16_t(pdep(uint64_t(f), fpos));
  }
  d->ncomp_hi = int(comp.size());
  for (size_t i = 0; i < comp.size(); ++i) d->comp_hi[i] = uint8_t(comp[i]);
  d->nsteps = uint64_t(1) << comp.size();
}

// ---- device: shared helpers --------------------------------------------------

__device__ __forceinline__ uint64_t step_base(const FusedDesc& d, uint64_t step) {
  uint64_t base = 0;
  for (int b = 0; b < d.ncomp_hi; ++b)
    if ((step >> b) & 1) base |= uint64_t(1) << d.comp_hi[b];
  return base;
}

// global address of local index l of a step
__device__ __forceinline__ uint64_t local_addr(const FusedDesc& d, uint64_t base, uint32_t l) {
  return base | (l & ((1u << d.lowbits) - 1)) | d.hitab[l >> d.lowbits];
}

// ---- CUDA-core f32 kernel ---------------------------------------------------

template <int KB>
__global__ void __launch_bounds__(256)
    k_fused_fp32(float2* __restrict__ s, const FusedDesc* __restrict__ gd,
                 const float2* __restrict__ U) {
  constexpr int D = 1 << KB;
  extern __shared__ __align__(16) unsigned char fp_raw[];
  float2* tile = reinterpret_cast<float2*>(fp_raw);  // kRows x D
  float2* um = tile + kRows * D;                     // D x D
  __shared__ FusedDesc d;
  for (int i = threadIdx.x; i < int(sizeof(FusedDesc) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&d)[i] = reinterpret_cast<const uint64_t*>(gd)[i];
  for (int i = threadIdx.x; i < D * D; i += blockDim.x) um[i] = U[i];
  __syncthreads();
  for (uint64_t step = blockIdx.x; step < d.nsteps; step += gridDim.x) {
    const uint64_t base = step_base(d, step);
    for (uint32_t l = threadIdx.x; l < uint32_t(kRows * D); l += blockDim.x) {
      const int r = d.rlo[l & 127] | d.rhi[l >> 7];
      const int f = d.flo[l & 127] | d.fhi[l >> 7];
      tile[r * D + f] = s[local_addr(d, base, l)];
    }
    __syncthreads();
    for (uint32_t o = threadIdx.x; o < uint32_t(kRows * D); o += blockDim.x) {
      const int r = o % kRows, a = o / kRows;  // consecutive threads: consecutive rows
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll 8
      for (int f = 0; f < D; ++f) {
        const float2 u = um[a * D + f], x = tile[r * D + f];
        acc.x = __fmaf_rn(u.x, x.x, __fmaf_rn(-u.y, x.y, acc.x));
        acc.y = __fmaf_rn(u.x, x.y, __fmaf_rn(u.y, x.x, acc.y));
      }
      s[base | d.rtab[r] | d.ftab[a]] = acc;
    }
    __syncthreads();
  }
}

// ---- tcgen05 kernel ------------------------------------------------------------

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  uint64_t desc = 0;
  desc |= uint64_t((addr & 0x3FFFF) >> 4);        // start address
  desc |= uint64_t(1) << 16;                      // leading byte offset (unused for SW128 K-major)
  desc |= uint64_t(1024 >> 4) << 32;              // stride byte offset
  desc |= uint64_t(1) << 46;                      // descriptor version
  desc |= uint64_t(2) << 61;                      // 128-byte swizzle
  return desc;
}

// Byte offset of element (row, kk) in a K-major SW128 operand of `rows` rows
// whose element size is esz bytes.
__device__ __forceinline__ uint32_t sw128_off(int row, int kk, int rows, int esz) {
  const int per_row = 128 / esz;  // elements per 128-byte swizzle row
  const int kb = kk / per_row, kin = kk % per_row;
  const int byte = kin * esz;
  return uint32_t(kb * rows * 128 + (row >> 3) * 1024 + (row & 7) * 128 +
                  ((((byte >> 4) ^ (row & 7))) << 4) + (byte & 15));
}

template <int VAR>
__device__ __forceinline__ void mma_issue(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t acc) {
  if constexpr (VAR == EV_FUSED_TF32X3) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  }
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t v[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

template <int VAR>
struct Elem;
template <>
struct Elem<EV_FUSED_TF32X3> {
  static constexpr int size = 4;
  static constexpr int kstep = 8;  // UMMA K per instruction
  static constexpr uint32_t fmt = 2;  // TF32
};
template <>
struct Elem<EV_FUSED_BF16X3> {
  static constexpr int size = 2;
  static constexpr int kstep = 16;
  static constexpr uint32_t fmt = 1;  // BF16
};

// Splits x into hi + lo parts of the operand type and stores both.
template <int VAR>
__device__ __forceinline__ void put_split(unsigned char* hi, unsigned char* lo, uint32_t off,
                                          float re, float im) {
  if constexpr (VAR == EV_FUSED_TF32X3) {
    const float hr = __uint_as_float(__float_as_uint(re) & 0xFFFFE000u);
    const float hm = __uint_as_float(__float_as_uint(im) & 0xFFFFE000u);
    *reinterpret_cast<float2*>(hi + off) = make_float2(hr, hm);
    *reinterpret_cast<float2*>(lo + off) = make_float2(re - hr, im - hm);
  } else {
    const __nv_bfloat16 hr = __float2bfloat16_rn(re), hm = __float2bfloat16_rn(im);
    const __nv_bfloat16 lr = __float2bfloat16_rn(re - __bfloat162float(hr));
    const __nv_bfloat16 lm = __float2bfloat16_rn(im - __bfloat162float(hm));
    __nv_bfloat162 h2, l2;
    h2.x = hr;
    h2.y = hm;
    l2.x = lr;
    l2.y = lm;
    *reinterpret_cast<__nv_bfloat162*>(hi + off) = h2;
    *reinterpret_cast<__nv_bfloat162*>(lo + off) = l2;
  }
}

template <int KB, int VAR>
struct TcShape {
  static constexpr int D = 1 << KB;
  static constexpr int K = 2 * D;  // = N
  static constexpr int ESZ = Elem<VAR>::size;
  static constexpr int A_BYTES = kRows * K * ESZ;
  static constexpr int B_BYTES = K * K * ESZ;
  static constexpr int SMEM = 2 * A_BYTES + 2 * B_BYTES + 1024 /* align */ + 64;
  static constexpr int TMEM_COLS = K < 32 ? 32 : K;
};

constexpr uint32_t kWaitLimit = 1u << 24;

constexpr int kTcThreads = 256;  // 8 warps: warps w and w+4 share TMEM lane quarter w

template <int KB, int VAR>
__global__ void __launch_bounds__(kTcThreads)
    k_fused_tc(float2* __restrict__ s, const FusedDesc* __restrict__ gd,
               const unsigned char* __restrict__ bmat, int* __restrict__ err) {
  using Sh = TcShape<KB, VAR>;
  constexpr int D = Sh::D, K = Sh::K, ESZ = Sh::ESZ;
  extern __shared__ unsigned char smem_raw[];
  __shared__ FusedDesc d;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_hi = sm;
  unsigned char* a_lo = sm + Sh::A_BYTES;
  unsigned char* b_hi = sm + 2 * Sh::A_BYTES;
  unsigned char* b_lo = b_hi + Sh::B_BYTES;
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int i = tid; i < int(sizeof(FusedDesc) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&d)[i] = reinterpret_cast<const uint64_t*>(gd)[i];
  // B operands (hi then lo, each [N][K] row-major in the element type) into
  // the swizzled layout
  for (int e = tid; e < K * K; e += blockDim.x) {
    const int nrow = e / K, kk = e % K;
    const uint32_t off = sw128_off(nrow, kk, K, ESZ);
    if constexpr (ESZ == 4) {
      *reinterpret_cast<uint32_t*>(b_hi + off) = reinterpret_cast<const uint32_t*>(bmat)[e];
      *reinterpret_cast<uint32_t*>(b_lo + off) = reinterpret_cast<const uint32_t*>(bmat)[K * K + e];
    } else {
      *reinterpret_cast<uint16_t*>(b_hi + off) = reinterpret_cast<const uint16_t*>(bmat)[e];
      *reinterpret_cast<uint16_t*>(b_lo + off) = reinterpret_cast<const uint16_t*>(bmat)[K * K + e];
    }
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_slot)),
                 "r"(uint32_t(Sh::TMEM_COLS)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  // instruction descriptor: f32 accumulate, A/B format, K-major, N, M
  const uint32_t idesc = (1u << 4) | (Elem<VAR>::fmt << 7) | (Elem<VAR>::fmt << 10) |
                         (uint32_t(K >> 3) << 17) | (uint32_t(kRows >> 4) << 24);
  uint32_t phase = 0;
  bool ok = true;
  // Thread t owns row r = t mod 128 (its TMEM lane) and the groups of four
  // consecutive complex values g = t/128, t/128 + 2, ...  A group is 8
  // reals: one 16-byte swizzle chunk in BF16, two in TF32, so the A operand
  // is written with whole-chunk stores; the 8 rows of a swizzle atom land in
  // 8 different bank groups.  A warp holds 32 consecutive rows, i.e. the
  // lowest qubits outside F, so its loads of one f are contiguous in HBM.
  const int quarter = warp & 3, half = warp >> 2;
  const int row = quarter * 32 + (tid & 31);
  constexpr int G = D / 4;                         // groups per row
  constexpr int GPT = G / (kTcThreads / kRows);    // groups per thread
  const uint32_t rsw = uint32_t((row >> 3) * 1024 + (row & 7) * 128);
  const uint32_t rx = uint32_t(row & 7);
  const uint64_t roff = d.rtab[row];
  // L2 prefetch of the rows two steps ahead: contiguous runs of 2^lowbits
  // amplitudes, one bulk prefetch per run from warp 1
  const int nruns = 1 << (d.k + 7 - d.lowbits);
  const uint32_t run_bytes = 8u << d.lowbits;
  for (uint64_t step = blockIdx.x; step < d.nsteps && ok; step += gridDim.x) {
    if (warp == 1 && (tid & 31) < nruns && step + 2 * uint64_t(gridDim.x) < d.nsteps) {
      const uint64_t b2 = step_base(d, step + 2 * uint64_t(gridDim.x));
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(s + (b2 | d.hitab[tid & 31])),
                   "r"(run_bytes)
                   : "memory");
    }
    const uint64_t rbase = step_base(d, step) | roff;
    float2 x[GPT][4];
#pragma unroll
    for (int gi = 0; gi < GPT; ++gi) {
      const int g = half + 2 * gi;
#pragma unroll
      for (int i = 0; i < 4; ++i) x[gi][i] = __ldcs(s + (rbase | d.ftab[4 * g + i]));
    }
#pragma unroll
    for (int gi = 0; gi < GPT; ++gi) {
      const int g = half + 2 * gi;
      if constexpr (VAR == EV_FUSED_TF32X3) {
        // reals 8g..8g+7: K-block g/4, chunks 2(g%4) and 2(g%4)+1
        const uint32_t kb = uint32_t(g / 4) * kRows * 128 + rsw;
        const uint32_t c0 = uint32_t(2 * (g % 4));
        float hi[8], lo[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float re = x[gi][i].x, im = x[gi][i].y;
          hi[2 * i] = __uint_as_float(__float_as_uint(re) & 0xFFFFE000u);
          hi[2 * i + 1] = __uint_as_float(__float_as_uint(im) & 0xFFFFE000u);
          lo[2 * i] = re - hi[2 * i];
          lo[2 * i + 1] = im - hi[2 * i + 1];
        }
        const uint32_t o0 = kb + (((c0) ^ rx) << 4), o1 = kb + (((c0 + 1) ^ rx) << 4);
        *reinterpret_cast<float4*>(a_hi + o0) = make_float4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<float4*>(a_hi + o1) = make_float4(hi[4], hi[5], hi[6], hi[7]);
        *reinterpret_cast<float4*>(a_lo + o0) = make_float4(lo[0], lo[1], lo[2], lo[3]);
        *reinterpret_cast<float4*>(a_lo + o1) = make_float4(lo[4], lo[5], lo[6], lo[7]);
      } else {
        // reals 8g..8g+7: K-block g/8, chunk g%8
        const uint32_t o = uint32_t(g / 8) * kRows * 128 + rsw + ((uint32_t(g % 8) ^ rx) << 4);
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float re = x[gi][i].x, im = x[gi][i].y;
          const __nv_bfloat16 hr = __float2bfloat16_rn(re), hm = __float2bfloat16_rn(im);
          const __nv_bfloat16 lr = __float2bfloat16_rn(re - __bfloat162float(hr));
          const __nv_bfloat16 lm = __float2bfloat16_rn(im - __bfloat162float(hm));
          hw[i] = uint32_t(__bfloat16_as_ushort(hr)) | (uint32_t(__bfloat16_as_ushort(hm)) << 16);
          lw[i] = uint32_t(__bfloat16_as_ushort(lr)) | (uint32_t(__bfloat16_as_ushort(lm)) << 16);
        }
        *reinterpret_cast<uint4*>(a_hi + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(a_lo + o) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = smem_addr(a_hi), al = smem_addr(a_lo);
      const uint32_t bh = smem_addr(b_hi), bl = smem_addr(b_lo);
      constexpr int per_row = 128 / ESZ;
      uint32_t acc = 0;
#pragma unroll
      for (int kk = 0; kk < K; kk += Elem<VAR>::kstep) {
        const int kb = kk / per_row;
        const uint32_t kin = uint32_t((kk % per_row) * ESZ);
        const uint32_t ao = uint32_t(kb * kRows * 128) + kin;
        const uint32_t bo = uint32_t(kb * K * 128) + kin;
        mma_issue<VAR>(tmem, sw128_desc(ah + ao), sw128_desc(bh + bo), idesc, acc);
        acc = 1;
        mma_issue<VAR>(tmem, sw128_desc(ah + ao), sw128_desc(bl + bo), idesc, 1);
        mma_issue<VAR>(tmem, sw128_desc(al + ao), sw128_desc(bh + bo), idesc, 1);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr(&bar))
          : "memory");
    }
    if (!mbar_wait(&bar, phase, kWaitLimit)) {
      ok = false;
      atomicExch(err, 1);
      break;
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t lane_base = tmem + (uint32_t(quarter * 32) << 16);
    const bool pair_store = d.ftab[1] == 1;  // f bit 0 is qubit 0: outputs a, a+1 adjacent
#pragma unroll
    for (int c0 = half * (K / 2); c0 < (half + 1) * (K / 2); c0 += 16) {
      uint32_t w[16];
      tmem_ld16(lane_base + uint32_t(c0), w);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (pair_store) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          const int a = c0 / 2 + j;
          __stcs(reinterpret_cast<float4*>(s + (rbase | d.ftab[a])),
                 make_float4(__uint_as_float(w[2 * j]), __uint_as_float(w[2 * j + 1]),
                             __uint_as_float(w[2 * j + 2]), __uint_as_float(w[2 * j + 3])));
        }
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int a = c0 / 2 + j;
          __stcs(s + (rbase | d.ftab[a]),
                 make_float2(__uint_as_float(w[2 * j]), __uint_as_float(w[2 * j + 1])));
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(uint32_t(Sh::TMEM_COLS)));
  }
}

// ---- tcgen05 kernel with TMA-staged streaming -------------------------------
//
// The same pass as k_fused_tc, with HBM traffic moved to the bulk-copy (TMA)
// engine.  A step's 128 x 2^k amplitudes are contiguous runs of 2^lowbits
// amplitudes (>= 1 KiB): thread 0 issues one cp.async.bulk per run into a
// shared-memory stage, STAGES steps ahead, completing on the stage's
// mbarrier (expect_tx).  The warps convert the stage into the split A
// operand, thread 0 issues the MMAs, the warps write the results back into
// the same stage (the input is already in A), and thread 0 streams the stage
// to HBM with bulk stores, waits until they have read it, and refills it
// with a later step.  On a wait that gives up, the kernel records the error,
// drains its outstanding copies (bounded), frees TMEM and returns.

template <int KB, int VAR, int STAGES>
struct TmaShape {
  using Sh = TcShape<KB, VAR>;
  static constexpr int RAW = kRows * Sh::D * 8;  // one step of complex64 amplitudes
  static constexpr int SMEM = 2 * Sh::A_BYTES + 2 * Sh::B_BYTES + STAGES * RAW + 1024;
};

constexpr int kTmaThreads = kTcThreads + 32;  // 8 compute warps + 1 producer warp

__device__ __forceinline__ void compute_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kTcThreads) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

template <int KB, int VAR, int STAGES>
__global__ void __launch_bounds__(kTmaThreads)
    k_fused_tma(float2* __restrict__ s, const FusedDesc* __restrict__ gd,
                const unsigned char* __restrict__ bmat, int* __restrict__ err) {
  using Sh = TcShape<KB, VAR>;
  using Tm = TmaShape<KB, VAR, STAGES>;
  constexpr int D = Sh::D, K = Sh::K, ESZ = Sh::ESZ;
  extern __shared__ unsigned char smem_raw[];
  __shared__ FusedDesc d;
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t mma_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int s_ok;
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_hi = sm;
  unsigned char* a_lo = sm + Sh::A_BYTES;
  unsigned char* b_hi = sm + 2 * Sh::A_BYTES;
  unsigned char* b_lo = b_hi + Sh::B_BYTES;
  unsigned char* raw0 = b_lo + Sh::B_BYTES;
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int i = tid; i < int(sizeof(FusedDesc) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&d)[i] = reinterpret_cast<const uint64_t*>(gd)[i];
  for (int e = tid; e < K * K; e += blockDim.x) {
    const int nrow = e / K, kk = e % K;
    const uint32_t off = sw128_off(nrow, kk, K, ESZ);
    if constexpr (ESZ == 4) {
      *reinterpret_cast<uint32_t*>(b_hi + off) = reinterpret_cast<const uint32_t*>(bmat)[e];
      *reinterpret_cast<uint32_t*>(b_lo + off) = reinterpret_cast<const uint32_t*>(bmat)[K * K + e];
    } else {
      *reinterpret_cast<uint16_t*>(b_hi + off) = reinterpret_cast<const uint16_t*>(bmat)[e];
      *reinterpret_cast<uint16_t*>(b_lo + off) = reinterpret_cast<const uint16_t*>(bmat)[K * K + e];
    }
  }
  if (tid == 0) {
    for (int st = 0; st < STAGES; ++st) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full_bar[st])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty_bar[st])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mma_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_ok = 1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_slot)),
                 "r"(uint32_t(Sh::TMEM_COLS)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const int nruns = (kRows * D) >> d.lowbits;
  const uint32_t run_bytes = 8u << d.lowbits;
  const uint64_t stride = gridDim.x;

  if (warp == kTcThreads / 32) {
    // ---- producer warp: all HBM traffic through the bulk-copy engine ----
    if ((tid & 31) == 0) {
      uint32_t pending = 0, ephase = 0;
      uint32_t armed[STAGES] = {};  // loads issued into each stage so far
      auto load = [&](uint64_t step, int st) {
        const uint64_t base = step_base(d, step);
        unsigned char* dst = raw0 + size_t(st) * Tm::RAW;
        mbar_expect_tx(&full_bar[st], uint32_t(Tm::RAW));
        for (int j = 0; j < nruns; ++j)
          bulk_g2s(dst + size_t(j) * run_bytes, s + (base | d.hitab[j]), run_bytes, &full_bar[st]);
        pending |= 1u << st;
        armed[st] += 1;
      };
      for (int st = 0; st < STAGES; ++st) {
        const uint64_t step = blockIdx.x + uint64_t(st) * stride;
        if (step < d.nsteps) load(step, st);
      }
      uint64_t i = 0;
      for (uint64_t step = blockIdx.x; step < d.nsteps; step += stride, ++i) {
        const int st = int(i % STAGES);
        // the compute warps have consumed the stage and written results into it
        if (!mbar_wait(&empty_bar[st], (ephase >> st) & 1u, kWaitLimit) || !s_ok) {
          atomicExch(err, 1);
          s_ok = 0;
          break;
        }
        ephase ^= 1u << st;
        pending &= ~(1u << st);
        const uint64_t base = step_base(d, step);
        for (int j = 0; j < nruns; ++j)
          bulk_s2g(s + (base | d.hitab[j]), raw0 + size_t(st) * Tm::RAW + size_t(j) * run_bytes,
                   run_bytes);
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        const uint64_t next = step + uint64_t(STAGES) * stride;
        if (next < d.nsteps) {
          asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          load(next, st);
        }
      }
      // drain: a load still in flight completes phase (armed - 1) of its
      // barrier (bounded wait); then every bulk store
      for (int st = 0; st < STAGES; ++st)
        if (pending & (1u << st)) mbar_wait(&full_bar[st], (armed[st] - 1) & 1u, kWaitLimit);
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
  } else {
    // ---- compute warps ----
    const uint32_t idesc = (1u << 4) | (Elem<VAR>::fmt << 7) | (Elem<VAR>::fmt << 10) |
                           (uint32_t(K >> 3) << 17) | (uint32_t(kRows >> 4) << 24);
    const int quarter = warp & 3, half = warp >> 2;
    const int row = quarter * 32 + (tid & 31);
    constexpr int G = D / 4;
    constexpr int GPT = G / (kTcThreads / kRows);
    const uint32_t rsw = uint32_t((row >> 3) * 1024 + (row & 7) * 128);
    const uint32_t rx = uint32_t(row & 7);
    const uint32_t lrow = d.lrow[row];
    uint32_t fphase = 0, mphase = 0;
    uint64_t i = 0;
    for (uint64_t step = blockIdx.x; step < d.nsteps; step += stride, ++i) {
      const int st = int(i % STAGES);
      float2* raw = reinterpret_cast<float2*>(raw0 + size_t(st) * Tm::RAW);
      if (!mbar_wait(&full_bar[st], (fphase >> st) & 1u, kWaitLimit)) {
        atomicExch(err, 1);
        s_ok = 0;
      }
      compute_sync();
      if (!s_ok) break;
      fphase ^= 1u << st;
#pragma unroll
      for (int gi = 0; gi < GPT; ++gi) {
        const int g = half + 2 * gi;
        float2 x[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = raw[lrow | d.lf[4 * g + q]];
        if constexpr (VAR == EV_FUSED_TF32X3) {
          const uint32_t kb = uint32_t(g / 4) * kRows * 128 + rsw;
          const uint32_t c0 = uint32_t(2 * (g % 4));
          float hi[8], lo[8];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            hi[2 * q] = __uint_as_float(__float_as_uint(x[q].x) & 0xFFFFE000u);
            hi[2 * q + 1] = __uint_as_float(__float_as_uint(x[q].y) & 0xFFFFE000u);
            lo[2 * q] = x[q].x - hi[2 * q];
            lo[2 * q + 1] = x[q].y - hi[2 * q + 1];
          }
          const uint32_t o0 = kb + ((c0 ^ rx) << 4), o1 = kb + (((c0 + 1) ^ rx) << 4);
          *reinterpret_cast<float4*>(a_hi + o0) = make_float4(hi[0], hi[1], hi[2], hi[3]);
          *reinterpret_cast<float4*>(a_hi + o1) = make_float4(hi[4], hi[5], hi[6], hi[7]);
          *reinterpret_cast<float4*>(a_lo + o0) = make_float4(lo[0], lo[1], lo[2], lo[3]);
          *reinterpret_cast<float4*>(a_lo + o1) = make_float4(lo[4], lo[5], lo[6], lo[7]);
        } else {
          const uint32_t o = uint32_t(g / 8) * kRows * 128 + rsw + ((uint32_t(g % 8) ^ rx) << 4);
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const __nv_bfloat16 hr = __float2bfloat16_rn(x[q].x), hm = __float2bfloat16_rn(x[q].y);
            const __nv_bfloat16 lr = __float2bfloat16_rn(x[q].x - __bfloat162float(hr));
            const __nv_bfloat16 lm = __float2bfloat16_rn(x[q].y - __bfloat162float(hm));
            hw[q] = uint32_t(__bfloat16_as_ushort(hr)) | (uint32_t(__bfloat16_as_ushort(hm)) << 16);
            lw[q] = uint32_t(__bfloat16_as_ushort(lr)) | (uint32_t(__bfloat16_as_ushort(lm)) << 16);
          }
          *reinterpret_cast<uint4*>(a_hi + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4*>(a_lo + o) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      compute_sync();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t ah = smem_addr(a_hi), al = smem_addr(a_lo);
        const uint32_t bh = smem_addr(b_hi), bl = smem_addr(b_lo);
        constexpr int per_row = 128 / ESZ;
        uint32_t acc = 0;
#pragma unroll
        for (int kk = 0; kk < K; kk += Elem<VAR>::kstep) {
          const int kb = kk / per_row;
          const uint32_t kin = uint32_t((kk % per_row) * ESZ);
          const uint32_t ao = uint32_t(kb * kRows * 128) + kin;
          const uint32_t bo = uint32_t(kb * K * 128) + kin;
          mma_issue<VAR>(tmem, sw128_desc(ah + ao), sw128_desc(bh + bo), idesc, acc);
          acc = 1;
          mma_issue<VAR>(tmem, sw128_desc(ah + ao), sw128_desc(bl + bo), idesc, 1);
          mma_issue<VAR>(tmem, sw128_desc(al + ao), sw128_desc(bh + bo), idesc, 1);
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_addr(&mma_bar))
            : "memory");
      }
      if (!mbar_wait(&mma_bar, mphase, kWaitLimit)) {
        atomicExch(err, 1);
        s_ok = 0;
      }
      compute_sync();
      if (!s_ok) break;
      mphase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t lane_base = tmem + (uint32_t(quarter * 32) << 16);
#pragma unroll
      for (int c0 = half * (K / 2); c0 < (half + 1) * (K / 2); c0 += 16) {
        uint32_t w[16];
        tmem_ld16(lane_base + uint32_t(c0), w);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 8; ++j)
          raw[lrow | d.lf[c0 / 2 + j]] =
              make_float2(__uint_as_float(w[2 * j]), __uint_as_float(w[2 * j + 1]));
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      compute_sync();
      if (tid == 0) mbar_arrive(&empty_bar[st]);
    }
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(uint32_t(Sh::TMEM_COLS)));
  }
}

// ---- tcgen05 kernel, complex128 by digit slicing (ev_ozaki.cuh) ---------------
//
// One CTA per SM: 16 worker warps and one MMA warp; seven A digit slices of
// 16 KiB, the B digit slices (56 KiB) and 448 TMEM columns.  Digits travel
// as FP16 (exact for |digit| <= 2048; A and B of one MMA share the type).
//
// Layouts.  B rows are ordered [half h][slice j][32 columns n mod 32] and the
// TMEM accumulators [half h][diagonal d][32 columns], so that for one output
// half the products of A slice i with B slices 0..6-i -- diagonals i..6 --
// are ONE MMA of N = 32 (7 - i) whose B rows and D columns are contiguous:
// 2 halves x 7 slices x 4 K-steps = 56 MMAs per step.
//
// Roles of a worker.  Preparation: warp w, lane l handles row 8w + l mod 8,
// quarter l/8 of it (groups of four amplitudes g = l/8 and g + 4); the four
// threads of a row (lanes l, l + 8, l + 16, l + 24) take the row's largest
// exponent with two shuffles, and the eight lanes of a store phase hold
// eight different rows (their 16-byte chunks land in eight bank groups).
// Recombination: thread t reads TMEM lane t mod 128 (its row), output
// columns 16 (t / 128) .. + 15.
//
// A step s: the workers write the A slices from the prepared digits of s,
// start loading the rows of s + 1, meet at a barrier (wbar: an mbarrier, so
// that the wait is bounded) and signal the MMA warp (abar); its lane 0 issues the MMAs of output half 0 (committed to
// bar[0]) and half 1 (bar[1]) -- issue blocks at about the tensor core's
// pace, hence a warp of its own; meanwhile the workers prepare s + 1
// (largest exponent, fixed-point values), then recombine s once its half is
// done.  A worker's arrival at the barrier of s + 1 also means its TMEM reads
// of s are complete.  Every wait is bounded; on timeout the kernel records an
// error, frees TMEM and returns.

constexpr int kOzWorkers = 512;                // 16 worker warps
constexpr int kOzThreads = kOzWorkers + 32;    // and the MMA warp

template <int ND>
struct OzShape {
  static constexpr int K = oz::kK;
  static constexpr int A_SLICE = kRows * K * 2;  // 128 rows x 64 FP16
  static constexpr int B_SLICE = K * K * 2;      // 64 x 64 FP16
  static constexpr int SMEM = ND * (A_SLICE + B_SLICE) + 1024;
  static constexpr int TMEM_COLS = 512;
  static constexpr int HALF_COLS = ND * 32;  // TMEM columns (and B rows) per half
  static constexpr int BLOB = ND * B_SLICE + K * 4;  // B slices, column exponents
};

__device__ __forceinline__ uint32_t hsub2_bits(uint32_t a, uint32_t b) {
  __half2 x, y;
  memcpy(&x, &a, 4);
  memcpy(&y, &b, 4);
  const __half2 r = __hsub2(x, y);
  uint32_t u;
  memcpy(&u, &r, 4);
  return u;
}

// FP16 digits (u - 128) of byte k of w0 and of w1, packed [w0's | w1's << 16]:
// f16 bits 0x6400 | u are 1024 + u, and 1024 + u - 1152 is exact.
template <int k>
__device__ __forceinline__ uint32_t oz_byte_digits(uint32_t w0, uint32_t w1) {
  const uint32_t t = __byte_perm(w0, w1, uint32_t(k | ((k + 4) << 8)));
  return hsub2_bits((t & 0x00FF00FFu) | 0x64006400u, 0x64806480u);
}

// The ND FP16 digits of two biased fixed-point values (b = M + kBias),
// packed per slice as one 32-bit word [first | second << 16].
template <int ND>
__device__ __forceinline__ void oz_digits(uint64_t b0, uint64_t b1, uint32_t w[ND]) {
  const uint32_t l0 = uint32_t(b0), h0 = uint32_t(b0 >> 32);
  const uint32_t l1 = uint32_t(b1), h1 = uint32_t(b1 >> 32);
  // top digits X0 in [-128, 128] (bits 48.. for seven digits, 40.. for
  // six): f16 bits 0x6600 + X0 are 1536 + X0
  constexpr int tsh = ND == 7 ? 16 : 8;
  const uint32_t t0 = uint32_t(0x6600 + (int32_t(h0) >> tsh));
  const uint32_t t1 = uint32_t(0x6600 + (int32_t(h1) >> tsh));
  w[0] = hsub2_bits(__byte_perm(t0, t1, 0x5410), 0x66006600u);
  if constexpr (ND == 7) {
    w[1] = oz_byte_digits<1>(h0, h1);
    w[2] = oz_byte_digits<0>(h0, h1);
    w[3] = oz_byte_digits<3>(l0, l1);
    w[4] = oz_byte_digits<2>(l0, l1);
    w[5] = oz_byte_digits<1>(l0, l1);
    w[6] = oz_byte_digits<0>(l0, l1);
  } else {
    w[1] = oz_byte_digits<0>(h0, h1);
    w[2] = oz_byte_digits<3>(l0, l1);
    w[3] = oz_byte_digits<2>(l0, l1);
    w[4] = oz_byte_digits<1>(l0, l1);
    w[5] = oz_byte_digits<0>(l0, l1);
  }
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t v[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                 "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}

// Row preparation, in place: v holds the bits of this thread's 16 reals of
// the row (two groups of four amplitudes, [re, im]) and becomes their biased
// fixed-point values; returns the row's largest exponent (over its four
// threads: lanes l, l + 8, l + 16, l + 24).
template <int ND>
__device__ __forceinline__ int oz_prepare(uint64_t (&v)[2][4][2], int* err) {
  int em = 0;
#pragma unroll
  for (int gi = 0; gi < 2; ++gi)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < 2; ++c) em = max(em, oz::exp_of(uint32_t(v[gi][i][c] >> 32)));
  em = max(em, __shfl_xor_sync(0xFFFFFFFFu, em, 8));
  em = max(em, __shfl_xor_sync(0xFFFFFFFFu, em, 16));
  if (em == 0x7FF) atomicCAS(err, 0, kFlagNonFinite);  // NaN or infinity in the row
#pragma unroll
  for (int gi = 0; gi < 2; ++gi)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < 2; ++c)
        v[gi][i][c] = uint64_t(oz::fixed<ND>(uint32_t(v[gi][i][c] >> 32), uint32_t(v[gi][i][c]), em)) +
                      oz::Fmt<ND>::kBias;
  return em;
}

// One amplitude's bits.
__device__ __forceinline__ void oz_load(const double2* p, uint64_t (&v)[2]) {
  const double2 a = __ldcs(p);
  v[0] = uint64_t(__double_as_longlong(a.x));
  v[1] = uint64_t(__double_as_longlong(a.y));
}

template <int ND>
__global__ void __launch_bounds__(kOzThreads, 1)
    k_fused_oz(double2* __restrict__ s, const FusedDesc* __restrict__ gd,
               const unsigned char* __restrict__ bmat, int* __restrict__ err) {
  using Sh = OzShape<ND>;
  constexpr int K = Sh::K;
  extern __shared__ unsigned char smem_raw[];
  __shared__ FusedDesc d;
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ __align__(8) uint64_t abar;  // A slices of a step written
  __shared__ __align__(8) uint64_t wbar;  // all workers past their digit writes
  __shared__ uint32_t tmem_slot;
  __shared__ int fexp[K];
  __shared__ int rowexp[2][kRows];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_sl = sm;
  unsigned char* b_sl = sm + ND * Sh::A_SLICE;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  for (int i = tid; i < int(sizeof(FusedDesc) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&d)[i] = reinterpret_cast<const uint64_t*>(gd)[i];
  {
    // blob [slice j][column n][k] -> B row (n / 32) * 224 + 32 j + n mod 32
    const uint16_t* src = reinterpret_cast<const uint16_t*>(bmat);
    for (int e = tid; e < ND * K * K; e += blockDim.x) {
      const int j = e / (K * K), n = (e / K) % K, k = e % K;
      const int brow = (n >> 5) * Sh::HALF_COLS + 32 * j + (n & 31);
      *reinterpret_cast<uint16_t*>(b_sl + sw128_off(brow, k, ND * K, 2)) = src[e];
    }
    const int* fe = reinterpret_cast<const int*>(bmat + ND * Sh::B_SLICE);
    for (int n = tid; n < K; n += blockDim.x) fexp[n] = fe[n];
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[1])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&abar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&wbar)),
                 "n"(kOzWorkers));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_slot)),
                 "r"(uint32_t(Sh::TMEM_COLS)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  if (warp == kOzWorkers / 32) {
    // the MMA warp
    if (lane == 0) {
      // descriptor start addresses are address >> 4: offsets add directly
      const uint64_t ad = sw128_desc(smem_addr(a_sl)), bd = sw128_desc(smem_addr(b_sl));
      uint32_t aphase = 0;
      for (uint64_t st = blockIdx.x; st < d.nsteps; st += gridDim.x) {
        if (!mbar_wait(&abar, aphase, kWaitLimit)) {
          atomicExch(err, 1);
          break;
        }
        aphase ^= 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
#pragma unroll 1
          for (int i = 0; i < ND; ++i) {
            const uint32_t n = uint32_t(32 * (ND - i));
            // f32 accumulate, FP16 A and B, K-major, N, M = 128
            const uint32_t idesc = (1u << 4) | ((n >> 3) << 17) | (uint32_t(kRows >> 4) << 24);
            const uint64_t a = ad + uint64_t(i * (Sh::A_SLICE >> 4));
            const uint64_t bb = bd + uint64_t(h * (Sh::HALF_COLS * 128 >> 4));
            const uint32_t dt = tmem + uint32_t(h * Sh::HALF_COLS + 32 * i);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              mma_f16(dt, a + uint64_t(kk * 2), bb + uint64_t(kk * 2), idesc, (i | kk) != 0);
          }
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                  smem_addr(&bar[h]))
              : "memory");
        }
      }
    }
    __syncwarp();
    __syncthreads();
    return;  // TMEM is freed by warp 0
  }
  uint32_t phase = 0;
  bool ok = true;
  // preparation role: the eight lanes of a store phase hold eight different
  // rows, so their 16-byte chunks land in eight different bank groups
  const int prow = 8 * warp + (lane & 7), pq = lane >> 3;
  const uint32_t prsw = uint32_t((prow >> 3) * 1024 + (prow & 7) * 128);
  const uint32_t prx = uint32_t(prow & 7);
  const uint64_t proff = d.rtab[prow];
  // recombination role
  const int quarter = warp & 3, part = warp >> 2, half = part >> 1;
  const int erow = quarter * 32 + lane;
  const uint64_t eroff = d.rtab[erow];
  const uint32_t lane_tmem = tmem + (uint32_t(quarter * 32) << 16);
  const uint32_t col0 = uint32_t(half * Sh::HALF_COLS + (part & 1) * 16);

  uint64_t b[2][4][2];  // the rows' bits, then their biased fixed-point values
  int em = 0;
  uint64_t step = blockIdx.x;
  // Step bases advance by a masked add: with M the mask of the step-index
  // qubits, base(s + grid) = ((base(s) | ~M) + base(grid)) & M.
  uint64_t cmask = 0;
  for (int q = 0; q < d.ncomp_hi; ++q) cmask |= uint64_t(1) << d.comp_hi[q];
  const uint64_t gbase = step_base(d, gridDim.x);
  const int nruns = 1 << (d.k + 7 - d.lowbits);  // the 2^(k+7) amplitudes of a step
  const uint32_t run_bytes = 16u << d.lowbits;
  uint64_t sb = step_base(d, step);
  if (step < d.nsteps) {
    const uint64_t rb = sb | proff;
#pragma unroll
    for (int gi = 0; gi < 2; ++gi)
#pragma unroll
      for (int i = 0; i < 4; ++i) oz_load(s + (rb | d.ftab[4 * (pq + 4 * gi) + i]), b[gi][i]);
    em = oz_prepare<ND>(b, err);
  }
  for (int par = 0; step < d.nsteps && ok; step += gridDim.x, par ^= 1) {
    // A slices of this step from the prepared digits
#pragma unroll
    for (int gi = 0; gi < 2; ++gi) {
      const int g = pq + 4 * gi;  // reals 8g..8g+7: chunk g of the row's 128-byte line
      const uint32_t o = prsw + ((uint32_t(g) ^ prx) << 4);
      uint32_t w[4][ND];
#pragma unroll
      for (int i = 0; i < 4; ++i) oz_digits<ND>(b[gi][i][0], b[gi][i][1], w[i]);
#pragma unroll
      for (int sl = 0; sl < ND; ++sl)
        *reinterpret_cast<uint4*>(a_sl + sl * Sh::A_SLICE + o) =
            make_uint4(w[0][sl], w[1][sl], w[2][sl], w[3][sl]);
    }
    if (pq == 0) rowexp[par][prow] = em;
    // the next step's rows, in flight while the MMAs are issued
    const uint64_t nstep = step + gridDim.x;
    if (nstep < d.nsteps) {
      const uint64_t nb = (((sb | ~cmask) + gbase) & cmask) | proff;
#pragma unroll
      for (int gi = 0; gi < 2; ++gi)
#pragma unroll
        for (int i = 0; i < 4; ++i) oz_load(s + (nb | d.ftab[4 * (pq + 4 * gi) + i]), b[gi][i]);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // the workers meet (every one arrives, the wait is bounded), then the
    // MMA warp is told that the A slices of this step are complete
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&wbar)) : "memory");
    if (!mbar_wait(&wbar, phase, kWaitLimit)) {
      ok = false;
      atomicExch(err, 1);
      break;
    }
    if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&abar)) : "memory");
    // the rows of the step after next into L2 (contiguous runs of 2^lowbits
    // amplitudes, at most 32 of them), so that next step's loads hit L2
    if (warp == 1 && lane < nruns && nstep + gridDim.x < d.nsteps) {
      const uint64_t b2 = (((((sb | ~cmask) + gbase) & cmask) | ~cmask) + gbase) & cmask;
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(s + (b2 | d.hitab[lane])),
                   "r"(run_bytes)
                   : "memory");
    }
    // prepare the next step while the tensor core works
    if (nstep < d.nsteps) em = oz_prepare<ND>(b, err);
    if (!mbar_wait(&bar[half], phase, kWaitLimit)) {
      ok = false;
      atomicExch(err, 1);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int rem = rowexp[par][erow];
    const uint64_t rbase = sb | eroff;
#pragma unroll
    for (int c0 = 0; c0 < 16; c0 += 8) {
      const uint32_t ta = lane_tmem + col0 + uint32_t(c0);
      int64_t acc[8];
      {
        uint32_t v[ND][8];
#pragma unroll
        for (int dg = 0; dg < ND; ++dg) tmem_ld8(ta + uint32_t(32 * dg), v[dg]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          int32_t g3, g2;
          oz::combine_hi(__uint_as_float(v[0][c]), __uint_as_float(v[1][c]),
                         __uint_as_float(v[2][c]), __uint_as_float(v[3][c]), g3, g2);
          if constexpr (ND == 7)
            acc[c] = oz::combine_g(g3, g2,
                                   oz::combine_lo(__uint_as_float(v[4][c]), __uint_as_float(v[5][c]),
                                                  __uint_as_float(v[6][c])));
          else
            acc[c] = oz::combine_g6(g3, g2,
                                    oz::combine_lo6(__uint_as_float(v[4][c]), __uint_as_float(v[5][c])));
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int n = half * 32 + (part & 1) * 16 + c0 + 2 * j;
        // three outputs in four converted on the FP64 pipe, which is idle
        // while the integer pipes recombine, the fourth on the integer pipes:
        // the same values either way.  30 qubits, ms per run (seven / six
        // digits): all on the integer pipes 903 / 865, half on FP64 838 /
        // 800, three quarters 825 / 771, all 832 / 766
        const int p_re = rem + fexp[n] - oz::Fmt<ND>::kPow2Bias;
        const int p_im = rem + fexp[n + 1] - oz::Fmt<ND>::kPow2Bias;
        const double re = oz::scaled_fp64(acc[2 * j], p_re);
        const double im = (j & 1) ? oz::scaled_fp64(acc[2 * j + 1], p_im) : oz::scaled(acc[2 * j + 1], p_im);
        __stcs(s + (rbase | d.ftab[n >> 1]), make_double2(re, im));
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // the A slices are rewritten next step: every MMA of this one must be done
    if (half == 0 && !mbar_wait(&bar[1], phase, kWaitLimit)) {
      ok = false;
      atomicExch(err, 1);
      break;
    }
    phase ^= 1;
    sb = ((sb | ~cmask) + gbase) & cmask;
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(uint32_t(Sh::TMEM_COLS)));
  }
}

// ---- host: launch ---------------------------------------------------------------

static uint32_t tf32_hi_bits(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u & 0xFFFFE000u;
}
static float bits_f(uint32_t u) {
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}
static uint16_t bf16_rn(float x) {  // round to nearest even
  uint32_t u;
  std::memcpy(&u, &x, 4);
  const uint32_t lsb = (u >> 16) & 1;
  u += 0x7FFFu + lsb;
  return uint16_t(u >> 16);
}
static float bf16_f(uint16_t h) { return bits_f(uint32_t(h) << 16); }

// Row-major [N][K] operand images (hi then lo) of W^T for one block.
static void build_bmat(const Block& b, int variant, std::vector<unsigned char>* out) {
  const int D = 1 << b.F.size(), K = 2 * D;
  std::vector<double> Wt(size_t(K) * K);  // Wt[n][k] = W[k][n]
  for (int a = 0; a < D; ++a)
    for (int f = 0; f < D; ++f) {
      const cd u = b.U[size_t(a) * D + f];
      Wt[size_t(2 * a) * K + 2 * f] = u.real();
      Wt[size_t(2 * a) * K + 2 * f + 1] = -u.imag();
      Wt[size_t(2 * a + 1) * K + 2 * f] = u.imag();
      Wt[size_t(2 * a + 1) * K + 2 * f + 1] = u.real();
    }
  if (variant == EV_FUSED_TF32X3) {
    out->assign(size_t(2) * K * K * 4, 0);
    uint32_t* hi = reinterpret_cast<uint32_t*>(out->data());
    uint32_t* lo = hi + size_t(K) * K;
    for (size_t e = 0; e < Wt.size(); ++e) {
      const float w = float(Wt[e]);
      const uint32_t h = tf32_hi_bits(w);
      const float l = float(Wt[e] - double(bits_f(h)));
      hi[e] = h;
      std::memcpy(&lo[e], &l, 4);
    }
  } else {
    out->assign(size_t(2) * K * K * 2, 0);
    uint16_t* hi = reinterpret_cast<uint16_t*>(out->data());
    uint16_t* lo = hi + size_t(K) * K;
    for (size_t e = 0; e < Wt.size(); ++e) {
      const uint16_t h = bf16_rn(float(Wt[e]));
      hi[e] = h;
      lo[e] = bf16_rn(float(Wt[e] - double(bf16_f(h))));
    }
  }
}

// FP16 bits of a small integer (|v| <= 2048: exact in FP16).
static uint16_t f16_of_int(int v) {
  if (v == 0) return 0;
  const uint32_t sign = v < 0 ? 0x8000u : 0u;
  const uint32_t a = uint32_t(v < 0 ? -v : v);
  int e = 0;
  while ((a >> (e + 1)) != 0) ++e;  // a in [2^e, 2^(e+1))
  return uint16_t(sign | (uint32_t(e + 15) << 10) | ((a << (10 - e)) & 0x3FFu));
}

// The integer an FP16 digit holds (inverse of f16_of_int).
static int int_of_f16(uint16_t h) {
  if ((h & 0x7FFFu) == 0) return 0;
  const int e = int((h >> 10) & 0x1F) - 15;
  const int mag = int((0x400u | (h & 0x3FFu)) >> (10 - e));
  return (h & 0x8000u) ? -mag : mag;
}

// Digit-sliced operand of W^T for the complex128 pass: row n of W^T (column n
// of W) is scaled by its own largest biased exponent F_n and written as seven
// FP16 digit slices [N][K] (slice 0 = most significant), followed by the 64
// exponents F_n (ev_ozaki.cuh).
template <int ND>
static void oz_slice_columns(const double* Wt, std::vector<unsigned char>* out) {
  constexpr int K = oz::kK;
  // FP16 bits of every digit value, -128..128
  static const std::vector<uint16_t> f16_tab = [] {
    std::vector<uint16_t> t(257);
    for (int v = -128; v <= 128; ++v) t[size_t(v + 128)] = f16_of_int(v);
    return t;
  }();
  out->assign(OzShape<ND>::BLOB, 0);
  uint16_t* sl = reinterpret_cast<uint16_t*>(out->data());
  int32_t* fe = reinterpret_cast<int32_t*>(out->data() + ND * OzShape<ND>::B_SLICE);
  for (int n = 0; n < K; ++n) {
    int E = 0;
    for (int k = 0; k < K; ++k) {
      uint64_t u;
      std::memcpy(&u, &Wt[size_t(n) * K + k], 8);
      E = std::max(E, oz::exp_of(uint32_t(u >> 32)));
    }
    fe[n] = E;
    for (int k = 0; k < K; ++k) {
      uint64_t u;
      std::memcpy(&u, &Wt[size_t(n) * K + k], 8);
      const int64_t M = oz::fixed<ND>(uint32_t(u >> 32), uint32_t(u), E);
      uint16_t* col = sl + size_t(n) * K + k;
      for (int i = 0; i < ND; ++i)
        col[size_t(i) * K * K] = f16_tab[size_t(oz::digit_of<ND>(M, i) + 128)];
    }
  }
}

template <int ND>
static void build_bmat_oz(const Block& b, std::vector<unsigned char>* out) {
  const int D = 1 << b.F.size(), K = 2 * D;
  std::vector<double> Wt(size_t(K) * K);
  for (int a = 0; a < D; ++a)
    for (int f = 0; f < D; ++f) {
      const cd u = b.U[size_t(a) * D + f];
      Wt[size_t(2 * a) * K + 2 * f] = u.real();
      Wt[size_t(2 * a) * K + 2 * f + 1] = -u.imag();
      Wt[size_t(2 * a + 1) * K + 2 * f] = u.imag();
      Wt[size_t(2 * a + 1) * K + 2 * f + 1] = u.real();
    }
  oz_slice_columns<ND>(Wt.data(), out);
}

template <int ND>
static int launch_oz(ev_state* s, const FusedDesc* dd, const unsigned char* db, uint64_t nsteps,
                     int* derr) {
  EV_TRY(prepare_smem_kernel(reinterpret_cast<const void*>(k_fused_oz<ND>)));
  uint64_t grid = uint64_t(s->num_sms);  // one CTA per SM (shared memory and TMEM)
  if (grid > nsteps) grid = nsteps;
  s->tc_ctas_per_sm = 1;
  if (debug_enabled())
    fprintf(stderr, "[ev] k_fused_oz<%d> smem %d per CTA, grid %llu\n", ND, OzShape<ND>::SMEM,
            (unsigned long long)grid);
  k_fused_oz<ND><<<unsigned(grid), kOzThreads, OzShape<ND>::SMEM, s->stream>>>(
      static_cast<double2*>(s->amps), dd, db, derr);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

template <int KB, int VAR>
static int launch_tc(ev_state* s, const FusedDesc* dd, const unsigned char* db, uint64_t nsteps,
                     int* derr) {
  using Sh = TcShape<KB, VAR>;
  EV_TRY(prepare_smem_kernel(reinterpret_cast<const void*>(k_fused_tc<KB, VAR>)));
  // resident CTAs from the SM's shared-memory budget (dynamic + static +
  // the 1 KiB the runtime reserves per CTA)
  cudaFuncAttributes fa{};
  EV_CUDA(cudaFuncGetAttributes(&fa, k_fused_tc<KB, VAR>));
  int smem_sm = 0;
  EV_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, s->device));
  int per_sm = smem_sm / int(Sh::SMEM + fa.sharedSizeBytes + 1024);
  int regs_sm = 0;
  EV_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, s->device));
  const int by_regs = regs_sm / ((fa.numRegs + 7) / 8 * 8 * kTcThreads);
  if (per_sm > by_regs) per_sm = by_regs;
  if (per_sm < 1) per_sm = 1;
  // keep every resident CTA's TMEM allocation satisfiable at once
  const int tmem_cap = 512 / Sh::TMEM_COLS;
  if (per_sm > tmem_cap) per_sm = tmem_cap;
  s->tc_ctas_per_sm = per_sm;
  uint64_t grid = uint64_t(s->num_sms) * per_sm;
  if (grid > nsteps) grid = nsteps;
  if (debug_enabled())
    fprintf(stderr, "[ev] k_fused_tc<%d,%d> smem %d+%zu per CTA, %d CTAs/SM, grid %llu\n", KB, VAR,
            Sh::SMEM, size_t(fa.sharedSizeBytes), per_sm, (unsigned long long)grid);
  k_fused_tc<KB, VAR><<<unsigned(grid), kTcThreads, Sh::SMEM, s->stream>>>(
      static_cast<float2*>(s->amps), dd, db, derr);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

template <int KB, int VAR, int STAGES>
static int launch_tma(ev_state* s, const FusedDesc* dd, const unsigned char* db, uint64_t nsteps,
                      int* derr) {
  using Tm = TmaShape<KB, VAR, STAGES>;
  using Sh = TcShape<KB, VAR>;
  EV_TRY(prepare_smem_kernel(reinterpret_cast<const void*>(k_fused_tma<KB, VAR, STAGES>)));
  cudaFuncAttributes fa{};
  EV_CUDA(cudaFuncGetAttributes(&fa, k_fused_tma<KB, VAR, STAGES>));
  int smem_sm = 0, regs_sm = 0;
  EV_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, s->device));
  EV_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, s->device));
  int per_sm = smem_sm / int(Tm::SMEM + fa.sharedSizeBytes + 1024);
  const int by_regs = regs_sm / ((fa.numRegs + 7) / 8 * 8 * kTmaThreads);
  if (per_sm > by_regs) per_sm = by_regs;
  if (per_sm > 512 / Sh::TMEM_COLS) per_sm = 512 / Sh::TMEM_COLS;
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = uint64_t(s->num_sms) * per_sm;
  if (grid > nsteps) grid = nsteps;
  if (debug_enabled())
    fprintf(stderr, "[ev] k_fused_tma<%d,%d,%d> smem %d+%zu per CTA, %d CTAs/SM, grid %llu\n", KB,
            VAR, STAGES, Tm::SMEM, size_t(fa.sharedSizeBytes), per_sm, (unsigned long long)grid);
  k_fused_tma<KB, VAR, STAGES><<<unsigned(grid), kTmaThreads, Tm::SMEM, s->stream>>>(
      static_cast<float2*>(s->amps), dd, db, derr);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

template <int KB>
static int launch_fp32(ev_state* s, const FusedDesc* dd, const float2* du, uint64_t nsteps) {
  constexpr int D = 1 << KB;
  const int smem = int(sizeof(float2)) * (kRows * D + D * D);
  EV_TRY(prepare_smem_kernel(reinterpret_cast<const void*>(k_fused_fp32<KB>)));
  uint64_t grid = uint64_t(s->num_sms) * 2;
  if (grid > nsteps) grid = nsteps;
  k_fused_fp32<KB><<<unsigned(grid), 256, smem, s->stream>>>(static_cast<float2*>(s->amps), dd, du);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int default_fused_bits() { return 5; }

int plan_tiled(ev_state* s, const ev_circuit* c, uint64_t first, uint64_t last, int tile_bits,
               PlanBlob* blob, std::vector<SegStep>* out);

// Fusion width actually used for a variant and a request (0 = default).
int fused_width(int variant, int kbits) {
  int k = kbits > 0 ? kbits : default_fused_bits();
  if (k > 6) k = 6;
  if (k < 1) k = 1;
  if (variant == EV_FUSED_TF32X3 || variant == EV_FUSED_OZAKI || variant == EV_FUSED_OZAKI6)
    return 5;
  if (variant == EV_FUSED_BF16X3) return k >= 6 ? 6 : 5;
  return k;
}

// Plans a gate run into fused-unitary passes: descriptors and operand
// images go into the blob.
static int plan_fused(ev_state* s, const ev_circuit* c, uint64_t first, uint64_t last, int kbits,
                      int variant, PlanBlob* blob, std::vector<SegStep>* out) {
  if (variant < EV_FUSED_TF32X3 || variant > EV_FUSED_OZAKI6)
    return fail(EV_ERR_INVALID_ARGUMENT, "unknown fused variant %d", variant);
  const bool ozaki = variant == EV_FUSED_OZAKI || variant == EV_FUSED_OZAKI6;
  if (ozaki != (s->dtype == EV_C128))
    return fail(EV_ERR_INVALID_ARGUMENT,
                ozaki ? "the ozaki fused variants need a complex128 state"
                      : "this fused variant needs a complex64 state");
  const int n = int(s->n);
  const int k = fused_width(variant, kbits);
  // registers too small for 128-row steps run through the tile pass
  if (n < k + 7) return plan_tiled(s, c, first, last, 0, blob, out);
  const bool tc = variant != EV_FUSED_FP32;
  // Register-staged streaming (default: the faster of the two on GB300, see
  // the measured comparison in the design notes) or the warp-specialised
  // TMA-staged pipeline (EV_FUSED_STAGING=tma), read when a run is planned.
  const char* staging = getenv("EV_FUSED_STAGING");
  const bool use_tma = staging != nullptr && std::strcmp(staging, "tma") == 0 && !ozaki;
  std::vector<Block> blocks = fuse_ops(c, first, last, n, k);
  std::vector<unsigned char> mat;
  for (const Block& b : blocks) {
    if (variant == EV_FUSED_OZAKI) {
      build_bmat_oz<7>(b, &mat);
    } else if (variant == EV_FUSED_OZAKI6) {
      build_bmat_oz<6>(b, &mat);
    } else if (tc) {
      build_bmat(b, variant, &mat);
    } else {
      const int D = 1 << b.F.size();
      mat.assign(size_t(D) * D * sizeof(float2), 0);
      float2* u = reinterpret_cast<float2*>(mat.data());
      for (int e = 0; e < D * D; ++e) u[e] = make_float2(float(b.U[e].real()), float(b.U[e].imag()));
    }
    FusedDesc d;
    std::memset(&d, 0, sizeof(d));
    build_desc(b, n, &d);
    SegStep st;
    st.fused = 1;
    st.off0 = blob->add(&d, sizeof(d));
    st.off1 = blob->add(mat.data(), mat.size());
    st.k = int(b.F.size());
    st.variant = variant;
    st.tma = use_tma ? 1 : 0;
    st.count = d.nsteps;
    out->push_back(st);
  }
  return EV_OK;
}

int launch_fused_step(ev_state* s, const SegStep& st, const unsigned char* dblob) {
  const FusedDesc* dd = reinterpret_cast<const FusedDesc*>(dblob + st.off0);
  const unsigned char* dm = dblob + st.off1;
  int* derr = reinterpret_cast<int*>(s->scratch.counter + 1);
  ProfScope prof(s, P_FUSED, 2.0 * double(s->len()) * (s->dtype == EV_C128 ? 16.0 : 8.0));
  s->launches += 1;
  const uint64_t nsteps = st.count;
  const bool tma = st.tma != 0;
  if (st.variant == EV_FUSED_OZAKI) return launch_oz<7>(s, dd, dm, nsteps, derr);
  if (st.variant == EV_FUSED_OZAKI6) return launch_oz<6>(s, dd, dm, nsteps, derr);
  if (st.variant == EV_FUSED_TF32X3)
    return tma ? launch_tma<5, EV_FUSED_TF32X3, 3>(s, dd, dm, nsteps, derr)
               : launch_tc<5, EV_FUSED_TF32X3>(s, dd, dm, nsteps, derr);
  if (st.variant == EV_FUSED_BF16X3) {
    if (st.k == 5)
      return tma ? launch_tma<5, EV_FUSED_BF16X3, 3>(s, dd, dm, nsteps, derr)
                 : launch_tc<5, EV_FUSED_BF16X3>(s, dd, dm, nsteps, derr);
    return launch_tc<6, EV_FUSED_BF16X3>(s, dd, dm, nsteps, derr);
  }
  const float2* du = reinterpret_cast<const float2*>(dm);
  switch (st.k) {
    case 1: return launch_fp32<1>(s, dd, du, nsteps);
    case 2: return launch_fp32<2>(s, dd, du, nsteps);
    case 3: return launch_fp32<3>(s, dd, du, nsteps);
    case 4: return launch_fp32<4>(s, dd, du, nsteps);
    case 5: return launch_fp32<5>(s, dd, du, nsteps);
    default: return launch_fp32<6>(s, dd, du, nsteps);
  }
}

// Host restatement of the digit-sliced product for checks: the same slicing
// of W's columns and x's rows, the diagonal sums formed exactly (as the
// tensor core forms them: every partial sum is an integer below 2^24), held
// as f32 and recombined with the device's own routines -- diagonal by
// diagonal, and checked against the kernel's grouped form (false if the two
// differ for any output).
template <int ND>
static bool oz_gemm_host(const double* x, uint64_t rows, const double* W, double* y) {
  constexpr int K = oz::kK;
  std::vector<double> Wt(size_t(K) * K);
  for (int k = 0; k < K; ++k)
    for (int n = 0; n < K; ++n) Wt[size_t(n) * K + k] = W[size_t(k) * K + n];
  std::vector<unsigned char> img;
  oz_slice_columns<ND>(Wt.data(), &img);
  const uint16_t* sl = reinterpret_cast<const uint16_t*>(img.data());
  const int32_t* fe = reinterpret_cast<const int32_t*>(img.data() + ND * OzShape<ND>::B_SLICE);
  for (uint64_t r = 0; r < rows; ++r) {
    const double* xr = x + r * K;
    int E = 0;
    for (int k = 0; k < K; ++k) {
      uint64_t u;
      std::memcpy(&u, &xr[k], 8);
      E = std::max(E, oz::exp_of(uint32_t(u >> 32)));
    }
    int X[K][ND];
    for (int k = 0; k < K; ++k) {
      uint64_t u;
      std::memcpy(&u, &xr[k], 8);
      const int64_t M = oz::fixed<ND>(uint32_t(u >> 32), uint32_t(u), E);
      for (int i = 0; i < ND; ++i) X[k][i] = oz::digit_of<ND>(M, i);
    }
    for (int n = 0; n < K; ++n) {
      float D[ND];
      for (int dg = 0; dg < ND; ++dg) {
        int64_t sum = 0;
        for (int i = 0; i <= dg; ++i)
          for (int k = 0; k < K; ++k)
            sum += int64_t(X[k][i]) * int_of_f16(sl[size_t(dg - i) * K * K + size_t(n) * K + k]);
        D[dg] = float(sum);  // |sum| < 2^24: exact
      }
      int64_t acc = 0;
      oz::accumulate_nd<ND, 0>(acc, D[0]);
      oz::accumulate_nd<ND, 1>(acc, D[1]);
      oz::accumulate_nd<ND, 2>(acc, D[2]);
      oz::accumulate_nd<ND, 3>(acc, D[3]);
      oz::accumulate_nd<ND, 4>(acc, D[4]);
      oz::accumulate_nd<ND, 5>(acc, D[5]);
      if constexpr (ND == 7) oz::accumulate_nd<ND, 6>(acc, D[6]);
      if (oz::combine_nd<ND>(D) != acc) return false;  // the kernel's grouped form
      y[r * K + n] = oz::scaled(acc, E + fe[n] - oz::Fmt<ND>::kPow2Bias);
    }
  }
  return true;
}

int plan_segment(ev_state* s, const ev_circuit* c, uint64_t first, uint64_t last, int mode,
                 int bits, int variant, PlanBlob* blob, std::vector<SegStep>* out) {
  if (mode == EV_MODE_FUSED) return plan_fused(s, c, first, last, bits, variant, blob, out);
  return plan_tiled(s, c, first, last, bits, blob, out);
}

}  // namespace ev

extern "C" int ev_ozaki_gemm_host(const double* x, uint64_t rows, const double* w, double* y) {
  return ev_ozaki_gemm_host_digits(x, rows, w, y, 7);
}

extern "C" int ev_ozaki_gemm_host_digits(const double* x, uint64_t rows, const double* w, double* y,
                                         int32_t digits) {
  ev::clear_error();
  if (!x || !w || !y) return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_ozaki_gemm_host: null argument");
  if (digits != 6 && digits != 7)
    return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_ozaki_gemm_host: %d digits (6 or 7)", digits);
  const bool ok = digits == 7 ? ev::oz_gemm_host<7>(x, rows, w, y) : ev::oz_gemm_host<6>(x, rows, w, y);
  if (!ok)
    return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_ozaki_gemm_host: grouped recombination differs");
  return EV_OK;
}
