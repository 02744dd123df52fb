// ev_tile.cu -- runs of gates applied to shared-memory tiles, one HBM pass
// per run.
//
// A tile is the 2^k amplitudes whose indices agree outside a qubit set T
// (|T| = k, T always holds the lowest L qubits so every tile row is a
// contiguous, fully used run of 2^L amplitudes).  A pass loads each tile
// into shared memory, applies a planned run of gate records in circuit
// order, and writes the tile back: the arithmetic per amplitude is exactly
// that of the per-gate kernels (ev_gates.cu, the reference's
// kernel.rs:100-289), so complex128 results stay bit-identical to the
// reference while HBM sees one read and one write per run instead of one per
// gate.
//
// Which gates fit: every data qubit of a record (1q target, 2q operands)
// must lie in T.  Controls need not: a control outside T is a fixed bit of
// the tile's base index, so the whole tile either takes the gate or skips
// it, and a control inside T becomes a local mask.
#include <algorithm>
#include <cstring>
#include <vector>

#include "ev_device.cuh"
#include "ev_internal.h"

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
  uint8_t pad;
  uint32_t lmask;  // local control mask
  uint32_t pad2;
  uint64_t emask;  // controls outside the tile (global bit mask)
  uint64_t ins;    // T_1Q: sorted local positions of (local controls + target),
                   // 4 bits each, lowest position in the low nibble
  uint64_t pad3[2];
  double m[32];
};

static_assert(sizeof(TileOp) % 16 == 0, "op records are staged with 16-byte copies");

struct TilePlan {
  int k, L;
  int nH;
  uint8_t H[40];     // local positions L..k-1 map to global qubits H[0..nH)
  int ncomp;
  uint8_t comp[64];  // global qubits outside T, ascending
};

template <typename V>
__device__ __forceinline__ V ldm(const double* m, int i) {
  return mkv<V>(m[2 * i], m[2 * i + 1]);
}

__device__ __forceinline__ uint32_t ins0(uint32_t i, int p) {
  return ((i >> p) << (p + 1)) | (i & ((1u << p) - 1));
}

// One (possibly controlled) 1-qubit record over the tile: the pair loop is
// specialised per matrix kind, with the matrix held in registers.
template <int K1, typename V>
__device__ __forceinline__ void tile_1q(V* t, uint32_t count, const TileOp& op) {
  const V m0 = ldm<V>(op.m, 0), m1 = ldm<V>(op.m, 1), m2 = ldm<V>(op.m, 2), m3 = ldm<V>(op.m, 3);
  using R = typename Real<V>::T;
  const uint32_t tbit = 1u << op.p0, lmask = op.lmask;
  const int nins = op.nins;
  const uint64_t ins = op.ins;
  const int ins_first = int(ins & 15);
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

template <int KIND, typename V>
__device__ __forceinline__ void tile_2q(V* t, uint32_t count, const TileOp& op) {
  const uint32_t ba = 1u << op.p0, bb = 1u << op.p1;
  const int lo = op.lo, hi = op.hi;
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
      t[base] = cmul(ldm<V>(op.m, 0), t[base]);
      t[i1] = cmul(ldm<V>(op.m, 5), t[i1]);
      t[i2] = cmul(ldm<V>(op.m, 10), t[i2]);
      t[i3] = cmul(ldm<V>(op.m, 15), t[i3]);
    } else {  // dense 4x4, rows summed left to right
      const V a[4] = {t[base], t[i1], t[i2], t[i3]};
      const uint32_t out[4] = {base, i1, i2, i3};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        V acc = cmul(ldm<V>(op.m, 4 * r + 0), a[0]);
        acc = cadd(acc, cmul(ldm<V>(op.m, 4 * r + 1), a[1]));
        acc = cadd(acc, cmul(ldm<V>(op.m, 4 * r + 2), a[2]));
        acc = cadd(acc, cmul(ldm<V>(op.m, 4 * r + 3), a[3]));
        t[out[r]] = acc;
      }
    }
  }
}

template <typename V>
__device__ void apply_tile_op(V* t, int k, const TileOp& op) {
  const uint32_t size = 1u << k;
  if (op.kind == T_1Q) {
    const uint32_t count = size >> op.nins;
    switch (op.k1) {
      case K1_DENSE: tile_1q<K1_DENSE>(t, count, op); break;
      case K1_REAL: tile_1q<K1_REAL>(t, count, op); break;
      case K1_DIAG: tile_1q<K1_DIAG>(t, count, op); break;
      case K1_PHASE: tile_1q<K1_PHASE>(t, count, op); break;
      case K1_ANTI: tile_1q<K1_ANTI>(t, count, op); break;
      default: break;
    }
    return;
  }
  const uint32_t count = size >> 2;
  switch (op.kind) {
    case T_CNOT: tile_2q<T_CNOT>(t, count, op); break;
    case T_CZ: tile_2q<T_CZ>(t, count, op); break;
    case T_SWAP: tile_2q<T_SWAP>(t, count, op); break;
    case T_DIAG2: tile_2q<T_DIAG2>(t, count, op); break;
    default: tile_2q<T_DENSE2>(t, count, op); break;
  }
}

constexpr int kTileThreads = 512;
constexpr int kMaxPassOps = 48;  // op records per pass (staged in shared memory)

// One persistent block per resident slot; tiles strided over the grid.  The
// pass's op records and index tables are staged in shared memory once per
// block: [tile 2^k amplitudes][row offsets 2^(k-L)][op records][comp qubits].
template <typename V>
__global__ void __launch_bounds__(kTileThreads, 2)
    k_tile(V* __restrict__ s, uint64_t ntiles, const TilePlan* __restrict__ gplan,
           const TileOp* __restrict__ gops, int nops, const uint8_t* pred) {
  if (pred != nullptr && *pred == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = gplan->k, L = gplan->L, nH = gplan->nH, ncomp = gplan->ncomp;
  const uint32_t size = 1u << k;
  const uint32_t nrows = 1u << (k - L);
  V* tile = reinterpret_cast<V*>(smem_raw);
  uint64_t* offs = reinterpret_cast<uint64_t*>(smem_raw + sizeof(V) * size);
  // op records start on a 16-byte boundary (they are staged with 16-byte
  // stores); tile + offsets is not a multiple of 16 bytes for tiny tiles
  const size_t ops_at = (sizeof(V) * size + sizeof(uint64_t) * nrows + 15) & ~size_t(15);
  TileOp* ops = reinterpret_cast<TileOp*>(smem_raw + ops_at);
  uint8_t* comp = reinterpret_cast<uint8_t*>(ops + nops);
  {
    const uint4* src = reinterpret_cast<const uint4*>(gops);
    uint4* dst = reinterpret_cast<uint4*>(ops);
    const int words = nops * int(sizeof(TileOp) / sizeof(uint4));
    for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
    if (threadIdx.x < 64) comp[threadIdx.x] = gplan->comp[threadIdx.x];
  }
  for (uint32_t h = threadIdx.x; h < nrows; h += blockDim.x) {
    uint64_t o = 0;
    for (int b = 0; b < nH; ++b)
      if ((h >> b) & 1) o |= uint64_t(1) << gplan->H[b];
    offs[h] = o;
  }
  const uint32_t lowmask = (1u << L) - 1;
  __syncthreads();
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    uint64_t base = 0;
    for (int b = 0; b < ncomp; ++b)
      if ((t >> b) & 1) base |= uint64_t(1) << comp[b];
#pragma unroll 4
    for (uint32_t l = threadIdx.x; l < size; l += blockDim.x)
      tile[l] = s[base | offs[l >> L] | (l & lowmask)];
    __syncthreads();
    for (int o = 0; o < nops; ++o) {
      const TileOp& op = ops[o];
      if ((base & op.emask) != op.emask) continue;  // uniform across the block
      apply_tile_op(tile, k, op);
      __syncthreads();
    }
#pragma unroll 4
    for (uint32_t l = threadIdx.x; l < size; l += blockDim.x)
      s[base | offs[l >> L] | (l & lowmask)] = tile[l];
    __syncthreads();
  }
}

// ---- host planning ---------------------------------------------------------

struct Pass {
  uint64_t first, last;  // op range [first, last)
  uint64_t tset;         // global qubits of the tile
};

static uint64_t data_qubits(const ev_op& op) {
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

static int popc(uint64_t x) { return __builtin_popcountll(x); }

// Greedy: extend the current pass while the union of data qubits (plus the
// L lowest qubits) fits in k, then fill T with the lowest unused qubits.
static std::vector<Pass> plan_passes(const ev_circuit* c, uint64_t first, uint64_t last, int n,
                                     int k, int L) {
  std::vector<Pass> passes;
  const uint64_t low = (L >= 64) ? ~0ull : ((uint64_t(1) << L) - 1);
  uint64_t pos = first;
  while (pos < last) {
    uint64_t set = low;
    uint64_t end = pos;
    while (end < last && end - pos < uint64_t(kMaxPassOps)) {
      const uint64_t want = set | data_qubits(c->ops[end]);
      if (popc(want) > k) break;
      set = want;
      ++end;
    }
    for (int q = 0; q < n && popc(set) < k; ++q) set |= uint64_t(1) << q;
    passes.push_back({pos, end, set});
    pos = end;
  }
  return passes;
}

static void encode_op(const ev_circuit* c, const ev_op& op, uint64_t tset, const int* local,
                      TileOp* out) {
  std::memset(out, 0, sizeof(*out));
  std::memcpy(out->m, op.m, sizeof(op.m));
  if (op.kind == EV_OP_APPLY2) {
    switch (classify2(op.m)) {
      case K2_CNOT: out->kind = T_CNOT; break;
      case K2_CZ: out->kind = T_CZ; break;
      case K2_SWAP: out->kind = T_SWAP; break;
      case K2_DIAG: out->kind = T_DIAG2; break;
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

template <typename V>
static int launch_tile(ev_state* s, uint64_t ntiles, const TilePlan& plan, const TilePlan* dplan,
                       const TileOp* dops, int nops, const uint8_t* pred) {
  const size_t ops_at = (sizeof(V) * (size_t(1) << plan.k) +
                         sizeof(uint64_t) * (size_t(1) << (plan.k - plan.L)) + 15) & ~size_t(15);
  const size_t smem = ops_at + sizeof(TileOp) * size_t(nops) + 64;
  EV_CUDA(cudaFuncSetAttribute(k_tile<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  EV_CUDA(cudaFuncSetAttribute(k_tile<V>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               int(cudaSharedmemCarveoutMaxShared)));
  int per_sm = 0;
  EV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<V>, kTileThreads, smem));
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = uint64_t(s->num_sms) * per_sm;
  if (grid > ntiles) grid = ntiles;
  ProfScope prof(s, P_TILE, 2.0 * double(s->len()) * double(sizeof(V)));
  s->launches += 1;
  k_tile<V><<<unsigned(grid), kTileThreads, smem, s->stream>>>(static_cast<V*>(s->amps), ntiles,
                                                               dplan, dops, nops, pred);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

int default_tile_bits(int dtype) { return dtype == EV_C128 ? 12 : 13; }

int tiled_run(ev_state* s, const ev_circuit* c, uint64_t first, uint64_t last, int tile_bits,
              const uint8_t* pred, uint64_t* passes_out) {
  const int n = int(s->n);
  int k = tile_bits > 0 ? tile_bits : default_tile_bits(s->dtype);
  if (k > 14) k = 14;
  if (k < 2) k = 2;
  if (k > n) k = n;
  const int L = std::min(k, 4);
  // one op may need 2 data qubits beyond the low ones
  if (k - L < 2 && k < n) k = std::min(n, L + 2);
  std::vector<Pass> passes = plan_passes(c, first, last, n, k, L);
  std::vector<TileOp> ops(last - first);
  std::vector<std::pair<int, int>> ranges;  // (offset, count) into ops per pass
  std::vector<TilePlan> plans;
  uint64_t w = 0;
  for (const Pass& p : passes) {
    TilePlan plan{};
    plan.k = k;
    plan.L = L;
    int local[64];
    for (int q = 0; q < 64; ++q) local[q] = -1;
    int nl = 0;
    for (int q = 0; q < n; ++q)
      if ((p.tset >> q) & 1) {
        local[q] = nl;
        if (nl >= L) plan.H[plan.nH++] = uint8_t(q);
        ++nl;
      } else {
        plan.comp[plan.ncomp++] = uint8_t(q);
      }
    for (uint64_t j = p.first; j < p.last; ++j) encode_op(c, c->ops[j], p.tset, local, &ops[w + (j - p.first)]);
    ranges.push_back({int(w), int(p.last - p.first)});
    plans.push_back(plan);
    w += p.last - p.first;
  }
  // one device buffer: plans, then op records
  const size_t plan_bytes = (passes.size() * sizeof(TilePlan) + 255) / 256 * 256;
  const size_t total = plan_bytes + std::max<size_t>(1, ops.size()) * sizeof(TileOp);
  std::vector<unsigned char> host(total, 0);
  std::memcpy(host.data(), plans.data(), passes.size() * sizeof(TilePlan));
  std::memcpy(host.data() + plan_bytes, ops.data(), ops.size() * sizeof(TileOp));
  unsigned char* dbuf = nullptr;
  EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dbuf), total, s->stream));
  EV_CUDA(cudaMemcpyAsync(dbuf, host.data(), total, cudaMemcpyHostToDevice, s->stream));
  const TilePlan* dplans = reinterpret_cast<const TilePlan*>(dbuf);
  const TileOp* dops = reinterpret_cast<const TileOp*>(dbuf + plan_bytes);
  int rc = EV_OK;
  const uint64_t ntiles = uint64_t(1) << (n - k);
  for (size_t i = 0; i < passes.size() && rc == EV_OK; ++i) {
    if (s->dtype == EV_C128)
      rc = launch_tile<double2>(s, ntiles, plans[i], dplans + i, dops + ranges[i].first,
                                ranges[i].second, pred);
    else
      rc = launch_tile<float2>(s, ntiles, plans[i], dplans + i, dops + ranges[i].first,
                               ranges[i].second, pred);
  }
  cudaFreeAsync(dbuf, s->stream);
  if (passes_out) *passes_out = passes.size();
  return rc;
}

}  // namespace ev
