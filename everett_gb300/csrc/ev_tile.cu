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
#include <cstdlib>
#include <cstring>

#include "ev_bulk.cuh"
#include "ev_tile.cuh"

namespace ev {

constexpr int kTileThreads = 512;
constexpr int kMaxPassOps = 48;  // op records per pass (staged in shared memory)

// Block shape of the pass: by default two blocks of 512 threads per SM with
// the records staged in shared memory; EV_TILE_THREADS=256 three blocks of
// 256 threads per SM (80 registers a thread instead of 64), the records read
// through L1 so that three tiles fit in shared memory; EV_TILE_THREADS=1x512
// one block of 512 threads (128 registers, no spills).  All give the same
// results.  Measured on the complex128 pass (28 qubits, depth 20, ms per
// circuit): two blocks of 512 2311, three of 256 2424, one of 512 2603 (2497
// with 2^13-amplitude tiles): the spills of the 64-register form cost less
// than the warps the other shapes give up.
static int tile_shape() {
  const char* e = getenv("EV_TILE_THREADS");
  if (e == nullptr) return 0;
  if (strcmp(e, "256") == 0) return 1;
  if (strcmp(e, "1x512") == 0) return 2;
  return 0;
}

// How many amplitudes of each pair have their complex128 products formed on
// the integer pipes (TileOp::soft), for real-matrix records and for the
// others.  EV_TILE_SOFT="rd" overrides both: d in 0-2, r in 0-6, where 3-6
// also form the first r - 2 of a real record's four adds per pair on the
// integer pipes (softfp::add).  All give the same results.
struct SoftLevels {
  int real, other;
};
constexpr SoftLevels kDefaultSoft{2, 2};
static SoftLevels tile_soft_levels() {
  const char* e = getenv("EV_TILE_SOFT");
  if (e == nullptr || e[0] < '0' || e[0] > '6' || e[1] < '0' || e[1] > '2' || e[2] != 0)
    return kDefaultSoft;
  return SoftLevels{e[0] - '0', e[1] - '0'};
}


// How tiles move between HBM and shared memory.  By default every thread
// loads and stores its share of the tile with 16-byte accesses.  With
// EV_TILE_STAGING=tma the bulk-copy (TMA) engine moves them instead: a tile
// is 2^(k-L) contiguous rows of 2^L amplitudes, warp 0 issues one
// cp.async.bulk per row, loads complete on an mbarrier and stores are drained
// (their reads of the tile) before the next tile's loads; rows shorter than
// 16 bytes (registers of fewer than 2 qubits) keep the plain path.  Both give
// the same results.  The TMA form measured slower on the complex128 pass
// (28 qubits: 2585 vs 2378 ms per depth-20 circuit): the pass is bound by
// its arithmetic, the 256-byte rows issue serially from one warp while the
// block waits, and the extra live state costs the 64-register threads spills.
static bool tile_bulk_enabled() {
  const char* e = getenv("EV_TILE_STAGING");
  return e != nullptr && e[0] == 't';
}

constexpr uint32_t kTileWaitLimit = 1u << 24;  // try_wait polls before giving up

// One persistent block per resident slot; tiles strided over the grid.  The
// pass's op records and index tables are staged in shared memory once per
// block: [tile 2^k amplitudes][row offsets 2^(k-L)][op records][comp qubits].
// A load that never completes sets *err (the run's device flag, reported as
// EV_ERR_TIMEOUT) and ends the block after a bounded drain.
template <typename V, bool BULK, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    k_tile(V* __restrict__ s, uint64_t ntiles, const TilePlan* __restrict__ gplan,
           const TileOp* __restrict__ gops, int nops, const uint8_t* pred, int* err) {
  constexpr bool kStageOps = MINB < 3;
  if (pred != nullptr && *pred == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  const int k = gplan->k, L = gplan->L, nH = gplan->nH, ncomp = gplan->ncomp;
  const uint32_t size = 1u << k;
  const uint32_t nrows = 1u << (k - L);
  const uint32_t rowbytes = uint32_t(sizeof(V)) << L;
  const bool use_bulk = BULK && rowbytes % 16 == 0;  // uniform across the block
  const int warp = int(threadIdx.x >> 5), lane = int(threadIdx.x & 31);
  V* tile = reinterpret_cast<V*>(smem_raw);
  uint64_t* offs = reinterpret_cast<uint64_t*>(smem_raw + sizeof(V) * size);
  // op records start on a 16-byte boundary (they are staged with 16-byte
  // stores); tile + offsets is not a multiple of 16 bytes for tiny tiles
  const size_t ops_at = (sizeof(V) * size + sizeof(uint64_t) * nrows + 15) & ~size_t(15);
  TileOp* sops = reinterpret_cast<TileOp*>(smem_raw + ops_at);
  const TileOp* ops = kStageOps ? sops : gops;
  uint8_t* comp = reinterpret_cast<uint8_t*>(sops + (kStageOps ? nops : 0));
  if (use_bulk && threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  {
    if (kStageOps) {
      const uint4* src = reinterpret_cast<const uint4*>(gops);
      uint4* dst = reinterpret_cast<uint4*>(sops);
      const int words = nops * int(sizeof(TileOp) / sizeof(uint4));
      for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
    }
    if (threadIdx.x < 64) comp[threadIdx.x] = gplan->comp[threadIdx.x];
  }
  for (uint32_t h = threadIdx.x; h < nrows; h += blockDim.x) {
    uint64_t o = 0;
    for (int b = 0; b < nH; ++b)
      if ((h >> b) & 1) o |= uint64_t(1) << gplan->H[b];
    offs[h] = o;
  }
  const uint32_t lowmask = (1u << L) - 1;
  uint32_t phase = 0;
  __syncthreads();
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    uint64_t base = 0;
    for (int b = 0; b < ncomp; ++b)
      if ((t >> b) & 1) base |= uint64_t(1) << comp[b];
    if (use_bulk) {
      if (warp == 0) {
        if (lane == 0) {
          fence_proxy_async_smem();
          mbar_expect_tx(&bar, rowbytes * nrows);
        }
        __syncwarp();
        for (uint32_t h = uint32_t(lane); h < nrows; h += 32)
          bulk_g2s(tile + (size_t(h) << L), s + (base | offs[h]), rowbytes, &bar);
      }
      const bool ok = mbar_wait(&bar, phase, kTileWaitLimit);
      if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        mbar_wait(&bar, phase, kTileWaitLimit);  // drain the loads in flight (bounded)
        if (warp == 0) bulk_wait_all();          // and the last tile's stores
        return;
      }
      phase ^= 1;
    } else {
#pragma unroll 4
      for (uint32_t l = threadIdx.x; l < size; l += blockDim.x)
        tile[l] = s[base | offs[l >> L] | (l & lowmask)];
      __syncthreads();
    }
    for (int o = 0; o < nops;) {
      const TileOp& op = ops[o];
      const int run = op.run > 1 ? op.run : 1;
      if ((base & op.emask) == op.emask) {  // uniform across the block
        if (run > 1 && op.ctype == CH_QUAD)
          tile_quad_chain(tile, size, ops + o, run, nullptr);
        else if (run > 1 && op.ctype == CH_DIAG)
          tile_diag_chain(tile, size, ops + o, run, nullptr);
        else if (run > 1)
          tile_chain(tile, size >> op.nins, ops + o, run, nullptr);
        else
          apply_tile_op(tile, k, op, op.m);
        __syncthreads();
      }
      o += run;
    }
    if (use_bulk) {
      fence_proxy_async_smem();
      __syncthreads();
      if (warp == 0) {
        for (uint32_t h = uint32_t(lane); h < nrows; h += 32)
          bulk_s2g(s + (base | offs[h]), tile + (size_t(h) << L), rowbytes);
        bulk_commit();
        bulk_wait_read();
      }
    } else {
#pragma unroll 4
      for (uint32_t l = threadIdx.x; l < size; l += blockDim.x)
        s[base | offs[l >> L] | (l & lowmask)] = tile[l];
    }
    __syncthreads();
  }
  if (use_bulk && warp == 0) bulk_wait_all();
}

template <typename V, bool BULK, int NT, int MINB>
static int launch_tile_as(ev_state* s, uint64_t ntiles, size_t smem, const TilePlan* dplan,
                          const TileOp* dops, int nops, const uint8_t* pred) {
  EV_TRY(prepare_smem_kernel(reinterpret_cast<const void*>(k_tile<V, BULK, NT, MINB>)));
  int per_sm = 0;
  EV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<V, BULK, NT, MINB>, NT,
                                                        smem));
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = uint64_t(s->num_sms) * per_sm;
  if (grid > ntiles) grid = ntiles;
  ProfScope prof(s, P_TILE, 2.0 * double(s->len()) * double(sizeof(V)));
  s->launches += 1;
  int* derr = reinterpret_cast<int*>(s->scratch.counter + 1);
  k_tile<V, BULK, NT, MINB><<<unsigned(grid), NT, smem, s->stream>>>(
      static_cast<V*>(s->amps), ntiles, dplan, dops, nops, pred, derr);
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

template <typename V>
static int launch_tile(ev_state* s, uint64_t ntiles, const TilePlan& plan, const TilePlan* dplan,
                       const TileOp* dops, int nops, const uint8_t* pred) {
  const size_t ops_at = (sizeof(V) * (size_t(1) << plan.k) +
                         sizeof(uint64_t) * (size_t(1) << (plan.k - plan.L)) + 15) & ~size_t(15);
  const bool bulk = tile_bulk_enabled();
  const int shape = tile_shape();
  if (shape == 1 && !bulk)
    return launch_tile_as<V, false, 256, 3>(s, ntiles, ops_at + 64, dplan, dops, nops, pred);
  const size_t smem = ops_at + sizeof(TileOp) * size_t(nops) + 64;
  if (shape == 2 && !bulk)
    return launch_tile_as<V, false, kTileThreads, 1>(s, ntiles, smem, dplan, dops, nops, pred);
  if (bulk) return launch_tile_as<V, true, kTileThreads, 2>(s, ntiles, smem, dplan, dops, nops, pred);
  return launch_tile_as<V, false, kTileThreads, 2>(s, ntiles, smem, dplan, dops, nops, pred);
}

int default_tile_bits(int dtype) { return dtype == EV_C128 ? 12 : 13; }

// Plans a gate run into tile passes; plans and records go into the blob.
int plan_tiled(ev_state* s, const ev_circuit* c, uint64_t first, uint64_t last, int tile_bits,
               PlanBlob* blob, std::vector<SegStep>* out) {
  const int n = int(s->n);
  int k = tile_bits > 0 ? tile_bits : default_tile_bits(s->dtype);
  const int kcap = s->dtype == EV_C128 ? 13 : 14;  // tile + records within 227 KiB
  if (k > kcap) k = kcap;
  if (k < 2) k = 2;
  if (k > n) k = n;
  const int L = std::min(k, 4);
  // one op may need 2 data qubits beyond the low ones
  if (k - L < 2 && k < n) k = std::min(n, L + 2);
  // complex64 may reorder commuting ops; complex128 keeps the reference's order
  std::vector<Pass> passes =
      plan_passes(c, first, last, n, k, L, uint64_t(kMaxPassOps), s->dtype == EV_C64);
  const uint64_t ntiles = uint64_t(1) << (n - k);
  const SoftLevels soft = tile_soft_levels();
  const ChainSet chains = chain_set("EV_TILE_CHAIN", ChainSet{true, true, true});
  std::vector<TileOp> ops;
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
    ops.assign(p.ops.size(), TileOp{});
    for (size_t j = 0; j < p.ops.size(); ++j) {
      encode_op(c, c->ops[p.ops[j]], p.tset, local, &ops[j]);
      if (s->dtype == EV_C64) pack_f32_matrix(ops[j].m, ops[j].kind == T_1Q ? 8 : 32);
      if (s->dtype == EV_C128 && ops[j].kind == T_1Q)
        ops[j].soft = uint8_t(ops[j].k1 == K1_REAL ? soft.real : soft.other);
    }
    mark_chains(ops.data(), ops.size(), chains);
    SegStep st;
    st.fused = 0;
    st.off0 = blob->add(&plan, sizeof(plan));
    st.off1 = blob->add(ops.data(), ops.size() * sizeof(TileOp));
    st.nops = int(ops.size());
    st.k = k;
    st.L = L;
    st.count = ntiles;
    out->push_back(st);
  }
  return EV_OK;
}

int launch_tile_step(ev_state* s, const SegStep& st, const unsigned char* dblob) {
  TilePlan plan{};
  plan.k = st.k;
  plan.L = st.L;
  const TilePlan* dplan = reinterpret_cast<const TilePlan*>(dblob + st.off0);
  const TileOp* dops = reinterpret_cast<const TileOp*>(dblob + st.off1);
  if (s->dtype == EV_C128) return launch_tile<double2>(s, st.count, plan, dplan, dops, st.nops, nullptr);
  return launch_tile<float2>(s, st.count, plan, dplan, dops, st.nops, nullptr);
}

// ---- device check of the integer-pipe product ------------------------------------
// Operands drawn from five families that reach every rounding case (full
// random significands, short significands with exact products and ties,
// significands next to 1 and 2, the edges of the fast-path exponent range,
// amplitude-like magnitudes), all inside the fast path's domain.

__device__ __forceinline__ uint64_t check_next(uint64_t& st) {  // SplitMix64
  uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ double check_operand(uint64_t& st, int family) {
  const uint64_t sign = check_next(st) & 1, r = check_next(st), r2 = check_next(st);
  const uint64_t fmask = (1ull << 52) - 1;
  uint64_t exp = 512 + r2 % 1023, frac = r;
  if (family == 1) {
    const int k = 1 + int(r2 % 30);
    frac = (r >> (64 - k)) << (52 - k);
    exp = 512 + (r2 >> 8) % 1023;
  } else if (family == 2) {
    const uint64_t small = r >> (12 + (r2 >> 20) % 52);
    frac = (r2 & 1) ? small : (fmask - small);
    exp = 512 + (r2 >> 8) % 1023;
  } else if (family == 3) {
    const uint64_t edges[4] = {512, 513, 1533, 1534};
    exp = edges[r2 & 3];
    frac = (r2 & 4) ? r : fmask;
  } else if (family == 4) {
    exp = 1023 - r2 % 41;
  }
  return __longlong_as_double((long long)((sign << 63) | (exp << 52) | (frac & fmask)));
}

__global__ void k_softfp_check(uint64_t seed, uint64_t per_thread, unsigned long long* bad) {
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint64_t st = seed ^ (gid * 0xD1B54A32D192ED03ULL);
  unsigned long long mine = 0;
  for (uint64_t i = 0; i < per_thread; ++i) {
    const int fam = int((gid + i) % 25);
    const double a = check_operand(st, fam % 5), b = check_operand(st, fam / 5);
    const softfp::Unpacked ua = softfp::unpack(a), ub = softfp::unpack(b);
    const double got = softfp::mul(ua, ub), want = __dmul_rn(a, b);
    mine += (!(ua.ok & ub.ok)) || __double_as_longlong(got) != __double_as_longlong(want);
  }
  if (mine) atomicAdd(bad, mine);
}

// softfp::add against the FP64 add: first operands from the product check's
// families, second operands from the same families or made from the first
// (opposite sign with changed low bits: cancellation; exponent gaps of 50..66
// with a random or an empty fraction: the alignment's edges and exact ties).
__global__ void k_softadd_check(uint64_t seed, uint64_t per_thread, unsigned long long* bad) {
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint64_t st = seed ^ (gid * 0xA0761D6478BD642FULL);
  unsigned long long mine = 0;
  for (uint64_t i = 0; i < per_thread; ++i) {
    const int fam = int((gid + i) % 40);
    const double a = check_operand(st, fam % 5);
    const int fb = fam / 5;
    double b;
    if (fb < 5) {
      b = check_operand(st, fb);
    } else if (fb == 5) {
      const uint64_t r = check_next(st);
      const int k = int(r % 53);
      const uint64_t flip = k ? (check_next(st) & ((1ull << k) - 1)) : 0;
      b = __longlong_as_double((long long)((uint64_t(__double_as_longlong(a)) ^ flip) ^ (1ull << 63)));
    } else {
      const uint64_t r = check_next(st), ua = uint64_t(__double_as_longlong(a));
      const uint64_t ea = (ua >> 52) & 0x7FF, gap = 50 + r % 17;
      const uint64_t eb = ea < 512 + gap ? 512 : ea - gap;
      const uint64_t frac = fb == 6 ? (check_next(st) & ((1ull << 52) - 1)) : 0;
      b = __longlong_as_double((long long)(((r >> 40) & 1) << 63 | eb << 52 | frac));
    }
    const double got = softfp::add(a, b), want = __dadd_rn(a, b);
    mine += (!softfp::add_ok(a, b)) || __double_as_longlong(got) != __double_as_longlong(want);
  }
  if (mine) atomicAdd(bad, mine);
}

// ff_to_f64 (ev_device.cuh) against the FP64 add of the pair's two exact
// f64 values, on renormalised double-float pairs (TwoSum of random floats
// whose exponents differ by 0..80, with ties and cancellations).
__global__ void k_ff_check(uint64_t seed, uint64_t per_thread, unsigned long long* bad) {
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint64_t st = seed ^ (gid * 0x9E3779B97F4A7C15ULL);
  unsigned long long mine = 0;
  for (uint64_t i = 0; i < per_thread; ++i) {
    const uint64_t r0 = check_next(st), r1 = check_next(st), r2 = check_next(st);
    const uint32_t ea = 1 + uint32_t(r0 % 253), gap = uint32_t((r0 >> 8) % 81);
    const uint32_t eb = ea > gap ? ea - gap : 1;
    uint32_t fa = uint32_t(r1) & 0x7FFFFFu, fb = uint32_t(r1 >> 32) & 0x7FFFFFu;
    if ((r2 & 7) == 0) fb = (r2 & 8) ? 0u : 0x400000u;  // short significands: ties
    const float a = __uint_as_float(uint32_t(r2 >> 63) << 31 | ea << 23 | fa);
    const float b = __uint_as_float(uint32_t((r2 >> 62) & 1) << 31 | eb << 23 | fb);
    FF f;
    f.add(a);
    f.add(b);
    const double got = ff_to_f64(f.hi, f.lo), want = f2d_exact(f.hi) + f2d_exact(f.lo);
    mine += __double_as_longlong(got) != __double_as_longlong(want);
  }
  if (mine) atomicAdd(bad, mine);
}

}  // namespace ev

extern "C" int ev_ff_check(uint64_t seed, uint64_t count, uint64_t* mismatches) {
  using namespace ev;
  clear_error();
  if (!mismatches) return fail(EV_ERR_INVALID_ARGUMENT, "ev_ff_check: null output");
  int dev = 0, sms = 0;
  EV_CUDA(cudaGetDevice(&dev));
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t threads = uint64_t(sms) * 4 * 256;
  const uint64_t per = (count + threads - 1) / threads;
  unsigned long long* d = nullptr;
  EV_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), sizeof(*d)));
  int rc = EV_OK;
  unsigned long long h = 0;
  if (cudaMemset(d, 0, sizeof(*d)) != cudaSuccess) {
    rc = fail(EV_ERR_CUDA, "ev_ff_check: memset failed");
  } else {
    k_ff_check<<<unsigned(sms * 4), 256>>>(seed, per, d);
    if (cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(EV_ERR_CUDA, "ev_ff_check: kernel failed");
  }
  cudaFree(d);
  if (rc == EV_OK) *mismatches = h;
  return rc;
}

static int run_soft_check(const char* name, void (*kernel)(uint64_t, uint64_t, unsigned long long*),
                          uint64_t seed, uint64_t count, uint64_t* mismatches) {
  using namespace ev;
  if (!mismatches) return fail(EV_ERR_INVALID_ARGUMENT, "%s: null output", name);
  int dev = 0, sms = 0;
  EV_CUDA(cudaGetDevice(&dev));
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t threads = uint64_t(sms) * 4 * 256;
  const uint64_t per = (count + threads - 1) / threads;
  unsigned long long* d = nullptr;
  EV_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), sizeof(*d)));
  int rc = EV_OK;
  unsigned long long h = 0;
  if (cudaMemset(d, 0, sizeof(*d)) != cudaSuccess) {
    rc = fail(EV_ERR_CUDA, "%s: memset failed", name);
  } else {
    kernel<<<unsigned(sms * 4), 256>>>(seed, per, d);
    if (cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(EV_ERR_CUDA, "%s: kernel failed", name);
  }
  cudaFree(d);
  if (rc == EV_OK) *mismatches = h;
  return rc;
}

extern "C" int ev_softfp_add_check(uint64_t seed, uint64_t count, uint64_t* mismatches) {
  ev::clear_error();
  return run_soft_check("ev_softfp_add_check", ev::k_softadd_check, seed, count, mismatches);
}

extern "C" int ev_softfp_check(uint64_t seed, uint64_t count, uint64_t* mismatches) {
  using namespace ev;
  clear_error();
  if (!mismatches) return fail(EV_ERR_INVALID_ARGUMENT, "ev_softfp_check: null output");
  int dev = 0, sms = 0;
  EV_CUDA(cudaGetDevice(&dev));
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t threads = uint64_t(sms) * 4 * 256;
  const uint64_t per = (count + threads - 1) / threads;
  unsigned long long* d = nullptr;
  EV_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), sizeof(*d)));
  int rc = EV_OK;
  unsigned long long h = 0;
  if (cudaMemset(d, 0, sizeof(*d)) != cudaSuccess) {
    rc = fail(EV_ERR_CUDA, "ev_softfp_check: memset failed");
  } else {
    k_softfp_check<<<unsigned(sms * 4), 256>>>(seed, per, d);
    if (cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(EV_ERR_CUDA, "ev_softfp_check: kernel failed");
  }
  cudaFree(d);
  if (rc == EV_OK) *mismatches = h;
  return rc;
}
