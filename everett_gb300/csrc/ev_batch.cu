// ev_batch.cu -- many independent circuits in one persistent launch over a
// device work queue.
//
// Each circuit (gate records only) runs from |0...0> and ends with <Z_0>
// and full-register shots.  The host plans every circuit with the tile
// planner and lays out a work queue:
//   BI_WHOLE  a circuit of at most k qubits: its whole state lives in one
//             CTA's shared memory; the CTA applies every record, then
//             computes <Z_0>, the sampling tree and the shots
//   BI_TILE   (circuit, pass, tile) of a larger circuit whose state lives in
//             HBM (L2-resident at these sizes); the item waits until every
//             tile of the previous pass of its circuit is done (a per-circuit
//             completion counter), loads its tile, applies the pass's records
//             and stores it back
//   BI_FINAL  <Z_0>, tree and shots of a larger circuit once all its passes
//             are done
// Items are claimed in queue order by persistent CTAs (atomic head); an item
// only ever waits for items earlier in the queue, all CTAs are resident, so
// the queue always drains.  Waits are bounded: a wait that gives up sets an
// error flag and the host reports EV_ERR_TIMEOUT.  State loads and stores of
// BI_TILE items bypass L1 (other CTAs wrote the data).
//
// Per-amplitude arithmetic is the tile pass's (ev_tile.cuh), so a batched
// circuit's state equals the single-circuit tiled run bit for bit, and its
// shots are drawn exactly as ev_sample draws them (same tree, same uniforms).
//
// Circuits with mid-circuit measurement and classical control
// (backend/mod.rs:51-72) run as BI_WHOLE items: the CTA walks the ops in
// order with the classical register in shared memory; an IfClassic prefix
// gates the op after it; a measurement sums p1 over the tile with a fixed
// block tree, draws its uniform from the circuit's own Rng
// (Rng::seed_from_u64(run_seed), one uniform per executed measurement, as
// measure.rs:15-51 does), decides, collapses and renormalises in shared
// memory.  Such circuits must fit one CTA (n <= the tile size).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <sys/stat.h>

#include "ev_tile.cuh"

namespace ev {

struct BatchOp {
  uint8_t kind, k1, p0, p1, lo, hi, nins, soft;  // as TileOp (soft is 0 here)
  uint8_t run, ctype;                            // chains, as TileOp
  uint16_t lmask;  // local control mask (tiles of at most 16 qubits), or a classical bit
  uint32_t mat;    // offset of the matrix in the pool (doubles)
  uint64_t emask;
  uint64_t ins;
};
static_assert(sizeof(BatchOp) == 32, "compact op record");
__device__ __forceinline__ const double* rec_m(const BatchOp& op, const double* mats) {
  return mats + op.mat;
}
__device__ __forceinline__ uint32_t rec_sok(const BatchOp&) { return 0; }

// Records staged in shared memory at a time, at most (the window is sized at
// launch from the shared memory the block has left).
constexpr uint32_t kMaxWindow = 32;

// A staged matrix slot, in doubles: a 4x4 complex matrix (complex64 records
// hold f32 pairs, pack_f32_matrix).
template <typename V>
__host__ __device__ constexpr uint32_t mat_slot_doubles() {
  return sizeof(V) == 16 ? 32 : 16;
}

// The 16-byte words of a record's matrix that its kernel reads.
template <typename V>
__device__ __forceinline__ uint32_t mat_words(uint8_t kind) {
  constexpr uint32_t full = mat_slot_doubles<V>() / 2;
  if (kind == T_1Q) return full / 4;  // 2x2
  if (kind == T_DIAG2 || kind == T_DENSE2) return full;
  return 0;  // permutations, CZ, measurements, IfClassic prefixes
}

struct BatchCirc {
  uint32_t n, k, npasses, pad;
  uint32_t plan0, pass0;
  uint64_t ntiles;
  uint64_t state, tree, uni, shots, shot_out, seed;
  uint64_t run_seed;  // Rng of mid-circuit measurements
  uint64_t cl;        // offset of the classical register in the results
  uint32_t ncl;       // classical bits
  uint32_t classical; // 1: the circuit measures or has classical control
};

// Batch-only op kinds (beside the tile kinds of ev_tile.cuh): a measurement
// (p0 = qubit, lmask = classical bit) and an IfClassic prefix (lmask =
// classical bit) that gates the next op.
constexpr uint8_t B_MEAS = 200, B_IF = 201;
constexpr int kBatchMaxClassical = 64;

struct PassRef {
  uint32_t op0, nops;
};

enum : uint32_t { BI_WHOLE = 0, BI_TILE = 1, BI_FINAL = 2, BI_STALL = 3 };
struct BatchItem {
  uint32_t circ, pass, tile, kind;
};

struct BatchArgs {
  void* states;
  double* trees;
  double* uni;
  uint64_t* shots;
  double* expz;
  const BatchCirc* circs;
  const BatchItem* items;
  uint64_t nitems;
  const PassRef* passes;
  const TilePlan* plans;
  const BatchOp* ops;
  const double* mats;
  uint32_t window;  // records staged in shared memory at a time (BatchWindow)
  unsigned* head;
  unsigned* done;
  int* err;
  uint8_t* cl;
};

constexpr uint32_t kSpinLimit = 1u << 25;  // x ~64 ns: a wait gives up after ~2 s

__device__ bool wait_count(const unsigned* ctr, unsigned want) {
  for (uint32_t it = 0; it < kSpinLimit; ++it) {
    if (*reinterpret_cast<const volatile unsigned*>(ctr) >= want) {
      __threadfence();
      return true;
    }
    __nanosleep(64);
  }
  return false;
}

template <typename V>
__device__ __forceinline__ V ld_amp(const V* p, bool global) {
  if (global) {
    if constexpr (sizeof(V) == 16) {
      const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
      return v;
    } else {
      const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
      return v;
    }
  }
  return *p;
}

// Block-wide sum of two doubles (fixed tree shape).
__device__ void block_sum2(double* red, double& x, double& y) {
  const int t = threadIdx.x, nb = blockDim.x;
  red[t] = x;
  red[nb + t] = y;
  __syncthreads();
  for (int w = nb / 2; w > 0; w >>= 1) {
    if (t < w) {
      red[t] += red[t + w];
      red[nb + t] += red[nb + t + w];
    }
    __syncthreads();
  }
  x = red[0];
  y = red[nb];
  __syncthreads();
}

// <Z_0>, sampling tree (level q at offset 2^q, as ev_sample builds it)
// and shots of one circuit whose amplitudes are at `amps` (shared memory or
// HBM).
template <typename V>
__device__ void finalize(const V* amps, bool global, const BatchCirc& c, uint32_t ci, double* red,
                         const BatchArgs& a) {
  const int t = threadIdx.x, nb = blockDim.x;
  const uint64_t N = uint64_t(1) << c.n, half = N / 2;
  double r0 = 0.0, r1 = 0.0;
  for (uint64_t j = t; j < N; j += nb) {
    const double p = nsq(ld_amp(amps + j, global));
    if (j & 1)
      r1 += p;
    else
      r0 += p;
  }
  block_sum2(red, r0, r1);
  if (t == 0) a.expz[ci] = (r0 - r1) / (r0 + r1);
  double* tr = a.trees + c.tree;
  for (uint64_t r = t; r < half; r += nb)
    __stcg(tr + half + r,
           __dadd_rn(nsq(ld_amp(amps + r, global)), nsq(ld_amp(amps + r + half, global))));
  __syncthreads();
  for (int q = int(c.n) - 2; q >= 0; --q) {
    const uint64_t w = uint64_t(1) << q;
    for (uint64_t r = t; r < w; r += nb)
      __stcg(tr + w + r, __dadd_rn(__ldcg(tr + 2 * w + r), __ldcg(tr + 2 * w + r + w)));
    __syncthreads();
  }
  const int n = int(c.n);
  for (uint64_t s = t; s < c.shots; s += nb) {
    uint64_t r = 0;
    for (int q = 0; q < n; ++q) {
      const uint64_t w = uint64_t(1) << q;
      const double m = __ldcg(tr + w + r);
      const double m1 = (q + 1 < n) ? __ldcg(tr + 2 * w + r + w) : nsq(ld_amp(amps + r + w, global));
      const double p1 = __ddiv_rn(m1, m);
      if (a.uni[c.uni + s * uint64_t(n) + q] < p1) r |= w;
    }
    a.shots[c.shot_out + s] = r;
  }
}

// Rescaling by the f64 factor of a measurement: complex128 in f64
// (Complex64 * f64, complex.rs:127-133); complex64 as a float pair in one FMA
// per component, as the single-state collapse does.
template <typename V>
__device__ __forceinline__ V batch_scale(V a, double s) {
  if constexpr (sizeof(V) == 16) {
    return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s));
  } else {
    const float sh = float(s);
    const float sl = float(s - double(sh));
    return make_float2(__fmaf_rn(a.x, sh, __fmul_rn(a.x, sl)), __fmaf_rn(a.y, sh, __fmul_rn(a.y, sl)));
  }
}

// measure_qubit (measure.rs:15-51) on a whole state in shared memory: p1 by
// a fixed block tree, the outcome from the circuit's next uniform, then the
// collapse and rescale.  rng holds the circuit's xoshiro256++ state.
template <typename V>
__device__ void batch_measure(V* tile, uint32_t size, int q, uint32_t cbit, double* red,
                              uint8_t* cl, uint64_t* rng, double* meas) {
  const int t = threadIdx.x, nb = blockDim.x;
  const uint32_t bit = 1u << q;
  double p1 = 0.0, unused = 0.0;
  for (uint32_t j = t; j < size; j += nb)
    if (j & bit) p1 += nsq(tile[j]);
  block_sum2(red, p1, unused);
  if (t == 0) {
    DevRng r(0);
    for (int w = 0; w < 4; ++w) r.s[w] = rng[w];
    const double u = r.next_f64();
    for (int w = 0; w < 4; ++w) rng[w] = r.s[w];
    const bool outcome = u < p1;
    const double surviving = outcome ? p1 : __dadd_rn(1.0, -p1);
    meas[0] = surviving > 0.0 ? __ddiv_rn(1.0, __dsqrt_rn(surviving)) : 0.0;
    meas[1] = outcome ? 1.0 : 0.0;
    cl[cbit] = outcome ? 1 : 0;
  }
  __syncthreads();
  const double scale = meas[0];
  const bool one = meas[1] != 0.0;
  V zero;
  zero.x = 0;
  zero.y = 0;
  for (uint32_t j = t; j < size; j += nb)
    tile[j] = (((j & bit) != 0) == one) ? batch_scale(tile[j], scale) : zero;
  __syncthreads();
}

// Compiled per block size: 256-thread CTAs, three of which fit an SM's
// shared memory with the default tile, get 80 registers a thread; 512-thread
// CTAs (two per SM) 64.
template <typename V, int NT>
__global__ void __launch_bounds__(NT, NT == 256 ? 3 : 2) k_batch(BatchArgs a, int kmax) {
  extern __shared__ __align__(16) unsigned char sm[];
  V* tile = reinterpret_cast<V*>(sm);
  uint64_t* offs = reinterpret_cast<uint64_t*>(sm + (sizeof(V) << kmax));
  double* red = reinterpret_cast<double*>(offs + (size_t(1) << (kmax > 4 ? kmax - 4 : 0)));
  // staged records and their matrices: [window records][window slots]
  const size_t stage_at = (reinterpret_cast<size_t>(red + 2 * blockDim.x) + 15) & ~size_t(15);
  BatchOp* srec = reinterpret_cast<BatchOp*>(stage_at);
  double* smat = reinterpret_cast<double*>(srec + a.window);
  constexpr uint32_t kSlot = mat_slot_doubles<V>();
  __shared__ uint32_t s_matoff[kMaxWindow];
  __shared__ TilePlan plan;
  __shared__ unsigned s_item;
  __shared__ int s_ok;
  __shared__ uint8_t s_cl[kBatchMaxClassical];
  __shared__ uint64_t s_rng[4];
  __shared__ double s_meas[2];
  const int t = threadIdx.x, nb = blockDim.x;
  for (;;) {
    if (t == 0) s_item = atomicAdd(a.head, 1u);
    __syncthreads();
    const unsigned i = s_item;
    if (i >= a.nitems) break;
    const BatchItem it = a.items[i];
    const BatchCirc c = a.circs[it.circ];
    V* st = static_cast<V*>(a.states) + c.state;
    if (it.kind != BI_WHOLE && !(it.kind == BI_TILE && it.pass == 0)) {
      // BI_STALL (test hook) waits for a count no item ever reaches
      const unsigned want = it.kind == BI_STALL  ? 0xFFFFFFFFu
                            : it.kind == BI_FINAL ? c.npasses * unsigned(c.ntiles)
                                                  : it.pass * unsigned(c.ntiles);
      if (t == 0) {
        s_ok = wait_count(a.done + it.circ, want) ? 1 : 0;
        if (!s_ok) atomicExch(a.err, 1);
      }
      __syncthreads();
      if (!s_ok) continue;
    }
    if (it.kind == BI_FINAL) {
      finalize(st, true, c, it.circ, red, a);
      __syncthreads();
      continue;
    }
    // load the pass's plan and row offsets
    if (t < int(sizeof(TilePlan) / 4))
      reinterpret_cast<uint32_t*>(&plan)[t] = reinterpret_cast<const uint32_t*>(a.plans + c.plan0 + it.pass)[t];
    __syncthreads();
    const int k = plan.k, L = plan.L;
    const uint32_t size = 1u << k, nrows = 1u << (k - L), lowmask = (1u << L) - 1;
    for (uint32_t h = t; h < nrows; h += nb) {
      uint64_t o = 0;
      for (int b = 0; b < plan.nH; ++b)
        if ((h >> b) & 1) o |= uint64_t(1) << plan.H[b];
      offs[h] = o;
    }
    uint64_t base = 0;
    for (int b = 0; b < plan.ncomp; ++b)
      if ((uint64_t(it.tile) >> b) & 1) base |= uint64_t(1) << plan.comp[b];
    __syncthreads();
    if (it.pass == 0) {
      V z;
      z.x = 0;
      z.y = 0;
      for (uint32_t l = t; l < size; l += nb) tile[l] = z;
      if (t == 0 && base == 0) tile[0].x = 1;
    } else {
      for (uint32_t l = t; l < size; l += nb) tile[l] = ld_amp(st + (base | offs[l >> L] | (l & lowmask)), true);
    }
    __syncthreads();
    const PassRef pr = a.passes[c.pass0 + it.pass];
    const bool classical = c.classical != 0;  // BI_WHOLE items only
    if (classical) {
      if (t < kBatchMaxClassical) s_cl[t] = 0;
      if (t == 0) {
        const DevRng r(c.run_seed);
        for (int w = 0; w < 4; ++w) s_rng[w] = r.s[w];
      }
      __syncthreads();
    }
    bool take = true;  // the IfClassic prefixes read so far hold
    for (uint32_t o = 0; o < pr.nops;) {
      // stage the next window of records and their matrices (records point
      // at their slot, smat + j * kSlot); a chain never spans more records
      // than a window holds
      const uint32_t cnt = min(a.window, pr.nops - o);
      __syncthreads();  // the previous window is no longer read
      for (uint32_t w = t; w < 2 * cnt; w += nb) {
        uint4 v = reinterpret_cast<const uint4*>(a.ops + pr.op0 + o)[w];
        if ((w & 1) == 0) {  // the first half holds BatchOp::mat (bytes 12..15)
          s_matoff[w >> 1] = v.w;
          v.w = (w >> 1) * kSlot;
        }
        reinterpret_cast<uint4*>(srec)[w] = v;
      }
      __syncthreads();
      for (uint32_t w = t; w < cnt * (kSlot / 2); w += nb) {
        const uint32_t j = w / (kSlot / 2), x = w % (kSlot / 2);
        if (x < mat_words<V>(srec[j].kind))
          reinterpret_cast<uint4*>(smat + j * kSlot)[x] =
              reinterpret_cast<const uint4*>(a.mats + s_matoff[j])[x];
      }
      __syncthreads();
      uint32_t j = 0;
      while (j < cnt) {
        const BatchOp* rec = srec + j;
        const BatchOp op = *rec;
        // chains (run > 1) are formed only in circuits without classical ops
        const uint32_t run = op.run > 1 ? op.run : 1;
        if (j + run > cnt) break;  // the next window starts at this chain
        j += run;
        if (op.kind == B_IF) {
          take = take && s_cl[op.lmask] != 0;
          continue;
        }
        const bool go = take;
        take = true;
        if (!go) continue;
        if (op.kind == B_MEAS) {
          batch_measure(tile, size, op.p0, op.lmask, red, s_cl, s_rng, s_meas);
          continue;
        }
        if ((base & op.emask) != op.emask) continue;
        if (run > 1 && op.ctype == CH_QUAD)
          tile_quad_chain(tile, size, rec, int(run), smat);
        else if (run > 1 && op.ctype == CH_DIAG)
          tile_diag_chain(tile, size, rec, int(run), smat);
        else if (run > 1)
          tile_chain(tile, size >> op.nins, rec, int(run), smat);
        else
          apply_tile_op(tile, k, op, smat + op.mat);
        __syncthreads();
      }
      if (j == 0) {  // cannot happen (runs are capped at the window): stop cleanly
        if (t == 0) atomicExch(a.err, 1);
        break;
      }
      o += j;
    }
    if (classical && t < int(c.ncl)) a.cl[c.cl + t] = s_cl[t];
    for (uint32_t l = t; l < size; l += nb) {
      V* p = st + (base | offs[l >> L] | (l & lowmask));
      if constexpr (sizeof(V) == 16)
        __stcg(reinterpret_cast<double2*>(p), tile[l]);
      else
        __stcg(reinterpret_cast<float2*>(p), tile[l]);
    }
    if (it.kind == BI_WHOLE) {
      finalize(tile, false, c, it.circ, red, a);
    } else {
      __threadfence();
      __syncthreads();
      if (t == 0) atomicAdd(a.done + it.circ, 1u);
    }
    __syncthreads();
  }
}

__global__ void k_batch_uniforms(const BatchCirc* __restrict__ circs, uint64_t count,
                                 double* __restrict__ uni) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const BatchCirc c = circs[i];
  DevRng r(c.seed);
  const uint64_t total = c.shots * c.n;
  for (uint64_t j = 0; j < total; ++j) uni[c.uni + j] = r.next_f64();
}

// ---- host --------------------------------------------------------------------

namespace {

struct Arena {
  std::mutex mu;
  int device = -1;
  void* dmeta = nullptr;
  size_t meta_cap = 0;
  void* dpool = nullptr;  // states | trees | uniforms | shots | expz | done | head | err
  size_t pool_cap = 0;
  void* hstage = nullptr;  // pinned staging (meta up, results down)
  size_t stage_cap = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};
// Arenas are leased one per concurrent call, so batched launches from
// different host threads (the serving workers) run side by side on their own
// streams instead of queueing on one arena.  Queue items wait only on earlier
// items, which CTAs already running have taken, so kernels sharing the GPU
// always drain.
struct ArenaPool {
  std::mutex mu;
  std::vector<Arena*> free_list;
};
ArenaPool g_pool;

Arena* acquire_arena(int dev) {
  std::lock_guard<std::mutex> lock(g_pool.mu);
  for (size_t i = 0; i < g_pool.free_list.size(); ++i)
    if (g_pool.free_list[i]->device == dev) {
      Arena* a = g_pool.free_list[i];
      g_pool.free_list.erase(g_pool.free_list.begin() + long(i));
      return a;
    }
  Arena* a = new Arena();
  a->device = dev;
  return a;
}

struct ArenaLease {
  Arena* a;
  ~ArenaLease() {
    std::lock_guard<std::mutex> lock(g_pool.mu);
    g_pool.free_list.push_back(a);
  }
};

std::mutex g_cache_mu;  // the tuning cache file

int grow_dev(void** p, size_t* cap, size_t need) {
  if (*cap >= need) return EV_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = need + need / 4;
  if (cudaMalloc(p, sz) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(EV_ERR_OOM, "batch: cannot allocate %zu bytes of device memory", sz);
  }
  *cap = sz;
  return EV_OK;
}

int grow_host(void** p, size_t* cap, size_t need) {
  if (*cap >= need) return EV_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = need + need / 4;
  if (cudaMallocHost(p, sz) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(EV_ERR_OOM, "batch: cannot allocate %zu bytes of pinned host memory", sz);
  }
  *cap = sz;
  return EV_OK;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Per-circuit host plan.
struct CircPlan {
  int n = 0, k = 0;
  bool classical = false;
  std::vector<TilePlan> plans;
  std::vector<PassRef> passes;  // op0 relative to this circuit's ops
  std::vector<BatchOp> ops;
  std::vector<double> mats;     // this circuit's matrix pool
  int rc = EV_OK;
};

struct MatKey {
  size_t h;
  bool operator==(const MatKey& o) const { return h == o.h; }
};

bool has_classical_ops(const ev_circuit* c) {
  for (uint64_t j = 0; j < c->nops; ++j)
    if (c->ops[j].kind == EV_OP_MEASURE || c->ops[j].kind == EV_OP_IF) return true;
  return false;
}

void plan_circuit(const ev_circuit* c, int kmax, bool c64, uint32_t window, CircPlan* out) {
  const bool reorder = c64;  // complex64 may reorder commuting ops
  const int n = int(c->num_qubits);
  out->n = n;
  const int k = n <= kmax ? n : kmax;
  out->k = k;
  const int L = std::min(k, 4);
  out->classical = has_classical_ops(c);
  std::vector<Pass> passes;
  if (out->classical) {
    // one whole-state pass with every op in circuit order (the caller has
    // checked n <= kmax); measurements and IfClassic prefixes stay in place
    Pass p;
    for (uint64_t j = 0; j < c->nops; ++j) p.ops.push_back(j);
    p.tset = (uint64_t(1) << n) - 1;
    passes.push_back(std::move(p));
  } else {
    passes = plan_passes(c, 0, c->nops, n, k, L, ~uint64_t(0), reorder);
  }
  // every circuit gets at least one pass: pass 0 is what writes |0...0>
  if (passes.empty()) passes.push_back({{}, (uint64_t(1) << k) - 1});
  std::unordered_map<size_t, std::vector<uint32_t>> seen;  // hash -> offsets
  std::vector<TileOp> recs;
  // diagonal chains by default: with the records staged in shared memory,
  // pair and quad chains measured no faster on the TFIM batch (4096
  // circuits: none 687, diagonal 673, pair and quad 700, all 677 ms)
  const ChainSet chains = chain_set("EV_BATCH_CHAIN", ChainSet{false, false, true});
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
    out->plans.push_back(plan);
    out->passes.push_back({uint32_t(out->ops.size()), uint32_t(p.ops.size())});
    // the pass's gate records, chained as the tile pass chains them (not in
    // circuits with measurements or classical control, whose records run one
    // by one in the classical register's order)
    recs.assign(p.ops.size(), TileOp{});
    for (size_t j = 0; j < p.ops.size(); ++j) {
      const ev_op& src = c->ops[p.ops[j]];
      if (src.kind != EV_OP_MEASURE && src.kind != EV_OP_IF) encode_op(c, src, p.tset, local, &recs[j]);
    }
    if (!out->classical) mark_chains(recs.data(), recs.size(), chains, window);
    for (size_t jj = 0; jj < p.ops.size(); ++jj) {
      const ev_op& src = c->ops[p.ops[jj]];
      if (src.kind == EV_OP_MEASURE || src.kind == EV_OP_IF) {
        BatchOp b{};
        b.kind = src.kind == EV_OP_MEASURE ? B_MEAS : B_IF;
        b.p0 = uint8_t(src.kind == EV_OP_MEASURE ? src.q0 : 0);
        b.lmask = uint16_t(src.kind == EV_OP_MEASURE ? src.q1 : src.q0);
        out->ops.push_back(b);
        continue;
      }
      TileOp& tmp = recs[jj];
      if (c64) pack_f32_matrix(tmp.m, tmp.kind == T_1Q ? 8 : 32);
      BatchOp b;
      b.kind = tmp.kind;
      b.k1 = tmp.k1;
      b.p0 = tmp.p0;
      b.p1 = tmp.p1;
      b.lo = tmp.lo;
      b.hi = tmp.hi;
      b.nins = tmp.nins;
      b.soft = 0;
      b.run = tmp.run;
      b.ctype = tmp.ctype;
      b.lmask = uint16_t(tmp.lmask);
      b.emask = tmp.emask;
      b.ins = tmp.ins;
      const int nd = tmp.kind == T_1Q ? 8 : 32;
      const size_t h = std::hash<std::string>()(std::string(reinterpret_cast<const char*>(tmp.m), nd * 8));
      uint32_t off = UINT32_MAX;
      auto itr = seen.find(h);
      if (itr != seen.end())
        for (uint32_t cand : itr->second)
          if (std::memcmp(out->mats.data() + cand, tmp.m, nd * 8) == 0) {
            off = cand;
            break;
          }
      if (off == UINT32_MAX) {
        off = uint32_t(out->mats.size());
        out->mats.insert(out->mats.end(), tmp.m, tmp.m + nd);
        seen[h].push_back(off);
      }
      b.mat = off;
      out->ops.push_back(b);
    }
  }
}

// ---- autotuning cache --------------------------------------------------------

std::string cache_path() {
  if (const char* p = getenv("EV_AUTOTUNE_CACHE")) return p;
  if (const char* x = getenv("XDG_CACHE_HOME")) return std::string(x) + "/everett_gb300_autotune.txt";
  if (const char* h = getenv("HOME")) return std::string(h) + "/.cache/everett_gb300_autotune.txt";
  return "everett_gb300_autotune.txt";
}

std::string batch_key(const ev_batch_circuit* items, uint64_t count, int dtype) {
  // (amplitude type, qubit-count histogram in 4-qubit buckets, share of
  // 2-qubit records in tenths)
  int hist[16] = {0};
  uint64_t ops = 0, two = 0;
  for (uint64_t i = 0; i < count; ++i) {
    const ev_circuit& c = items[i].circuit;
    hist[std::min<uint64_t>(15, c.num_qubits / 4)]++;
    for (uint64_t j = 0; j < c.nops; ++j) {
      ++ops;
      if (c.ops[j].kind == EV_OP_APPLY2 || c.ops[j].kind == EV_OP_CONTROLLED) ++two;
    }
  }
  std::ostringstream k;
  k << (dtype == EV_C128 ? "c128" : "c64") << ":n";
  for (int b = 0; b < 16; ++b)
    if (hist[b]) k << b * 4 << "-" << b * 4 + 3 << "x" << (hist[b] * 10 + int(count) / 2) / int(count) << ",";
  k << ":2q" << (ops ? (two * 10 + ops / 2) / ops : 0);
  return k.str();
}

bool cache_lookup(const std::string& key, int* kbits, int* threads) {
  std::ifstream f(cache_path());
  std::string k;
  int a, b;
  while (f >> k >> a >> b)
    if (k == key) {
      *kbits = a;
      *threads = b;
      return true;
    }
  return false;
}

void cache_store(const std::string& key, int kbits, int threads) {
  const std::string path = cache_path();
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos && slash > 0) mkdir(path.substr(0, slash).c_str(), 0755);
  std::ofstream f(path, std::ios::app);
  if (f) f << key << " " << kbits << " " << threads << "\n";
}

// Tile sizes: the default fits two 512-thread CTAs per SM; the maximum one
// CTA with a 128 KiB tile.
int default_tile_bits_batch(int dtype) { return dtype == EV_C128 ? 12 : 13; }
int max_tile_bits(int dtype) { return dtype == EV_C128 ? 13 : 14; }

}  // namespace

// Runs one configuration; fills stats (device_ms, host_ms, items).
static int batch_once(Arena& A, const ev_batch_circuit* items, uint64_t count, int dtype, int kmax,
                      int threads, ev_batch_stats* st, bool stall = false) {
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  const int dev = A.device;
  if (!A.stream) {
    EV_CUDA(cudaStreamCreateWithFlags(&A.stream, cudaStreamNonBlocking));
    EV_CUDA(cudaEventCreate(&A.e0));
    EV_CUDA(cudaEventCreate(&A.e1));
  }
  int sms = 0;
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t ab = dtype == EV_C128 ? 16 : 8;
  // shared memory: tile | row offsets | reduction scratch | staged records
  // and matrices.  The record window is as large as fits without costing a
  // resident CTA (at least 4 records).
  const void* kfn = dtype == EV_C128
                        ? (threads == 256 ? reinterpret_cast<const void*>(k_batch<double2, 256>)
                                          : reinterpret_cast<const void*>(k_batch<double2, 512>))
                        : (threads == 256 ? reinterpret_cast<const void*>(k_batch<float2, 256>)
                                          : reinterpret_cast<const void*>(k_batch<float2, 512>));
  EV_TRY(prepare_smem_kernel(kfn));
  const size_t smem_base =
      ((ab << kmax) + (size_t(8) << (kmax > 4 ? kmax - 4 : 0)) + 2 * size_t(threads) * 8 + 15) &
      ~size_t(15);
  const size_t per_rec = sizeof(BatchOp) + 8 * size_t(dtype == EV_C128 ? mat_slot_doubles<double2>()
                                                                      : mat_slot_doubles<float2>());
  int per_sm = 0;
  EV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, threads, smem_base + 4 * per_rec));
  if (per_sm < 1) return fail(EV_ERR_INVALID_ARGUMENT, "batch: configuration does not fit an SM");
  uint32_t window = 4;
  for (uint32_t w = kMaxWindow; w > 4; w -= 4) {
    int fit = 0;
    EV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kfn, threads, smem_base + w * per_rec));
    if (fit >= per_sm) {
      window = w;
      break;
    }
  }
  const size_t smem = smem_base + window * per_rec;
  for (uint64_t i = 0; i < count; ++i)
    if (int(items[i].circuit.num_qubits) > kmax && has_classical_ops(&items[i].circuit))
      return fail(EV_ERR_INVALID_ARGUMENT,
                  "batch circuit %llu: measurement and classical control in a batch need a "
                  "circuit of at most %d qubits (the tile size); it has %llu",
                  (unsigned long long)i, kmax,
                  (unsigned long long)items[i].circuit.num_qubits);
  // plan all circuits (in parallel)
  std::vector<CircPlan> cp(count);
  {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < hw; ++w)
      pool.emplace_back([&, w] {
        for (uint64_t i = w; i < count; i += hw)
          plan_circuit(&items[i].circuit, kmax, dtype == EV_C64, window, &cp[i]);
      });
    for (auto& th : pool) th.join();
  }
  // layout
  std::vector<BatchCirc> circs(count);
  uint64_t amps = 0, tree = 0, uni = 0, shots = 0, nplans = 0, nops = 0, nmats = 0, ncl = 0;
  for (uint64_t i = 0; i < count; ++i) {
    BatchCirc& b = circs[i];
    const CircPlan& p = cp[i];
    b.n = uint32_t(p.n);
    b.k = uint32_t(p.k);
    b.npasses = uint32_t(p.passes.size());
    b.ntiles = uint64_t(1) << (p.n - p.k);
    b.plan0 = uint32_t(nplans);
    b.pass0 = uint32_t(nplans);
    b.state = amps;
    b.tree = tree;
    b.uni = uni;
    b.shots = items[i].shots;
    b.shot_out = shots;
    b.seed = items[i].seed;
    b.run_seed = items[i].run_seed;
    b.cl = ncl;
    b.ncl = uint32_t(items[i].circuit.num_classical);
    b.classical = p.classical ? 1u : 0u;
    ncl += items[i].circuit.num_classical;
    amps += uint64_t(1) << p.n;
    tree += uint64_t(1) << p.n;
    uni += items[i].shots * uint64_t(p.n);
    shots += items[i].shots;
    nplans += p.plans.size();
    nops += p.ops.size();
    nmats += p.mats.size();
  }
  // work queue: tile items by pass (all larger circuits), interleaved with
  // whole-state circuits, then the final items of the larger circuits
  std::vector<BatchItem> q;
  std::vector<uint32_t> small, large;
  uint32_t maxp = 0;
  for (uint64_t i = 0; i < count; ++i) {
    if (circs[i].ntiles == 1 && circs[i].npasses <= 1)
      small.push_back(uint32_t(i));
    else {
      large.push_back(uint32_t(i));
      maxp = std::max(maxp, circs[i].npasses);
    }
  }
  size_t si = 0;
  const size_t small_per_pass = maxp ? (small.size() + maxp - 1) / (maxp + 1) : small.size();
  for (uint32_t p = 0; p < maxp; ++p) {
    for (uint32_t ci : large)
      if (p < circs[ci].npasses)
        for (uint64_t tl = 0; tl < circs[ci].ntiles; ++tl) q.push_back({ci, p, uint32_t(tl), BI_TILE});
    for (size_t j = 0; j < small_per_pass && si < small.size(); ++j, ++si)
      q.push_back({small[si], 0, 0, BI_WHOLE});
  }
  for (uint32_t ci : large) q.push_back({ci, 0, 0, BI_FINAL});
  for (; si < small.size(); ++si) q.push_back({small[si], 0, 0, BI_WHOLE});
  if (stall) q.push_back({0, 0, 0, BI_STALL});
  // meta blob: circs | items | passes | plans | ops | mats
  std::vector<PassRef> passes;
  std::vector<TilePlan> plans;
  passes.reserve(nplans);
  plans.reserve(nplans);
  std::vector<BatchOp> ops;
  ops.reserve(nops);
  std::vector<double> mats;
  mats.reserve(nmats);
  for (uint64_t i = 0; i < count; ++i) {
    const uint32_t op_base = uint32_t(ops.size()), mat_base = uint32_t(mats.size());
    for (const TilePlan& pl : cp[i].plans) plans.push_back(pl);
    for (const PassRef& pr : cp[i].passes) passes.push_back({pr.op0 + op_base, pr.nops});
    for (BatchOp o : cp[i].ops) {
      o.mat += mat_base;
      ops.push_back(o);
    }
    mats.insert(mats.end(), cp[i].mats.begin(), cp[i].mats.end());
  }
  const size_t o_circ = 0, o_items = align256(o_circ + circs.size() * sizeof(BatchCirc));
  const size_t o_pass = align256(o_items + q.size() * sizeof(BatchItem));
  const size_t o_plan = align256(o_pass + passes.size() * sizeof(PassRef));
  const size_t o_ops = align256(o_plan + plans.size() * sizeof(TilePlan));
  const size_t o_mats = align256(o_ops + ops.size() * sizeof(BatchOp));
  const size_t meta = align256(o_mats + mats.size() * sizeof(double));
  const size_t p_states = 0, p_tree = align256(amps * ab), p_uni = align256(p_tree + tree * 8);
  const size_t p_shots = align256(p_uni + uni * 8), p_expz = align256(p_shots + shots * 8);
  const size_t p_done = align256(p_expz + count * 8), p_head = align256(p_done + count * 4);
  const size_t p_cl = align256(p_head + 64);
  const size_t pool = align256(p_cl + ncl);
  const size_t result_bytes = shots * 8 + count * 8 + ncl;
  EV_TRY(grow_dev(&A.dmeta, &A.meta_cap, meta));
  EV_TRY(grow_dev(&A.dpool, &A.pool_cap, pool));
  EV_TRY(grow_host(&A.hstage, &A.stage_cap, std::max(meta, result_bytes)));
  unsigned char* hs = static_cast<unsigned char*>(A.hstage);
  std::memcpy(hs + o_circ, circs.data(), circs.size() * sizeof(BatchCirc));
  std::memcpy(hs + o_items, q.data(), q.size() * sizeof(BatchItem));
  std::memcpy(hs + o_pass, passes.data(), passes.size() * sizeof(PassRef));
  std::memcpy(hs + o_plan, plans.data(), plans.size() * sizeof(TilePlan));
  std::memcpy(hs + o_ops, ops.data(), ops.size() * sizeof(BatchOp));
  std::memcpy(hs + o_mats, mats.data(), mats.size() * sizeof(double));
  unsigned char* dm = static_cast<unsigned char*>(A.dmeta);
  unsigned char* dp = static_cast<unsigned char*>(A.dpool);
  EV_CUDA(cudaMemcpyAsync(dm, hs, meta, cudaMemcpyHostToDevice, A.stream));
  EV_CUDA(cudaMemsetAsync(dp + p_done, 0, pool - p_done, A.stream));
  BatchArgs args;
  args.states = dp + p_states;
  args.trees = reinterpret_cast<double*>(dp + p_tree);
  args.uni = reinterpret_cast<double*>(dp + p_uni);
  args.shots = reinterpret_cast<uint64_t*>(dp + p_shots);
  args.expz = reinterpret_cast<double*>(dp + p_expz);
  args.circs = reinterpret_cast<const BatchCirc*>(dm + o_circ);
  args.items = reinterpret_cast<const BatchItem*>(dm + o_items);
  args.nitems = q.size();
  args.passes = reinterpret_cast<const PassRef*>(dm + o_pass);
  args.plans = reinterpret_cast<const TilePlan*>(dm + o_plan);
  args.ops = reinterpret_cast<const BatchOp*>(dm + o_ops);
  args.mats = reinterpret_cast<const double*>(dm + o_mats);
  args.done = reinterpret_cast<unsigned*>(dp + p_done);
  args.head = reinterpret_cast<unsigned*>(dp + p_head);
  args.err = reinterpret_cast<int*>(dp + p_head + 16);
  args.cl = dp + p_cl;
  args.window = window;
  const auto t1 = clk::now();
  EV_CUDA(cudaEventRecord(A.e0, A.stream));
  k_batch_uniforms<<<unsigned((count + 127) / 128), 128, 0, A.stream>>>(args.circs, count, args.uni);
  // every CTA of the persistent grid must be resident (items wait on each other)
  const unsigned grid = unsigned(sms * per_sm);
  if (debug_enabled())
    fprintf(stderr, "[ev] k_batch dtype %d tile %d threads %d smem %zu window %u: %d CTAs/SM, %zu items\n",
            dtype, kmax, threads, smem, window, per_sm, q.size());
  if (dtype == EV_C128 && threads == 256)
    k_batch<double2, 256><<<grid, threads, smem, A.stream>>>(args, kmax);
  else if (dtype == EV_C128)
    k_batch<double2, 512><<<grid, threads, smem, A.stream>>>(args, kmax);
  else if (threads == 256)
    k_batch<float2, 256><<<grid, threads, smem, A.stream>>>(args, kmax);
  else
    k_batch<float2, 512><<<grid, threads, smem, A.stream>>>(args, kmax);
  EV_CUDA(cudaGetLastError());
  EV_CUDA(cudaEventRecord(A.e1, A.stream));
  // results: shots | expz, one copy down
  EV_CUDA(cudaMemcpyAsync(hs, dp + p_shots, shots * 8, cudaMemcpyDeviceToHost, A.stream));
  EV_CUDA(cudaMemcpyAsync(hs + shots * 8, dp + p_expz, count * 8, cudaMemcpyDeviceToHost, A.stream));
  if (ncl)
    EV_CUDA(cudaMemcpyAsync(hs + shots * 8 + count * 8, dp + p_cl, ncl, cudaMemcpyDeviceToHost,
                            A.stream));
  int err = 0;
  EV_CUDA(cudaMemcpyAsync(&err, args.err, sizeof(int), cudaMemcpyDeviceToHost, A.stream));
  EV_CUDA(cudaStreamSynchronize(A.stream));
  float ms = 0.f;
  EV_CUDA(cudaEventElapsedTime(&ms, A.e0, A.e1));
  if (err) return fail(EV_ERR_TIMEOUT, "batch: a bounded device wait gave up");
  const uint64_t* hshots = reinterpret_cast<const uint64_t*>(hs);
  const double* hexpz = reinterpret_cast<const double*>(hs + shots * 8);
  for (uint64_t i = 0; i < count; ++i) {
    if (items[i].shots_out && items[i].shots)
      std::memcpy(items[i].shots_out, hshots + circs[i].shot_out, items[i].shots * 8);
    if (items[i].expz_out) *items[i].expz_out = hexpz[i];
    if (items[i].classical_out && circs[i].ncl)
      std::memcpy(items[i].classical_out, hs + shots * 8 + count * 8 + circs[i].cl, circs[i].ncl);
  }
  // final states on request (test hook)
  for (uint64_t i = 0; i < count; ++i) {
    if (!items[i].amps_out) continue;
    const uint64_t len = uint64_t(1) << circs[i].n;
    if (dtype == EV_C128) {
      EV_CUDA(cudaMemcpy(items[i].amps_out, dp + p_states + circs[i].state * 16, len * 16,
                         cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> tmp(2 * len);
      EV_CUDA(cudaMemcpy(tmp.data(), dp + p_states + circs[i].state * 8, len * 8, cudaMemcpyDeviceToHost));
      for (uint64_t j = 0; j < 2 * len; ++j) items[i].amps_out[j] = double(tmp[j]);
    }
  }
  const auto t2 = clk::now();
  if (st) {
    st->device_ms = ms;
    st->host_ms = std::chrono::duration<double, std::milli>((t1 - t0) + (t2 - t1)).count() - ms;
    if (st->host_ms < 0) st->host_ms = 0;
    st->items = q.size();
    st->launches = 2;
    st->tile_bits = kmax;
    st->threads = threads;
  }
  return EV_OK;
}

}  // namespace ev

using namespace ev;

extern "C" int ev_batch_run(const ev_batch_circuit* items, uint64_t count, const ev_batch_options* opts,
                            ev_batch_stats* stats) {
  clear_error();
  if (count && !items) return fail(EV_ERR_INVALID_ARGUMENT, "ev_batch_run: null items");
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (count == 0) return EV_OK;
  const int dtype = opts ? opts->dtype : EV_C64;
  if (dtype != EV_C64 && dtype != EV_C128) return fail(EV_ERR_INVALID_ARGUMENT, "unknown amplitude type");
  for (uint64_t i = 0; i < count; ++i) {
    const ev_circuit& c = items[i].circuit;
    EV_TRY(ev_validate(&c));
    if (c.num_qubits < 1 || c.num_qubits > 30)
      return fail(EV_ERR_INVALID_ARGUMENT, "batch circuit %llu: 1..30 qubits supported", (unsigned long long)i);
    if (c.num_classical > uint64_t(kBatchMaxClassical))
      return fail(EV_ERR_INVALID_ARGUMENT, "batch circuit %llu: at most %d classical bits",
                  (unsigned long long)i, kBatchMaxClassical);
    if (items[i].shots && !items[i].shots_out)
      return fail(EV_ERR_INVALID_ARGUMENT, "batch circuit %llu: shots requested without an output",
                  (unsigned long long)i);
  }
  int dev = 0;
  EV_CUDA(cudaGetDevice(&dev));
  ArenaLease lease{acquire_arena(dev)};
  Arena& A = *lease.a;
  int kbits = opts ? opts->tile_bits : 0, threads = opts ? opts->threads : 0;
  const int kcap = max_tile_bits(dtype);
  int from_cache = 0;
  if (kbits <= 0 || threads <= 0) {
    const std::string key = batch_key(items, count, dtype);
    int ck = 0, ct = 0;
    bool cached;
    {
      std::lock_guard<std::mutex> cl(g_cache_mu);
      cached = cache_lookup(key, &ck, &ct);
    }
    if (cached) {
      if (kbits <= 0) kbits = ck;
      if (threads <= 0) threads = ct;
      from_cache = 1;
    } else if (opts && opts->autotune) {
      // time each candidate on an evenly strided sample of the batch
      std::vector<ev_batch_circuit> sample;
      const uint64_t stride = std::max<uint64_t>(1, count / 256);
      for (uint64_t i = 0; i < count; i += stride) {
        ev_batch_circuit b = items[i];
        b.shots_out = nullptr;
        b.expz_out = nullptr;
        b.amps_out = nullptr;
        b.classical_out = nullptr;
        b.shots = 0;
        sample.push_back(b);
      }
      double best = 1e300;
      int bk = default_tile_bits_batch(dtype), bt = 512;
      for (int kc = kcap - 2; kc <= kcap; ++kc)
        for (int tc : {256, 512}) {
          if (kbits > 0 && kc != kbits) continue;
          if (threads > 0 && tc != threads) continue;
          ev_batch_stats s{};
          int rc = batch_once(A, sample.data(), sample.size(), dtype, kc, tc, &s);
          if (rc == EV_OK) rc = batch_once(A, sample.data(), sample.size(), dtype, kc, tc, &s);
          if (rc != EV_OK) {
            clear_error();
            continue;
          }
          if (s.device_ms < best) {
            best = s.device_ms;
            bk = kc;
            bt = tc;
          }
        }
      {
        std::lock_guard<std::mutex> cl(g_cache_mu);
        cache_store(key, bk, bt);
      }
      if (kbits <= 0) kbits = bk;
      if (threads <= 0) threads = bt;
    }
  }
  if (kbits <= 0) kbits = default_tile_bits_batch(dtype);
  if (threads <= 0) threads = 512;
  if (kbits > kcap) kbits = kcap;
  if (kbits < 4) kbits = 4;
  if (threads != 256 && threads != 512)
    return fail(EV_ERR_INVALID_ARGUMENT, "batch: threads must be 256 or 512");
  const int rc = batch_once(A, items, count, dtype, kbits, threads, stats,
                            opts != nullptr && opts->test_stall != 0);
  if (rc == EV_OK && stats) stats->from_cache = from_cache;
  return rc;
}
