// ev_internal.h -- types shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/everett_cuda.h"

namespace ev {

// Records a printf-style message for ev_last_error() and returns code.
int fail(int code, const char* fmt, ...);
// Clears the thread's last error.
void clear_error();
// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum and prefers the max-shared carveout, once per kernel.  Launches
// then pass their own (smaller) sizes; setting the limit per launch would
// race between host threads launching the same kernel with different sizes.
int prepare_smem_kernel(const void* func);
// True when EV_DEBUG is set in the environment (launch configurations are
// then printed to stderr).
bool debug_enabled();

#define EV_CUDA(call)                                                                \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return ::ev::fail(e_ == cudaErrorMemoryAllocation ? EV_ERR_OOM : EV_ERR_CUDA,   \
                        "%s: %s", #call, cudaGetErrorString(e_));                    \
  } while (0)

#define EV_TRY(expr)            \
  do {                          \
    int rc_ = (expr);           \
    if (rc_ != EV_OK) return rc_; \
  } while (0)

// Upper bound on blocks of a reduction grid (partials live in the state's
// scratch area).
constexpr int kMaxRedBlocks = 2048;

// Per-state device scratch: reduction partials, measurement results and the
// device-resident classical register of a run.
struct Scratch {
  double* partials;   // kMaxRedBlocks * 4 doubles
  double* result;     // 8 doubles: reduction results
  double* meas;       // 4 doubles: p1, scale, outcome (as double), u
  uint8_t* pred;      // 64 bytes: combined predicates of nested IfClassic
  uint32_t* counter;  // 4 words: uniforms consumed by device-side measurement
};

}  // namespace ev

namespace ev {
// Kernel classes of the profiler.
enum ProfClass { P_TILE = 0, P_GATE, P_MEASURE, P_SAMPLE, P_FUSED, P_PERMUTE, P_OTHER, P_COUNT };
struct ProfRec {
  int cls;
  cudaEvent_t a, b;
  double bytes;
};
struct ProfStat {
  uint64_t launches;
  double ms;
  double bytes;
};
}  // namespace ev

struct ev_state {
  uint64_t n = 0;
  int32_t dtype = EV_C128;
  int device = 0;
  int num_sms = 0;
  void* amps = nullptr;  // 2^n amplitudes, double2 or float2
  cudaStream_t stream = nullptr;
  void* scratch_block = nullptr;
  ev::Scratch scratch{};
  double* mass = nullptr;  // sampling tree, 2^n - 1 doubles, allocated on demand
  uint64_t mass_len = 0;
  mutable uint64_t launches = 0;  // kernels launched for this state
  int tc_ctas_per_sm = 0;         // last tensor-core launch: resident CTAs per SM
  cudaEvent_t slots[16] = {};
  bool profiling = false;
  bool capturing = false;  // launches are being recorded into a graph
  std::vector<ev::ProfRec> pending;
  std::vector<cudaEvent_t> event_pool;
  ev::ProfStat stats[ev::P_COUNT] = {};
  uint64_t len() const { return uint64_t(1) << n; }
  size_t amp_bytes() const { return dtype == EV_C128 ? 16 : 8; }
};

namespace ev {
// Brackets the launches of one kernel class with events while profiling.
struct ProfScope {
  ev_state* s;
  int cls;
  double bytes;
  cudaEvent_t a = nullptr;
  ProfScope(ev_state* st, int c, double b);
  ~ProfScope();
};
// Resolves pending profile records (waits for their events).
void profile_flush(ev_state* s);
}  // namespace ev

namespace ev {

// A 1-qubit matrix, already in the state's precision.
enum Kind1 { K1_DENSE = 0, K1_REAL, K1_DIAG, K1_PHASE, K1_ANTI, K1_IDENT };
Kind1 classify1(const double m[8]);

enum Kind2 { K2_DENSE = 0, K2_CNOT, K2_CZ, K2_SWAP, K2_DIAG };
Kind2 classify2(const double m[32]);

// Predicate of a conditional launch: nullptr = unconditional, else the
// kernel runs only if *pred != 0 (device memory).
int launch_apply1(ev_state* s, uint64_t k, const double m[8], const uint8_t* pred);
int launch_apply2(ev_state* s, uint64_t a, uint64_t b, const double m[32], const uint8_t* pred);
int launch_controlled(ev_state* s, uint64_t ctrl_mask, uint64_t target, const double m[8],
                      const uint8_t* pred);
// Device-side measurement: the uniform is u_host when u_dev is null, else
// u_dev[*counter] (and the counter advances when the measurement runs).
int launch_measure(ev_state* s, uint64_t k, double u_host, const double* u_dev,
                   uint8_t* outcome_dev, const uint8_t* pred);
// pred_out = AND of classical[bits[i]]
int launch_pred_and(ev_state* s, const uint8_t* classical, const uint64_t* bits, int nbits,
                    uint8_t* pred_out);

// Host bytes gathered while planning a run, uploaded once (256-byte
// aligned sections).
struct PlanBlob {
  std::vector<unsigned char> host;
  size_t add(const void* p, size_t n) {
    const size_t off = (host.size() + 255) / 256 * 256;
    host.resize(off + n);
    if (n) memcpy(host.data() + off, p, n);
    return off;
  }
};

// One shared-memory tile pass or one fused-unitary pass of a planned run.
struct SegStep {
  int fused = 0;        // 0: tile pass, 1: fused unitary
  size_t off0 = 0;      // tile: TilePlan offset; fused: FusedDesc offset (in the blob)
  size_t off1 = 0;      // tile: first op record; fused: matrix operands
  int nops = 0;         // tile: op records
  int k = 0, L = 0;     // tile: tile bits, contiguous low bits; fused: k = qubits
  int variant = 0;      // fused: EV_FUSED_*
  int tma = 0;          // fused: TMA-staged pipeline
  uint64_t count = 0;   // tile: tiles; fused: 128-row steps
};

// Plans ops [first, last) of a gate run (mode EV_MODE_TILED or
// EV_MODE_FUSED) into segment steps whose data are appended to the blob.
// Value a kernel leaves in the run's device flag (scratch counter 1) when a
// fused complex128 pass meets a NaN or an infinity (other non-zero values: a
// bounded wait gave up).
constexpr int kFlagNonFinite = 2;

int plan_segment(ev_state* s, const ev_circuit* c, uint64_t first, uint64_t last, int mode,
                 int bits, int variant, PlanBlob* blob, std::vector<SegStep>* out);
// Launches one planned segment step (dblob = the uploaded blob).
int launch_tile_step(ev_state* s, const SegStep& st, const unsigned char* dblob);
int launch_fused_step(ev_state* s, const SegStep& st, const unsigned char* dblob);

int reduce_norm(const ev_state* s, double* out_host);
// Queues State::normalize (FP64 norm, then scaling) on the state's stream.
int launch_normalize(ev_state* s);
int state_zero(ev_state* s);

// Host restatement of the reference's xoshiro256++ seeded through
// SplitMix64 (src/rng.rs:18-58): the engine draws measurement and shot
// uniforms with it so they match the CPU crate's stream.
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (int w = 0; w < 4; ++w) {
      seed += 0x9E3779B97F4A7C15ULL;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      s[w] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
  uint64_t next_u64() {
    const uint64_t result = rotl(s[0] + s[3], 23) + s[0];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  double next_f64() { return double(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
};

// 256-thread blocks of a kernel that one SM holds at once (its register and
// shared-memory use decide), at most 8, queried once per kernel.  A
// grid-stride or chunked launch sized to one full wave of these leaves no
// partial second wave draining on part of the SMs.
template <auto Kernel>
int resident_blocks() {
  static const int per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, Kernel, 256, 0) != cudaSuccess) {
      (void)cudaGetLastError();
      v = 0;
    }
    return v < 1 ? 1 : (v > 8 ? 8 : v);
  }();
  return per_sm;
}

}  // namespace ev
