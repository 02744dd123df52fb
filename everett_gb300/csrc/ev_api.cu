// ev_api.cu -- library state, storage and the statevector run loop.
//
// The run loop restates StateVectorBackend::run_seeded
// (src/backend/statevector.rs:77-90) and drive/apply_op
// (src/backend/mod.rs:43-72) with the state resident on the device:
//   - every op is a kernel on the state's stream; the host never waits
//     inside a run;
//   - the classical register lives in device memory, Measure writes its
//     outcome there and IfClassic turns into a device predicate that the
//     gated kernel reads before doing any work;
//   - measurement uniforms come from the reference's Rng stream, drawn on the
//     host one per Measure record in op order and consumed on the device
//     through a counter, so a conditional Measure that does not run does not
//     consume one (matching rng.next_f64() being called only inside
//     measure_qubit).
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "ev_device.cuh"
#include "ev_internal.h"
#include "ev_softfp.cuh"

namespace ev {

static thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}
void clear_error() { g_err[0] = 0; }

int prepare_smem_kernel(const void* func) {
  static std::mutex mu;
  static std::vector<const void*> done;
  std::lock_guard<std::mutex> lock(mu);
  for (const void* f : done)
    if (f == func) return EV_OK;
  int dev = 0, optin = 0;
  EV_CUDA(cudaGetDevice(&dev));
  EV_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa{};
  EV_CUDA(cudaFuncGetAttributes(&fa, func));
  EV_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               optin - int(fa.sharedSizeBytes)));
  EV_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout,
                               int(cudaSharedmemCarveoutMaxShared)));
  done.push_back(func);
  return EV_OK;
}

bool debug_enabled() {
  static const bool on = [] {
    const char* v = getenv("EV_DEBUG");
    return v != nullptr && v[0] != 0 && v[0] != '0';
  }();
  return on;
}

__global__ void k_set_basis0_c128(double2* a) { a[0] = make_double2(1.0, 0.0); }
__global__ void k_set_basis0_c64(float2* a) { a[0] = make_float2(1.0f, 0.0f); }

__global__ void k_f64_to_c64(const double2* __restrict__ in, float2* __restrict__ out, uint64_t n) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride)
    out[j] = make_float2(float(in[j].x), float(in[j].y));
}
__global__ void k_c64_to_f64(const float2* __restrict__ in, double2* __restrict__ out, uint64_t n) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride)
    out[j] = make_double2(double(in[j].x), double(in[j].y));
}

static cudaEvent_t take_event(ev_state* s) {
  if (!s->event_pool.empty()) {
    cudaEvent_t e = s->event_pool.back();
    s->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

ProfScope::ProfScope(ev_state* st, int c, double b) : s(st), cls(c), bytes(b) {
  if (s->profiling && !s->capturing) {
    a = take_event(s);
    if (a) cudaEventRecord(a, s->stream);
  }
}

ProfScope::~ProfScope() {
  if (!a) return;
  cudaEvent_t b = take_event(s);
  if (!b) return;
  cudaEventRecord(b, s->stream);
  s->pending.push_back({cls, a, b, bytes});
}

void profile_flush(ev_state* s) {
  for (const ProfRec& r : s->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      s->stats[r.cls].launches += 1;
      s->stats[r.cls].ms += ms;
      s->stats[r.cls].bytes += r.bytes;
    } else {
      cudaGetLastError();
    }
    s->event_pool.push_back(r.a);
    s->event_pool.push_back(r.b);
  }
  s->pending.clear();
}

int state_zero(ev_state* s) {
  s->launches += 1;
  EV_CUDA(cudaMemsetAsync(s->amps, 0, s->len() * s->amp_bytes(), s->stream));
  if (s->dtype == EV_C128)
    k_set_basis0_c128<<<1, 1, 0, s->stream>>>(static_cast<double2*>(s->amps));
  else
    k_set_basis0_c64<<<1, 1, 0, s->stream>>>(static_cast<float2*>(s->amps));
  EV_CUDA(cudaGetLastError());
  return EV_OK;
}

// ---- validation (src/circuit.rs:245-306) --------------------------------

static int qubit_err(uint64_t q, uint64_t n) {
  return fail(EV_ERR_QUBIT_OUT_OF_RANGE, "qubit q%llu out of range for %llu-qubit register",
              (unsigned long long)q, (unsigned long long)n);
}
static int check_qubit(const ev_circuit* c, uint64_t q) {
  return q < c->num_qubits ? EV_OK : qubit_err(q, c->num_qubits);
}
static int check_classical(const ev_circuit* c, uint64_t b) {
  if (b < c->num_classical) return EV_OK;
  return fail(EV_ERR_CLASSICAL_BIT_OUT_OF_RANGE,
              "classical bit c%llu out of range for %llu-bit register", (unsigned long long)b,
              (unsigned long long)c->num_classical);
}

static int validate_op(const ev_circuit* c, uint64_t* pos) {
  if (*pos >= c->nops)
    return fail(EV_ERR_INVALID_ARGUMENT, "op list ends inside an IfClassic record");
  const ev_op& op = c->ops[*pos];
  *pos += 1;
  switch (op.kind) {
    case EV_OP_APPLY1:
      return check_qubit(c, op.q0);
    case EV_OP_APPLY2:
      EV_TRY(check_qubit(c, op.q0));
      EV_TRY(check_qubit(c, op.q1));
      if (op.q0 == op.q1)
        return fail(EV_ERR_DUPLICATE_QUBIT, "qubit q%llu used more than once in a single gate",
                    (unsigned long long)op.q0);
      return EV_OK;
    case EV_OP_CONTROLLED:
      EV_TRY(check_qubit(c, op.q0));
      if (op.nctrl && (!c->ctrl_pool || op.ctrl_off + op.nctrl > c->pool_len))
        return fail(EV_ERR_INVALID_ARGUMENT, "control list outside the control pool");
      for (uint32_t j = 0; j < op.nctrl; ++j) {
        const uint64_t q = c->ctrl_pool[op.ctrl_off + j];
        EV_TRY(check_qubit(c, q));
        if (q == op.q0)
          return fail(EV_ERR_DUPLICATE_QUBIT, "qubit q%llu used more than once in a single gate",
                      (unsigned long long)q);
      }
      return EV_OK;
    case EV_OP_MEASURE:
      EV_TRY(check_qubit(c, op.q0));
      return check_classical(c, op.q1);
    case EV_OP_IF:
      EV_TRY(check_classical(c, op.q0));
      return validate_op(c, pos);
    default:
      return fail(EV_ERR_INVALID_ARGUMENT, "unknown op kind %u", op.kind);
  }
}

static int validate(const ev_circuit* c) {
  if (!c) return fail(EV_ERR_INVALID_ARGUMENT, "null circuit");
  if (c->nops && !c->ops) return fail(EV_ERR_INVALID_ARGUMENT, "null op list");
  uint64_t pos = 0;
  while (pos < c->nops) EV_TRY(validate_op(c, &pos));
  return EV_OK;
}

// ---- run --------------------------------------------------------------

// Keeps freed stream-ordered memory in the device pool instead of returning
// it to the driver at every synchronisation.
void keep_pool_warm(int device) {
  static bool done[256] = {};
  if (device < 0 || device >= 256 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t threshold = ~uint64_t(0);
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  cudaGetLastError();
  done[device] = true;
}

// Uniforms of a prepared run, drawn on the device from the seed that the
// graph copied in (the same generator as the host's Rng, src/rng.rs:18-58).
__global__ void k_run_uniforms(const uint64_t* seed, double* out, uint64_t n) {
  DevRng r(*seed);
  for (uint64_t j = 0; j < n; ++j) out[j] = r.next_f64();
}

enum RunStepKind { RS_APPLY1 = 0, RS_APPLY2, RS_CTRL, RS_MEASURE, RS_PRED_AND, RS_SEGMENT };

// One launch group of a planned run.  Everything a step needs is held here
// or in the uploaded blob, so a plan outlives the circuit it came from.
struct RunStep {
  int kind = 0;
  int pred = 0;        // 0: unconditional; 1: classical[pbit]; 2: the AND of an IF chain
  uint64_t pbit = 0;
  uint64_t q0 = 0, q1 = 0, mask = 0;
  size_t bits_off = 0;  // RS_PRED_AND: classical bit list in the blob
  int nbits = 0;
  double m[32];
  SegStep seg;
};

// A run planned once: steps, one device blob (IF bit lists, tile plans and
// records, fused descriptors and operand images), classical register and
// uniforms.  Executing it only enqueues memsets, copies and kernels on the
// state's stream, so it can be captured into a CUDA graph.
struct RunPlan {
  cudaStream_t stream = nullptr;
  std::vector<RunStep> steps;
  PlanBlob blob;
  uint64_t nmeas = 0, num_classical = 0;
  bool normalize = false;
  unsigned char* dblob = nullptr;
  uint8_t* classical = nullptr;
  double* uniforms = nullptr;
  uint64_t* dseed = nullptr;
  void release() {
    if (dblob) cudaFreeAsync(dblob, stream);
    if (classical) cudaFreeAsync(classical, stream);
    if (uniforms) cudaFreeAsync(uniforms, stream);
    if (dseed) cudaFreeAsync(dseed, stream);
    dblob = nullptr;
    classical = nullptr;
    uniforms = nullptr;
    dseed = nullptr;
  }
  ~RunPlan() { release(); }
};

// The device flag of a run: 0 ok, kFlagNonFinite when the digit-sliced
// complex128 pass met a non-finite amplitude, otherwise a bounded wait that
// gave up.
static int device_flag_status(uint32_t flag) {
  if (flag == 0) return EV_OK;
  if (flag == uint32_t(kFlagNonFinite))
    return fail(EV_ERR_INVALID_ARGUMENT,
                "a non-finite amplitude reached the fused complex128 pass, whose fixed-point digits "
                "cannot carry it");
  return fail(EV_ERR_TIMEOUT, "a bounded device wait gave up during the run");
}

static int build_plan(ev_state* s, const ev_circuit* c, const ev_run_options* o, bool device_seed,
                      RunPlan* plan) {
  // without options: the tiled mode, bit-identical to the exact one and the
  // fastest complex128 mode that keeps the reference's arithmetic
  const int mode = o ? o->mode : EV_MODE_TILED;
  const int tile_bits = o ? o->tile_bits : 0;
  const int variant = o ? o->variant : 0;
  if (mode == EV_MODE_FUSED && (variant == EV_FUSED_OZAKI || variant == EV_FUSED_OZAKI6) != (s->dtype == EV_C128))
    return fail(EV_ERR_INVALID_ARGUMENT, (variant == EV_FUSED_OZAKI || variant == EV_FUSED_OZAKI6)
                                             ? "the ozaki fused variants need complex128 amplitudes"
                                             : "fused mode needs complex64 amplitudes");
  if (mode < EV_MODE_EXACT || mode > EV_MODE_FUSED)
    return fail(EV_ERR_INVALID_ARGUMENT, "unknown run mode %d", mode);
  plan->stream = s->stream;
  plan->num_classical = c->num_classical;
  // complex64 runs end with an FP64 renormalisation: FP32-rounded gate
  // matrices are unitary only to ~1e-7, and the drift of the norm over a deep
  // circuit would otherwise dominate the error against the f64 result.
  plan->normalize = s->dtype == EV_C64;
  std::vector<SegStep> segs;
  uint64_t pos = 0;
  while (pos < c->nops) {
    // collect an IF prefix chain
    uint64_t chain[64];
    int nchain = 0;
    while (c->ops[pos].kind == EV_OP_IF) {
      if (nchain < 64) chain[nchain++] = c->ops[pos].q0;
      ++pos;
    }
    RunStep head;
    if (nchain == 1) {
      head.pred = 1;
      head.pbit = chain[0];
    } else if (nchain > 1) {
      RunStep st;
      st.kind = RS_PRED_AND;
      st.bits_off = plan->blob.add(chain, nchain * sizeof(uint64_t));
      st.nbits = nchain;
      plan->steps.push_back(st);
      head.pred = 2;
    }
    // tiled and fused modes: one segment per run of unconditional gates
    if (mode != EV_MODE_EXACT && nchain == 0 && c->ops[pos].kind != EV_OP_MEASURE) {
      uint64_t end = pos;
      while (end < c->nops && c->ops[end].kind != EV_OP_MEASURE && c->ops[end].kind != EV_OP_IF)
        ++end;
      segs.clear();
      EV_TRY(plan_segment(s, c, pos, end, mode, tile_bits, variant, &plan->blob, &segs));
      for (const SegStep& g : segs) {
        RunStep st;
        st.kind = RS_SEGMENT;
        st.seg = g;
        plan->steps.push_back(st);
      }
      pos = end;
      continue;
    }
    const ev_op& op = c->ops[pos];
    RunStep st = head;
    st.q0 = op.q0;
    st.q1 = op.q1;
    switch (op.kind) {
      case EV_OP_APPLY1:
        st.kind = RS_APPLY1;
        std::memcpy(st.m, op.m, 8 * sizeof(double));
        break;
      case EV_OP_APPLY2:
        st.kind = RS_APPLY2;
        std::memcpy(st.m, op.m, 32 * sizeof(double));
        break;
      case EV_OP_CONTROLLED:
        st.kind = RS_CTRL;
        for (uint32_t j = 0; j < op.nctrl; ++j) st.mask |= uint64_t(1) << c->ctrl_pool[op.ctrl_off + j];
        std::memcpy(st.m, op.m, 8 * sizeof(double));
        break;
      case EV_OP_MEASURE:
        st.kind = RS_MEASURE;
        ++plan->nmeas;
        break;
    }
    plan->steps.push_back(st);
    ++pos;
  }
  // device buffers: stream-ordered, so planning never synchronises the device
  const uint64_t ncl = c->num_classical ? c->num_classical : 1;
  EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&plan->classical), ncl, s->stream));
  EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&plan->uniforms),
                          (plan->nmeas ? plan->nmeas : 1) * sizeof(double), s->stream));
  if (device_seed)
    EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&plan->dseed), sizeof(uint64_t), s->stream));
  if (!plan->blob.host.empty()) {
    EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&plan->dblob), plan->blob.host.size(), s->stream));
    EV_CUDA(cudaMemcpyAsync(plan->dblob, plan->blob.host.data(), plan->blob.host.size(),
                            cudaMemcpyHostToDevice, s->stream));
  }
  return EV_OK;
}

// Enqueues a planned run.  zero: reset the state to |0...0> first.  The
// classical register and the two device flags are copied to the host
// buffers given (flags[1]: see device_flag_status).
static int execute_plan(ev_state* s, const RunPlan& plan, bool zero, uint8_t* classical_host,
                        uint32_t* flags_host) {
  if (zero) EV_TRY(state_zero(s));
  const uint64_t ncl = plan.num_classical ? plan.num_classical : 1;
  EV_CUDA(cudaMemsetAsync(plan.classical, 0, ncl, s->stream));
  // counter[0]: uniforms consumed; counter[1]: device flag (timeout, non-finite)
  EV_CUDA(cudaMemsetAsync(s->scratch.counter, 0, 2 * sizeof(uint32_t), s->stream));
  if (plan.dseed && plan.nmeas) {
    k_run_uniforms<<<1, 1, 0, s->stream>>>(plan.dseed, plan.uniforms, plan.nmeas);
    s->launches += 1;
    EV_CUDA(cudaGetLastError());
  }
  for (const RunStep& st : plan.steps) {
    const uint8_t* pred = st.pred == 1   ? plan.classical + st.pbit
                          : st.pred == 2 ? s->scratch.pred
                                         : nullptr;
    switch (st.kind) {
      case RS_APPLY1:
        EV_TRY(launch_apply1(s, st.q0, st.m, pred));
        break;
      case RS_APPLY2:
        EV_TRY(launch_apply2(s, st.q0, st.q1, st.m, pred));
        break;
      case RS_CTRL:
        EV_TRY(launch_controlled(s, st.mask, st.q0, st.m, pred));
        break;
      case RS_MEASURE:
        EV_TRY(launch_measure(s, st.q0, 0.0, plan.uniforms, plan.classical + st.q1, pred));
        break;
      case RS_PRED_AND:
        EV_TRY(launch_pred_and(s, plan.classical,
                               reinterpret_cast<const uint64_t*>(plan.dblob + st.bits_off), st.nbits,
                               s->scratch.pred));
        break;
      case RS_SEGMENT:
        if (st.seg.fused)
          EV_TRY(launch_fused_step(s, st.seg, plan.dblob));
        else
          EV_TRY(launch_tile_step(s, st.seg, plan.dblob));
        break;
    }
  }
  if (plan.normalize) EV_TRY(launch_normalize(s));
  if (plan.num_classical)
    EV_CUDA(cudaMemcpyAsync(classical_host, plan.classical, plan.num_classical,
                            cudaMemcpyDeviceToHost, s->stream));
  EV_CUDA(cudaMemcpyAsync(flags_host, s->scratch.counter, 2 * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, s->stream));
  return EV_OK;
}

static int run_ops(ev_state* s, const ev_circuit* c, uint64_t seed, const ev_run_options* o,
                   uint8_t* classical_out) {
  RunPlan plan;
  EV_TRY(build_plan(s, c, o, false, &plan));
  // uniforms from the host generator, one per Measure record (the host
  // vector lives until the stream has been synchronised)
  std::vector<double> uni(plan.nmeas);
  if (plan.nmeas) {
    Rng rng(seed);
    for (uint64_t j = 0; j < plan.nmeas; ++j) uni[j] = rng.next_f64();
    EV_CUDA(cudaMemcpyAsync(plan.uniforms, uni.data(), uni.size() * sizeof(double),
                            cudaMemcpyHostToDevice, s->stream));
  }
  uint32_t flags[2] = {0, 0};
  EV_TRY(execute_plan(s, plan, false, classical_out, flags));
  EV_CUDA(cudaStreamSynchronize(s->stream));
  return device_flag_status(flags[1]);
}

static int create_state(uint64_t n, int32_t dtype, ev_state** out) {
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_create: null output");
  if (dtype != EV_C128 && dtype != EV_C64)
    return fail(EV_ERR_INVALID_ARGUMENT, "unknown amplitude type %d", dtype);
  if (n > 40) return fail(EV_ERR_OOM, "2^%llu amplitudes cannot be stored", (unsigned long long)n);
  std::unique_ptr<ev_state> s(new ev_state());
  s->n = n;
  s->dtype = dtype;
  EV_CUDA(cudaGetDevice(&s->device));
  EV_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device));
  keep_pool_warm(s->device);
  const size_t bytes = size_t(s->len()) * s->amp_bytes();
  cudaError_t e = cudaMalloc(&s->amps, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    s->amps = nullptr;
    return fail(EV_ERR_OOM, "cannot allocate %zu bytes for a %llu-qubit state", bytes,
                (unsigned long long)n);
  }
  const size_t sb = kMaxRedBlocks * 4 * sizeof(double) + 8 * sizeof(double) + 4 * sizeof(double) +
                    64 + 16;
  e = cudaMalloc(&s->scratch_block, sb);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(s->amps);
    return fail(EV_ERR_OOM, "cannot allocate state scratch");
  }
  char* p = static_cast<char*>(s->scratch_block);
  s->scratch.partials = reinterpret_cast<double*>(p);
  p += kMaxRedBlocks * 4 * sizeof(double);
  s->scratch.result = reinterpret_cast<double*>(p);
  p += 8 * sizeof(double);
  s->scratch.meas = reinterpret_cast<double*>(p);
  p += 4 * sizeof(double);
  s->scratch.pred = reinterpret_cast<uint8_t*>(p);
  p += 64;
  s->scratch.counter = reinterpret_cast<uint32_t*>(p);
  e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaFree(s->amps);
    cudaFree(s->scratch_block);
    return fail(EV_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  int rc = state_zero(s.get());
  if (rc == EV_OK) {
    e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "state init: %s", cudaGetErrorString(e));
  }
  if (rc != EV_OK) {
    cudaFree(s->amps);
    cudaFree(s->scratch_block);
    cudaStreamDestroy(s->stream);
    return rc;
  }
  *out = s.release();
  return EV_OK;
}

}  // namespace ev

using namespace ev;

extern "C" const char* ev_last_error(void) { return g_err; }
extern "C" const char* ev_version(void) { return "everett-gb300 0.1.0 (sm_103a)"; }

extern "C" int ev_device_count(int* out) {
  clear_error();
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "null output");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *out = n;
  return EV_OK;
}

extern "C" int ev_state_create(uint64_t n, int32_t dtype, ev_state** out) {
  clear_error();
  return create_state(n, dtype, out);
}

// Destroying never fails and leaves the last error message in place (a run
// that fails frees its own state before returning the error).
extern "C" int ev_state_destroy(ev_state* s) {
  if (!s) return EV_OK;
  cudaSetDevice(s->device);
  cudaStreamSynchronize(s->stream);
  if (s->amps) cudaFree(s->amps);
  if (s->scratch_block) cudaFree(s->scratch_block);
  if (s->mass) cudaFree(s->mass);
  profile_flush(s);
  for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : s->slots)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(s->stream);
  delete s;
  return EV_OK;
}

extern "C" int ev_state_num_qubits(const ev_state* s, uint64_t* out) {
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "null argument");
  *out = s->n;
  return EV_OK;
}

extern "C" int ev_state_dtype(const ev_state* s, int32_t* out) {
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "null argument");
  *out = s->dtype;
  return EV_OK;
}

extern "C" int ev_state_set_zero(ev_state* s) {
  clear_error();
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "null state");
  EV_CUDA(cudaSetDevice(s->device));
  return state_zero(s);
}

extern "C" int ev_state_synchronize(const ev_state* s) {
  clear_error();
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "null state");
  EV_CUDA(cudaSetDevice(s->device));
  EV_CUDA(cudaStreamSynchronize(s->stream));
  return EV_OK;
}

// Staging size for complex64 conversions (complex amplitudes per chunk).
static const uint64_t kStage = uint64_t(1) << 24;

extern "C" int ev_state_upload(ev_state* s, const double* amps, uint64_t len) {
  clear_error();
  if (!s || (len && !amps)) return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_upload: null argument");
  if (len != s->len())
    return fail(EV_ERR_DIMENSION_MISMATCH, "amplitude buffer has length %llu, expected %llu",
                (unsigned long long)len, (unsigned long long)s->len());
  EV_CUDA(cudaSetDevice(s->device));
  if (s->dtype == EV_C128) {
    EV_CUDA(cudaMemcpyAsync(s->amps, amps, len * 16, cudaMemcpyHostToDevice, s->stream));
    EV_CUDA(cudaStreamSynchronize(s->stream));
    return EV_OK;
  }
  const uint64_t chunk = len < kStage ? len : kStage;
  double2* stage = nullptr;
  EV_CUDA(cudaMalloc(&stage, chunk * 16));
  int rc = EV_OK;
  for (uint64_t off = 0; off < len && rc == EV_OK; off += chunk) {
    const uint64_t cnt = (len - off) < chunk ? (len - off) : chunk;
    cudaError_t e = cudaMemcpyAsync(stage, amps + 2 * off, cnt * 16, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
      k_f64_to_c64<<<unsigned((cnt + 255) / 256 < 4096 ? (cnt + 255) / 256 : 4096), 256, 0, s->stream>>>(
          stage, static_cast<float2*>(s->amps) + off, cnt);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "ev_state_upload: %s", cudaGetErrorString(e));
  }
  cudaFree(stage);
  return rc;
}

extern "C" int ev_state_download(const ev_state* s, double* amps, uint64_t len) {
  clear_error();
  if (!s || (len && !amps)) return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_download: null argument");
  if (len != s->len())
    return fail(EV_ERR_DIMENSION_MISMATCH, "amplitude buffer has length %llu, expected %llu",
                (unsigned long long)len, (unsigned long long)s->len());
  EV_CUDA(cudaSetDevice(s->device));
  if (s->dtype == EV_C128) {
    EV_CUDA(cudaMemcpyAsync(amps, s->amps, len * 16, cudaMemcpyDeviceToHost, s->stream));
    EV_CUDA(cudaStreamSynchronize(s->stream));
    return EV_OK;
  }
  const uint64_t chunk = len < kStage ? len : kStage;
  double2* stage = nullptr;
  EV_CUDA(cudaMalloc(&stage, chunk * 16));
  int rc = EV_OK;
  for (uint64_t off = 0; off < len && rc == EV_OK; off += chunk) {
    const uint64_t cnt = (len - off) < chunk ? (len - off) : chunk;
    k_c64_to_f64<<<unsigned((cnt + 255) / 256 < 4096 ? (cnt + 255) / 256 : 4096), 256, 0, s->stream>>>(
        static_cast<const float2*>(s->amps) + off, stage, cnt);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(amps + 2 * off, stage, cnt * 16, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "ev_state_download: %s", cudaGetErrorString(e));
  }
  cudaFree(stage);
  return rc;
}

extern "C" int ev_validate(const ev_circuit* c) {
  clear_error();
  return validate(c);
}

extern "C" int ev_run_seeded(const ev_circuit* c, uint64_t seed, const ev_run_options* opts,
                             ev_state** state_out, uint8_t* classical_out) {
  clear_error();
  EV_TRY(validate(c));
  if (!state_out || (c->num_classical && !classical_out))
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_run_seeded: null output");
  const int32_t dtype = opts ? opts->dtype : EV_C128;
  ev_state* s = nullptr;
  EV_TRY(create_state(c->num_qubits, dtype, &s));
  const int rc = run_ops(s, c, seed, opts, classical_out);
  if (rc != EV_OK) {
    ev_state_destroy(s);
    return rc;
  }
  *state_out = s;
  return EV_OK;
}

extern "C" int ev_state_run(ev_state* s, const ev_circuit* c, uint64_t seed,
                            const ev_run_options* opts, uint8_t* classical_out) {
  clear_error();
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_run: null state");
  EV_TRY(validate(c));
  if (c->num_qubits != s->n)
    return fail(EV_ERR_DIMENSION_MISMATCH, "circuit has %llu qubits, state has %llu",
                (unsigned long long)c->num_qubits, (unsigned long long)s->n);
  if (opts && opts->dtype != s->dtype)
    return fail(EV_ERR_INVALID_ARGUMENT, "run options name a different amplitude type");
  if (c->num_classical && !classical_out)
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_run: null classical output");
  EV_CUDA(cudaSetDevice(s->device));
  EV_TRY(state_zero(s));
  return run_ops(s, c, seed, opts, classical_out);
}

// backend/mod.rs:43-72 (drive): the op walk on the state as it stands.
extern "C" int ev_state_drive(ev_state* s, const ev_circuit* c, uint64_t seed,
                              const ev_run_options* opts, uint8_t* classical_out) {
  clear_error();
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_drive: null state");
  EV_TRY(validate(c));
  if (c->num_qubits != s->n)
    return fail(EV_ERR_DIMENSION_MISMATCH, "circuit has %llu qubits, state has %llu",
                (unsigned long long)c->num_qubits, (unsigned long long)s->n);
  if (opts && opts->dtype != s->dtype)
    return fail(EV_ERR_INVALID_ARGUMENT, "run options name a different amplitude type");
  if (c->num_classical && !classical_out)
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_state_drive: null classical output");
  EV_CUDA(cudaSetDevice(s->device));
  return run_ops(s, c, seed, opts, classical_out);
}

// ---- prepared runs ----------------------------------------------------------

struct ev_prepared {
  ev_state* s = nullptr;
  ev::RunPlan plan;
  unsigned char* pinned = nullptr;  // seed (8 B), flags (8 B), classical register
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;
  uint64_t* seed_host() { return reinterpret_cast<uint64_t*>(pinned); }
  uint32_t* flags_host() { return reinterpret_cast<uint32_t*>(pinned + 8); }
  uint8_t* classical_host() { return pinned + 16; }
};

static void free_prepared(ev_prepared* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->plan.release();
  cudaStreamSynchronize(p->s->stream);
  if (p->pinned) cudaFreeHost(p->pinned);
  cudaGetLastError();
  delete p;
}

extern "C" int ev_prepare(ev_state* s, const ev_circuit* c, const ev_run_options* opts,
                          ev_prepared** out) {
  clear_error();
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_prepare: null argument");
  EV_TRY(validate(c));
  if (c->num_qubits != s->n)
    return fail(EV_ERR_DIMENSION_MISMATCH, "circuit has %llu qubits, state has %llu",
                (unsigned long long)c->num_qubits, (unsigned long long)s->n);
  if (opts && opts->dtype != s->dtype)
    return fail(EV_ERR_INVALID_ARGUMENT, "run options name a different amplitude type");
  EV_CUDA(cudaSetDevice(s->device));
  ev_prepared* p = new ev_prepared();
  p->s = s;
  int rc = build_plan(s, c, opts, true, &p->plan);
  if (rc == EV_OK) {
    cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&p->pinned), 16 + (c->num_classical | 1));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p->pinned = nullptr;
      rc = fail(EV_ERR_OOM, "cannot allocate pinned run buffers");
    }
  }
  if (rc == EV_OK) {
    // Record the launch-only half of the run.  Relaxed capture: kernel
    // attribute queries made while launching stay legal.
    const uint64_t before = s->launches;
    cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
      rc = fail(EV_ERR_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
    } else {
      s->capturing = true;
      e = cudaMemcpyAsync(p->plan.dseed, p->seed_host(), sizeof(uint64_t), cudaMemcpyHostToDevice,
                          s->stream);
      rc = e == cudaSuccess ? execute_plan(s, p->plan, true, p->classical_host(), p->flags_host())
                            : fail(EV_ERR_CUDA, "seed copy: %s", cudaGetErrorString(e));
      s->capturing = false;
      const cudaError_t e2 = cudaStreamEndCapture(s->stream, &p->graph);
      if (rc == EV_OK && e2 != cudaSuccess)
        rc = fail(EV_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e2));
    }
    p->kernels = s->launches - before;
    s->launches = before;
  }
  if (rc == EV_OK) {
    const cudaError_t e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  }
  if (rc == EV_OK) {
    // planning's uploads must land before the first replay
    const cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "ev_prepare: %s", cudaGetErrorString(e));
  }
  if (rc != EV_OK) {
    cudaGetLastError();
    free_prepared(p);
    return rc;
  }
  *out = p;
  return EV_OK;
}

extern "C" int ev_prepared_launch(ev_prepared* p, uint64_t seed, uint8_t* classical_out) {
  clear_error();
  if (!p) return fail(EV_ERR_INVALID_ARGUMENT, "ev_prepared_launch: null argument");
  const uint64_t ncl = p->plan.num_classical;
  if (ncl && !classical_out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_prepared_launch: null classical output");
  ev_state* s = p->s;
  EV_CUDA(cudaSetDevice(s->device));
  *p->seed_host() = seed;  // read by the graph's first copy
  EV_CUDA(cudaGraphLaunch(p->exec, s->stream));
  EV_CUDA(cudaStreamSynchronize(s->stream));
  s->launches += p->kernels;
  if (ncl) std::memcpy(classical_out, p->classical_host(), ncl);
  return device_flag_status(p->flags_host()[1]);
}

extern "C" int ev_prepared_kernels(const ev_prepared* p, uint64_t* out) {
  clear_error();
  if (!p || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_prepared_kernels: null argument");
  *out = p->kernels;
  return EV_OK;
}

extern "C" int ev_prepared_destroy(ev_prepared* p) {
  clear_error();
  if (!p) return EV_OK;
  cudaSetDevice(p->s->device);
  free_prepared(p);
  return EV_OK;
}

// ---- measurement hooks ------------------------------------------------------

extern "C" int ev_state_record_event(ev_state* s, int32_t slot) {
  clear_error();
  if (!s || slot < 0 || slot >= 16) return fail(EV_ERR_INVALID_ARGUMENT, "bad event slot");
  EV_CUDA(cudaSetDevice(s->device));
  if (!s->slots[slot]) EV_CUDA(cudaEventCreate(&s->slots[slot]));
  EV_CUDA(cudaEventRecord(s->slots[slot], s->stream));
  return EV_OK;
}

extern "C" int ev_state_elapsed_ms(ev_state* s, int32_t from_slot, int32_t to_slot, float* ms) {
  clear_error();
  if (!s || !ms || from_slot < 0 || from_slot >= 16 || to_slot < 0 || to_slot >= 16 ||
      !s->slots[from_slot] || !s->slots[to_slot])
    return fail(EV_ERR_INVALID_ARGUMENT, "bad event slot");
  EV_CUDA(cudaSetDevice(s->device));
  EV_CUDA(cudaEventSynchronize(s->slots[to_slot]));
  EV_CUDA(cudaEventElapsedTime(ms, s->slots[from_slot], s->slots[to_slot]));
  return EV_OK;
}

extern "C" int ev_state_launch_count(const ev_state* s, uint64_t* out) {
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "null argument");
  *out = s->launches;
  return EV_OK;
}

extern "C" int ev_state_profile(ev_state* s, int32_t enable) {
  clear_error();
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "null state");
  EV_CUDA(cudaSetDevice(s->device));
  profile_flush(s);
  if (enable)
    for (auto& st : s->stats) st = ProfStat{};
  s->profiling = enable != 0;
  return EV_OK;
}

extern "C" int ev_state_profile_read(ev_state* s, ev_kernel_stat* out, int32_t max, int32_t* count) {
  clear_error();
  if (!s || !count || (max > 0 && !out)) return fail(EV_ERR_INVALID_ARGUMENT, "null argument");
  EV_CUDA(cudaSetDevice(s->device));
  profile_flush(s);
  static const char* names[P_COUNT] = {"tile_pass", "gate", "measure", "sample",
                                       "fused_unitary", "permute", "other"};
  int w = 0;
  for (int c = 0; c < P_COUNT; ++c) {
    if (s->stats[c].launches == 0) continue;
    if (w < max) {
      std::memset(out[w].name, 0, sizeof(out[w].name));
      std::strncpy(out[w].name, names[c], sizeof(out[w].name) - 1);
      out[w].launches = s->stats[c].launches;
      out[w].ms = s->stats[c].ms;
      out[w].bytes = s->stats[c].bytes;
    }
    ++w;
  }
  *count = w;
  return EV_OK;
}

namespace ev {
// Eight independent FMA chains per thread; the final compare keeps every
// chain live without a store per thread.
__global__ void __launch_bounds__(256) k_probe_fp64(double* out, int iters, double seed) {
  double a[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) a[c] = seed + double(threadIdx.x + c);
  const double m = 0.9999999, add = 1e-7;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = __fma_rn(a[c], m, add);
  double t = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) t += a[c];
  if (t == -1.0) out[0] = t;
}
// Independent chains of integer-pipe adds (softfp::add), as k_probe_fp64
// runs FMA chains: the rate against which moving an add off the FP64 pipe
// is weighed.
__global__ void __launch_bounds__(256) k_probe_softadd(double* out, int iters, double seed) {
  double a[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) a[c] = seed + double(threadIdx.x + c);
  const double add = 1.0000001e-7;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = softfp::add(a[c], add);
  double t = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) t += a[c];
  if (t == -1.0) out[0] = t;
}
}  // namespace ev

// Best of three timed launches of a probe kernel: operations per second
// (blocks x 256 threads x iters x 8 chains per launch time).
static int probe_rate(void (*kernel)(double*, int, double), int iters, const char* name,
                      double* per_s) {
  using namespace ev;
  int dev = 0, sms = 0;
  EV_CUDA(cudaGetDevice(&dev));
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t st = nullptr;
  EV_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = EV_OK;
  const int blocks = sms * 8;
  if (cudaMallocAsync(reinterpret_cast<void**>(&out), sizeof(double), st) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = fail(EV_ERR_CUDA, "%s: setup failed", name);
  } else {
    kernel<<<blocks, 256, 0, st>>>(out, iters, 1.0);  // warm-up
    double best = 0.0;
    for (int rep = 0; rep < 3 && rc == EV_OK; ++rep) {
      cudaEventRecord(e0, st);
      kernel<<<blocks, 256, 0, st>>>(out, iters, 2.0 + rep);
      cudaEventRecord(e1, st);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f) {
        rc = fail(EV_ERR_CUDA, "%s: timing failed", name);
      } else {
        const double r = double(blocks) * 256.0 * double(iters) * 8.0 / (double(ms) * 1e-3);
        if (r > best) best = r;
      }
    }
    if (rc == EV_OK) *per_s = best;
  }
  if (out) cudaFreeAsync(out, st);
  cudaStreamSynchronize(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  cudaGetLastError();
  return rc;
}

extern "C" int ev_probe_softadd(double* adds_per_s) {
  ev::clear_error();
  if (!adds_per_s) return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_probe_softadd: null output");
  return probe_rate(ev::k_probe_softadd, 1 << 12, "ev_probe_softadd", adds_per_s);
}

extern "C" int ev_probe_fp64(double* fma_per_s) {
  clear_error();
  if (!fma_per_s) return fail(EV_ERR_INVALID_ARGUMENT, "ev_probe_fp64: null output");
  int dev = 0, sms = 0;
  EV_CUDA(cudaGetDevice(&dev));
  EV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t st = nullptr;
  EV_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = EV_OK;
  const int iters = 1 << 15, blocks = sms * 8;
  if (cudaMallocAsync(reinterpret_cast<void**>(&out), sizeof(double), st) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = fail(EV_ERR_CUDA, "ev_probe_fp64: setup failed");
  } else {
    k_probe_fp64<<<blocks, 256, 0, st>>>(out, iters, 1.0);  // warm-up
    double best = 0.0;
    for (int rep = 0; rep < 3 && rc == EV_OK; ++rep) {  // best of three
      cudaEventRecord(e0, st);
      k_probe_fp64<<<blocks, 256, 0, st>>>(out, iters, 2.0 + rep);
      cudaEventRecord(e1, st);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f) {
        rc = fail(EV_ERR_CUDA, "ev_probe_fp64: timing failed");
      } else {
        const double r = double(blocks) * 256.0 * double(iters) * 8.0 / (double(ms) * 1e-3);
        if (r > best) best = r;
      }
    }
    if (rc == EV_OK) *fma_per_s = best;
  }
  if (out) cudaFreeAsync(out, st);
  cudaStreamSynchronize(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  cudaGetLastError();
  return rc;
}

extern "C" int ev_host_alloc(uint64_t bytes, void** out) {
  clear_error();
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "null output");
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return fail(EV_ERR_OOM, "cudaMallocHost(%llu): %s", (unsigned long long)bytes, cudaGetErrorString(e));
  }
  return EV_OK;
}

extern "C" int ev_host_free(void* p) {
  clear_error();
  if (p) EV_CUDA(cudaFreeHost(p));
  return EV_OK;
}
