// ev_stab.cu -- stabilizer tableau in HBM (src/backend/stabilizer.rs).
//
// The Aaronson-Gottesman tableau (2n + 1 rows: destabilizers, stabilizers,
// one scratch row; per row an x and a z bit per qubit and a phase bit) is
// bit-packed word-major: word w of row i lives at [w * rows + i], so threads
// that own consecutive rows touch consecutive words.  Clifford conjugation
// acts on every row independently, so a whole run of gates between two
// measurements is one kernel: each thread walks the gate list on its own
// row.  Measurement follows the reference: the first stabilizer with x_q set
// decides random vs determined; the random branch multiplies that row into
// every other anticommuting row (one thread per row, the phase exponent
// summed 64 qubits at a time with bit masks and popcounts); the determined
// branch accumulates the product into the scratch row.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "ev_device.cuh"
#include "ev_internal.h"

struct ev_stab {
  uint64_t n = 0;
  uint64_t rows = 0;   // 2n + 1
  uint64_t words = 0;  // ceil(n / 64)
  uint64_t* x = nullptr;
  uint64_t* z = nullptr;
  uint8_t* r = nullptr;
  int* found = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
};

namespace ev {
namespace {

enum PrimKind : uint32_t { PR_H = 0, PR_S, PR_SDG, PR_X, PR_Y, PR_Z, PR_CNOT };
struct Prim {
  uint32_t kind, a, b, pad;
};

constexpr int kStThreads = 256;

// Applies prims[0 .. count) to rows [0, 2n) (stabilizer.rs:254-320).
__global__ void __launch_bounds__(kStThreads)
    k_st_gates(uint64_t* __restrict__ X, uint64_t* __restrict__ Z, uint8_t* __restrict__ R,
               uint64_t rows, uint64_t active, const Prim* __restrict__ prims, int count) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= active) return;
  uint32_t r = R[i];
  for (int p = 0; p < count; ++p) {
    const Prim g = prims[p];
    const uint64_t wa = uint64_t(g.a >> 6) * rows + i;
    const uint64_t ma = uint64_t(1) << (g.a & 63);
    uint64_t xa = X[wa], za = Z[wa];
    const uint32_t bx = (xa & ma) != 0, bz = (za & ma) != 0;
    switch (g.kind) {
      case PR_H:
        r ^= bx & bz;
        xa = (xa & ~ma) | (bz ? ma : 0);
        za = (za & ~ma) | (bx ? ma : 0);
        X[wa] = xa;
        Z[wa] = za;
        break;
      case PR_S:
        r ^= bx & bz;
        if (bx) Z[wa] = za ^ ma;
        break;
      case PR_SDG:  // S then Z
        r ^= bx & bz;
        if (bx) Z[wa] = za ^ ma;
        r ^= bx;
        break;
      case PR_X: r ^= bz; break;
      case PR_Y: r ^= bx ^ bz; break;
      case PR_Z: r ^= bx; break;
      default: {  // CNOT(a, b): r ^= x_a z_b (x_b ^ z_a ^ 1); x_b ^= x_a; z_a ^= z_b
        const uint64_t wb = uint64_t(g.b >> 6) * rows + i;
        const uint64_t mb = uint64_t(1) << (g.b & 63);
        const uint64_t xb = X[wb], zb = Z[wb];
        const uint32_t cx = (xb & mb) != 0, cz = (zb & mb) != 0;
        r ^= bx & cz & (cx ^ bz ^ 1u);
        if (bx) X[wb] = xb ^ mb;
        if (cz) Z[wa] = Z[wa] ^ ma;  // re-read: wa may equal wb
        break;
      }
    }
  }
  R[i] = uint8_t(r & 1);
}

// First stabilizer row (n <= i < 2n) with x_q set, by atomicMin.
__global__ void k_st_find(const uint64_t* __restrict__ X, uint64_t rows, uint64_t n, uint32_t q,
                          int* found) {
  const uint64_t i = n + uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= 2 * n) return;
  if ((X[uint64_t(q >> 6) * rows + i] >> (q & 63)) & 1) atomicMin(found, int(i));
}

// Sum over 64 qubits of g(x1, z1, x2, z2) (stabilizer.rs:381-390) for the
// row pair (j = 1, h = 2): +1 and -1 terms counted with bit masks.
__device__ __forceinline__ int g_word(uint64_t x1, uint64_t z1, uint64_t x2, uint64_t z2) {
  const uint64_t y1 = x1 & z1, xo = x1 & ~z1, zo = ~x1 & z1;
  const uint64_t plus = (y1 & z2 & ~x2) | (xo & z2 & x2) | (zo & x2 & ~z2);
  const uint64_t minus = (y1 & x2 & ~z2) | (xo & z2 & ~x2) | (zo & x2 & z2);
  return __popcll(plus) - __popcll(minus);
}

// Random branch: rowsum(i, p) for every row i != p of [0, 2n) with x_q set.
__global__ void __launch_bounds__(kStThreads)
    k_st_rowsum_all(uint64_t* __restrict__ X, uint64_t* __restrict__ Z, uint8_t* __restrict__ R,
                    uint64_t rows, uint64_t n, uint64_t words, uint32_t q, int p) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= 2 * n || int(i) == p) return;
  if (!((X[uint64_t(q >> 6) * rows + i] >> (q & 63)) & 1)) return;
  int sum = 2 * int(R[i]) + 2 * int(R[p]);
  for (uint64_t w = 0; w < words; ++w) {
    const uint64_t xj = X[w * rows + p], zj = Z[w * rows + p];
    const uint64_t xh = X[w * rows + i], zh = Z[w * rows + i];
    sum += g_word(xj, zj, xh, zh);
    X[w * rows + i] = xh ^ xj;
    Z[w * rows + i] = zh ^ zj;
  }
  R[i] = uint8_t((((sum % 4) + 4) % 4) == 2);
}

// Random branch, after the rowsums: row p - n <- row p; row p <- +/- Z_q.
__global__ void k_st_settle(uint64_t* __restrict__ X, uint64_t* __restrict__ Z, uint8_t* R,
                            uint64_t rows, uint64_t n, uint64_t words, uint32_t q, int p,
                            int outcome) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w < words) {
    X[w * rows + (p - n)] = X[w * rows + p];
    Z[w * rows + (p - n)] = Z[w * rows + p];
    X[w * rows + p] = 0;
    Z[w * rows + p] = w == (q >> 6) ? (uint64_t(1) << (q & 63)) : 0;
  }
  if (w == 0) {
    R[p - n] = R[p];
    R[p] = uint8_t(outcome);
  }
}

// Determined branch (stabilizer.rs:346-363): the scratch row becomes the
// product of the stabilizers n + i whose destabilizer i has x_q set, and its
// sign is the outcome.  The reference folds the rows in one at a time,
// reducing the phase sum mod 4 at every step; since every partial sum is
// even, that equals the total sum mod 4, and since XOR and the phase terms
// of word w depend only on word w's history, each thread owns one word,
// walks all the rows, and adds its sum mod 4 into acc.  One extra thread
// adds the rows' own signs (2 r_j each).
__global__ void __launch_bounds__(kStThreads)
    k_st_determined(uint64_t* __restrict__ X, uint64_t* __restrict__ Z, const uint8_t* __restrict__ R,
                    uint64_t rows, uint64_t n, uint64_t words, uint32_t q, int* acc) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t qw = uint64_t(q >> 6) * rows;
  const int qs = int(q & 63);
  if (w < words) {
    uint64_t xh = 0, zh = 0;
    int g = 0;
    for (uint64_t i = 0; i < n; ++i) {
      if (!((X[qw + i] >> qs) & 1)) continue;
      const uint64_t xj = X[w * rows + n + i], zj = Z[w * rows + n + i];
      g += g_word(xj, zj, xh, zh);
      xh ^= xj;
      zh ^= zj;
    }
    X[w * rows + 2 * n] = xh;
    Z[w * rows + 2 * n] = zh;
    atomicAdd(acc, ((g % 4) + 4) % 4);
  }
  if (w == 0) {
    int rs = 0;
    for (uint64_t i = 0; i < n; ++i)
      if ((X[qw + i] >> qs) & 1) rs += 2 * int(R[n + i]);
    atomicAdd(acc, rs % 4);
  }
}

__global__ void k_st_determined_sign(const int* acc, uint8_t* R, uint64_t n) {
  R[2 * n] = uint8_t((*acc % 4) == 2);
}

// ---- host: Clifford recognition up to global phase (stabilizer.rs:476-563) ----

struct Cx {
  double re, im;
};
Cx cx_mul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
double cx_abs(Cx a) { return std::hypot(a.re, a.im); }

bool phase_aligned(const double* a, const double* b, int len) {
  const double eps = 1e-9;
  int p = -1;
  for (int i = 0; i < len; ++i)
    if (std::hypot(b[2 * i], b[2 * i + 1]) > eps) {
      p = i;
      break;
    }
  if (p < 0) {
    for (int i = 0; i < len; ++i)
      if (std::hypot(a[2 * i], a[2 * i + 1]) > eps) return false;
    return true;
  }
  if (std::hypot(a[2 * p], a[2 * p + 1]) <= eps) return false;
  const Cx ap{a[2 * p], a[2 * p + 1]}, bp{b[2 * p], b[2 * p + 1]};
  const double ns = bp.re * bp.re + bp.im * bp.im;
  const Cx num = cx_mul(ap, Cx{bp.re, -bp.im});
  const Cx phase{num.re / ns, num.im / ns};
  if (std::fabs(cx_abs(phase) - 1.0) > eps) return false;
  for (int i = 0; i < len; ++i) {
    const Cx pb = cx_mul(phase, Cx{b[2 * i], b[2 * i + 1]});
    if (std::hypot(a[2 * i] - pb.re, a[2 * i + 1] - pb.im) > eps) return false;
  }
  return true;
}

const double kI[8] = {1, 0, 0, 0, 0, 0, 1, 0}, kX[8] = {0, 0, 1, 0, 1, 0, 0, 0},
             kY[8] = {0, 0, 0, -1, 0, 1, 0, 0}, kZ[8] = {1, 0, 0, 0, 0, 0, -1, 0},
             kS[8] = {1, 0, 0, 0, 0, 0, 0, 1}, kSdg[8] = {1, 0, 0, 0, 0, 0, 0, -1};
const double kH = 0.7071067811865476;  // FRAC_1_SQRT_2
const double kHm[8] = {kH, 0, kH, 0, kH, 0, -kH, 0};
const double kCnot[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                          0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0};
const double kCz[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                        0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, -1, 0};
const double kSwap[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0,
                          0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0};

bool clifford1(const double* m, uint32_t t, std::vector<Prim>* out) {
  if (phase_aligned(m, kI, 4)) return true;
  const struct {
    const double* ref;
    uint32_t kind;
  } table[] = {{kHm, PR_H}, {kS, PR_S}, {kSdg, PR_SDG}, {kX, PR_X}, {kY, PR_Y}, {kZ, PR_Z}};
  for (const auto& e : table)
    if (phase_aligned(m, e.ref, 4)) {
      out->push_back(Prim{e.kind, t, 0, 0});
      return true;
    }
  return false;
}

bool clifford2(const double* m, uint32_t a, uint32_t b, std::vector<Prim>* out) {
  if (phase_aligned(m, kCnot, 16)) {
    out->push_back(Prim{PR_CNOT, a, b, 0});
    return true;
  }
  if (phase_aligned(m, kCz, 16)) {
    out->push_back(Prim{PR_H, b, 0, 0});
    out->push_back(Prim{PR_CNOT, a, b, 0});
    out->push_back(Prim{PR_H, b, 0, 0});
    return true;
  }
  if (phase_aligned(m, kSwap, 16)) {
    out->push_back(Prim{PR_CNOT, a, b, 0});
    out->push_back(Prim{PR_CNOT, b, a, 0});
    out->push_back(Prim{PR_CNOT, a, b, 0});
    return true;
  }
  return false;
}

bool controlled_clifford(const double* m, uint32_t c, uint32_t t, std::vector<Prim>* out) {
  if (phase_aligned(m, kX, 4)) {
    out->push_back(Prim{PR_CNOT, c, t, 0});
    return true;
  }
  if (phase_aligned(m, kZ, 4)) {
    out->push_back(Prim{PR_H, t, 0, 0});
    out->push_back(Prim{PR_CNOT, c, t, 0});
    out->push_back(Prim{PR_H, t, 0, 0});
    return true;
  }
  return phase_aligned(m, kI, 4);
}

struct StRun {
  ev_stab* t;
  std::vector<Prim> pending;
  Prim* dprims = nullptr;  // device gate list
  Prim* hprims = nullptr;  // pinned staging; reused only after a synchronising measurement
  size_t dcap = 0;
  Rng rng;
  const char* poison = nullptr;
  explicit StRun(uint64_t seed) : rng(seed) {}
  ~StRun() {
    if (dprims) cudaFreeAsync(dprims, t->stream);
    cudaStreamSynchronize(t->stream);
    if (hprims) cudaFreeHost(hprims);
  }
};

unsigned blocks_for(uint64_t work) { return unsigned((work + kStThreads - 1) / kStThreads); }

int flush(StRun* s) {
  if (s->pending.empty()) return EV_OK;
  ev_stab* t = s->t;
  const size_t count = s->pending.size();
  if (count > s->dcap) {
    // the previous staging may still be read by an earlier copy
    EV_CUDA(cudaStreamSynchronize(t->stream));
    if (s->dprims) cudaFreeAsync(s->dprims, t->stream);
    if (s->hprims) cudaFreeHost(s->hprims);
    s->dprims = nullptr;
    s->hprims = nullptr;
    s->dcap = std::max<size_t>(count, 4096);
    EV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&s->dprims), s->dcap * sizeof(Prim), t->stream));
    EV_CUDA(cudaMallocHost(reinterpret_cast<void**>(&s->hprims), s->dcap * sizeof(Prim)));
  }
  std::memcpy(s->hprims, s->pending.data(), count * sizeof(Prim));
  EV_CUDA(cudaMemcpyAsync(s->dprims, s->hprims, count * sizeof(Prim), cudaMemcpyHostToDevice,
                          t->stream));
  const uint64_t active = 2 * t->n;
  if (active)
    k_st_gates<<<blocks_for(active), kStThreads, 0, t->stream>>>(t->x, t->z, t->r, t->rows, active,
                                                                 s->dprims, int(count));
  EV_CUDA(cudaGetLastError());
  s->pending.clear();
  return EV_OK;
}

int measure(StRun* s, uint32_t q, bool* outcome) {
  EV_TRY(flush(s));
  ev_stab* t = s->t;
  const uint64_t n = t->n;
  const int none = INT_MAX;
  EV_CUDA(cudaMemcpyAsync(t->found, &none, sizeof(int), cudaMemcpyHostToDevice, t->stream));
  k_st_find<<<blocks_for(n), kStThreads, 0, t->stream>>>(t->x, t->rows, n, q, t->found);
  int p = none;
  EV_CUDA(cudaMemcpyAsync(&p, t->found, sizeof(int), cudaMemcpyDeviceToHost, t->stream));
  EV_CUDA(cudaStreamSynchronize(t->stream));
  if (p != none) {
    k_st_rowsum_all<<<blocks_for(2 * n), kStThreads, 0, t->stream>>>(t->x, t->z, t->r, t->rows, n,
                                                                     t->words, q, p);
    const int o = int(s->rng.next_u64() & 1);
    k_st_settle<<<blocks_for(t->words), kStThreads, 0, t->stream>>>(t->x, t->z, t->r, t->rows, n,
                                                                    t->words, q, p, o);
    EV_CUDA(cudaGetLastError());
    *outcome = o != 0;
    return EV_OK;
  }
  EV_CUDA(cudaMemsetAsync(t->found, 0, sizeof(int), t->stream));  // reused as the phase sum
  k_st_determined<<<blocks_for(t->words ? t->words : 1), kStThreads, 0, t->stream>>>(
      t->x, t->z, t->r, t->rows, n, t->words, q, t->found);
  k_st_determined_sign<<<1, 1, 0, t->stream>>>(t->found, t->r, n);
  EV_CUDA(cudaGetLastError());
  uint8_t r = 0;
  EV_CUDA(cudaMemcpyAsync(&r, t->r + 2 * n, 1, cudaMemcpyDeviceToHost, t->stream));
  EV_CUDA(cudaStreamSynchronize(t->stream));
  *outcome = r != 0;
  return EV_OK;
}

int apply_op(const ev_circuit* c, uint64_t* pos, StRun* s, uint8_t* classical) {
  const ev_op& op = c->ops[*pos];
  *pos += 1;
  switch (op.kind) {
    case EV_OP_APPLY1:
      if (!s->poison && !clifford1(op.m, uint32_t(op.q0), &s->pending))
        s->poison = "non-Clifford 1-qubit gate";
      return EV_OK;
    case EV_OP_APPLY2:
      if (!s->poison && !clifford2(op.m, uint32_t(op.q0), uint32_t(op.q1), &s->pending))
        s->poison = "non-Clifford 2-qubit gate";
      return EV_OK;
    case EV_OP_CONTROLLED:
      if (!s->poison &&
          !(op.nctrl == 1 && controlled_clifford(op.m, uint32_t(c->ctrl_pool[op.ctrl_off]),
                                                 uint32_t(op.q0), &s->pending)))
        s->poison = "non-Clifford controlled gate";
      return EV_OK;
    case EV_OP_MEASURE: {
      bool o = false;
      if (!s->poison) EV_TRY(measure(s, uint32_t(op.q0), &o));
      classical[op.q1] = o ? 1 : 0;
      return EV_OK;
    }
    case EV_OP_IF:
      if (classical[op.q0]) return apply_op(c, pos, s, classical);
      while (c->ops[*pos].kind == EV_OP_IF) *pos += 1;
      *pos += 1;
      return EV_OK;
  }
  return EV_OK;
}

__global__ void k_st_identity(uint64_t* X, uint64_t* Z, uint64_t rows, uint64_t n) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  X[(i >> 6) * rows + i] = uint64_t(1) << (i & 63);            // destabilizer i = X_i
  Z[(i >> 6) * rows + n + i] = uint64_t(1) << (i & 63);        // stabilizer i = Z_i
}

int stab_create(uint64_t n, ev_stab** out) {
  if (n > (uint64_t(1) << 24))
    return fail(EV_ERR_OOM, "a %llu-qubit tableau is beyond this engine's limit", (unsigned long long)n);
  ev_stab* t = new ev_stab();
  t->n = n;
  t->rows = 2 * n + 1;
  t->words = (n + 63) / 64;
  cudaGetDevice(&t->device);
  const size_t wbytes = size_t(t->rows) * size_t(t->words ? t->words : 1) * sizeof(uint64_t);
  cudaError_t e = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->x), wbytes);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->z), wbytes);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->r), size_t(t->rows) + 16);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->found), sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(t->x, 0, wbytes, t->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->z, 0, wbytes, t->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->r, 0, size_t(t->rows), t->stream);
  if (e == cudaSuccess && n) {
    k_st_identity<<<blocks_for(n), kStThreads, 0, t->stream>>>(t->x, t->z, t->rows, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ev_stab_destroy(t);
    return fail(e == cudaErrorMemoryAllocation ? EV_ERR_OOM : EV_ERR_CUDA, "tableau setup: %s",
                cudaGetErrorString(e));
  }
  *out = t;
  return EV_OK;
}

}  // namespace
}  // namespace ev

using namespace ev;

// Destroying never fails and leaves the last error message in place (a run
// that fails frees its own state before returning the error).
extern "C" int ev_stab_destroy(ev_stab* t) {
  if (!t) return EV_OK;
  cudaSetDevice(t->device);
  if (t->stream) cudaStreamSynchronize(t->stream);
  cudaFree(t->x);
  cudaFree(t->z);
  cudaFree(t->r);
  cudaFree(t->found);
  if (t->stream) cudaStreamDestroy(t->stream);
  cudaGetLastError();
  delete t;
  return EV_OK;
}

extern "C" int ev_stab_num_qubits(const ev_stab* t, uint64_t* out) {
  clear_error();
  if (!t || !out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_stab_num_qubits: null argument");
  *out = t->n;
  return EV_OK;
}

extern "C" int ev_stab_generators(const ev_stab* t, uint8_t* x, uint8_t* z, uint8_t* neg) {
  clear_error();
  if (!t || (t->n && (!x || !z || !neg)))
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_stab_generators: null argument");
  const uint64_t n = t->n, W = t->words, rows = t->rows;
  if (n == 0) return EV_OK;
  EV_CUDA(cudaSetDevice(t->device));
  std::vector<uint64_t> hx(rows * W), hz(rows * W);
  std::vector<uint8_t> hr(rows);
  EV_CUDA(cudaMemcpyAsync(hx.data(), t->x, hx.size() * 8, cudaMemcpyDeviceToHost, t->stream));
  EV_CUDA(cudaMemcpyAsync(hz.data(), t->z, hz.size() * 8, cudaMemcpyDeviceToHost, t->stream));
  EV_CUDA(cudaMemcpyAsync(hr.data(), t->r, rows, cudaMemcpyDeviceToHost, t->stream));
  EV_CUDA(cudaStreamSynchronize(t->stream));
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t row = n + i;
    for (uint64_t q = 0; q < n; ++q) {
      x[i * n + q] = uint8_t((hx[(q >> 6) * rows + row] >> (q & 63)) & 1);
      z[i * n + q] = uint8_t((hz[(q >> 6) * rows + row] >> (q & 63)) & 1);
    }
    neg[i] = hr[row];
  }
  return EV_OK;
}

extern "C" int ev_validate(const ev_circuit* c);

extern "C" int ev_stab_run(const ev_circuit* c, uint64_t seed, ev_stab** out,
                           uint8_t* classical_out) {
  clear_error();
  EV_TRY(ev_validate(c));
  if (!out || (c->num_classical && !classical_out))
    return fail(EV_ERR_INVALID_ARGUMENT, "ev_stab_run: null output");
  ev_stab* t = nullptr;
  EV_TRY(stab_create(c->num_qubits, &t));
  std::vector<uint8_t> classical(c->num_classical + 1, 0);
  int rc = EV_OK;
  {
    StRun s(seed);
    s.t = t;
    uint64_t pos = 0;
    while (pos < c->nops && rc == EV_OK) rc = apply_op(c, &pos, &s, classical.data());
    if (rc == EV_OK) rc = flush(&s);
    if (rc == EV_OK && s.poison)
      rc = fail(EV_ERR_NON_CLIFFORD,
                "%s is not in the Clifford group; the stabilizer backend cannot simulate it",
                s.poison);
  }
  if (rc == EV_OK) {
    const cudaError_t e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) rc = fail(EV_ERR_CUDA, "ev_stab_run: %s", cudaGetErrorString(e));
  }
  if (rc != EV_OK) {
    ev_stab_destroy(t);
    return rc;
  }
  if (c->num_classical) std::memcpy(classical_out, classical.data(), c->num_classical);
  *out = t;
  return EV_OK;
}
