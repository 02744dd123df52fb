// ev_oracle.cpp -- CPU restatement of everett's dense statevector path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
// engine: it restates, in scalar C++, the arithmetic of the reference crate
// (hz2/everett 0.1.2) that the engine must reproduce.  Only the test suite,
// the smoke check and the CPU-baseline leg of the benchmark may load it; the
// engine itself never calls it.
//
// Pinning.  The reference is Rust and no Rust toolchain exists where this is
// built, so the oracle is pinned against the reference's own known-answer
// tests (kernel.rs:515-770, measure.rs:59-106, state.rs:192-234,
// tests/algorithms_*.rs, tests/properties.rs), re-expressed in
// tests/test_oracle.py.  The xoshiro256++ stream has no golden values in the
// reference (rng.rs:62-95 tests only determinism, range and mean); the tests
// pin it to the published output vectors of SplitMix64 and xoshiro256++
// (oracle_rng_seed_words, oracle_rng_raw).
//
// Build: -O2 -ffp-contract=off (no implicit FMA contraction), with std::fma
// wherever the Rust source calls mul_add, so every rounding step matches the
// reference's.  Loops that the reference runs sequentially stay sequential
// unless noted; the OpenMP pragmas only split loops whose iterations are
// independent (each amplitude pair / quad is written by exactly one
// iteration), so the parallel build produces bit-identical results.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <vector>

#include "../include/everett_cuda.h"

namespace {

// ---- Complex64 (src/complex.rs:22-124) ------------------------------------
struct C {
  double re, im;
};

// (a + bi)(c + di): re = fma(a, c, -(b*d)), im = fma(a, d, b*c)
// (complex.rs:115-124).
inline C cmul(C a, C b) {
  return C{std::fma(a.re, b.re, -(a.im * b.im)), std::fma(a.re, b.im, a.im * b.re)};
}
inline C cadd(C a, C b) { return C{a.re + b.re, a.im + b.im}; }
inline C conj(C a) { return C{a.re, -a.im}; }
// norm_sqr = re.mul_add(re, im*im) (complex.rs:80-82).
inline double norm_sqr(C a) { return std::fma(a.re, a.re, a.im * a.im); }
// Complex64 * f64 (complex.rs:127-133).
inline C cscale(C a, double s) { return C{a.re * s, a.im * s}; }

inline C ld(const double* m, int i) { return C{m[2 * i], m[2 * i + 1]}; }

// ---- index math (src/kernel.rs:39-66) --------------------------------------
inline void index_pair(uint64_t k, uint64_t i, uint64_t* i0, uint64_t* i1) {
  const uint64_t low_mask = (uint64_t(1) << k) - 1;
  *i0 = ((i >> k) << (k + 1)) | (i & low_mask);
  *i1 = *i0 | (uint64_t(1) << k);
}

inline void index_quad(uint64_t a, uint64_t b, uint64_t i, uint64_t idx[4]) {
  const uint64_t lo = a < b ? a : b, hi = a < b ? b : a;
  const uint64_t low_mask = (uint64_t(1) << lo) - 1;
  const uint64_t t = ((i >> lo) << (lo + 1)) | (i & low_mask);
  const uint64_t mid_mask = (uint64_t(1) << hi) - 1;
  const uint64_t base = ((t >> hi) << (hi + 1)) | (t & mid_mask);
  const uint64_t bit_a = uint64_t(1) << a, bit_b = uint64_t(1) << b;
  idx[0] = base;
  idx[1] = base | bit_b;
  idx[2] = base | bit_a;
  idx[3] = base | bit_a | bit_b;
}

// ---- Gate2 constants used by the exact-match dispatch (gate.rs:189-232) ----
bool is_perm2(const double* m, const int rows[4], double last_sign) {
  // matrix with a single 1 per row at column rows[r] (times last_sign on row 3)
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double want = (c == rows[r]) ? (r == 3 ? last_sign : 1.0) : 0.0;
      if (!(m[2 * (4 * r + c)] == want && m[2 * (4 * r + c) + 1] == 0.0)) return false;
    }
  return true;
}
const int kCnotRows[4] = {0, 1, 3, 2};
const int kIdRows[4] = {0, 1, 2, 3};
const int kSwapRows[4] = {0, 2, 1, 3};

// ---- Rng: xoshiro256++ seeded by SplitMix64 (src/rng.rs:18-58) -------------
struct Rng {
  uint64_t s[4];
  Rng(uint64_t s0, uint64_t s1, uint64_t s2, uint64_t s3) : s{s0, s1, s2, s3} {}
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
  // (u64 >> 11) * 2^-53 (rng.rs:52-56).
  double next_f64() { return double(next_u64() >> 11) * (1.0 / double(uint64_t(1) << 53)); }
};

// ---- kernels ----------------------------------------------------------------

// apply_1q_scalar (kernel.rs:100-119).  The reference's AVX2 branch is never
// taken on the aarch64 host and is pinned equal to this one (kernel.rs:728).
void apply_1q(C* amps, uint64_t len, uint64_t k, const double* mm) {
  const C m0 = ld(mm, 0), m1 = ld(mm, 1), m2 = ld(mm, 2), m3 = ld(mm, 3);
  const int64_t pairs = int64_t(len / 2);
#pragma omp parallel for schedule(static) if (pairs >= (1 << 16))
  for (int64_t i = 0; i < pairs; ++i) {
    uint64_t i0, i1;
    index_pair(k, uint64_t(i), &i0, &i1);
    const C a0 = amps[i0], a1 = amps[i1];
    amps[i0] = cadd(cmul(m0, a0), cmul(m1, a1));
    amps[i1] = cadd(cmul(m2, a0), cmul(m3, a1));
  }
}

// dense 4x4 quad loop (kernel.rs:214-243): rows in index_quad order, each row
// summed left to right.
void apply_2q_dense(C* amps, uint64_t len, uint64_t a, uint64_t b, const double* mm) {
  const int64_t groups = int64_t(len / 4);
#pragma omp parallel for schedule(static) if (groups >= (1 << 15))
  for (int64_t i = 0; i < groups; ++i) {
    uint64_t idx[4];
    index_quad(a, b, uint64_t(i), idx);
    const C amp[4] = {amps[idx[0]], amps[idx[1]], amps[idx[2]], amps[idx[3]]};
    for (int row = 0; row < 4; ++row) {
      C acc = cmul(ld(mm, row * 4 + 0), amp[0]);
      acc = cadd(acc, cmul(ld(mm, row * 4 + 1), amp[1]));
      acc = cadd(acc, cmul(ld(mm, row * 4 + 2), amp[2]));
      acc = cadd(acc, cmul(ld(mm, row * 4 + 3), amp[3]));
      amps[idx[row]] = acc;
    }
  }
}

// apply_2q with the exact-match dispatch (kernel.rs:192-289).
void apply_2q(C* amps, uint64_t len, uint64_t a, uint64_t b, const double* mm) {
  const int64_t groups = int64_t(len / 4);
  if (is_perm2(mm, kCnotRows, 1.0)) {  // swap i10 <-> i11 (kernel.rs:248-260)
#pragma omp parallel for schedule(static) if (groups >= (1 << 15))
    for (int64_t i = 0; i < groups; ++i) {
      uint64_t idx[4];
      index_quad(a, b, uint64_t(i), idx);
      const C tmp = amps[idx[2]];
      amps[idx[2]] = amps[idx[3]];
      amps[idx[3]] = tmp;
    }
    return;
  }
  if (is_perm2(mm, kIdRows, -1.0)) {  // CZ: negate i11 (kernel.rs:263-274)
#pragma omp parallel for schedule(static) if (groups >= (1 << 15))
    for (int64_t i = 0; i < groups; ++i) {
      uint64_t idx[4];
      index_quad(a, b, uint64_t(i), idx);
      amps[idx[3]] = C{-amps[idx[3]].re, -amps[idx[3]].im};
    }
    return;
  }
  if (is_perm2(mm, kSwapRows, 1.0)) {  // swap i01 <-> i10 (kernel.rs:277-289)
#pragma omp parallel for schedule(static) if (groups >= (1 << 15))
    for (int64_t i = 0; i < groups; ++i) {
      uint64_t idx[4];
      index_quad(a, b, uint64_t(i), idx);
      const C tmp = amps[idx[1]];
      amps[idx[1]] = amps[idx[2]];
      amps[idx[2]] = tmp;
    }
    return;
  }
  apply_2q_dense(amps, len, a, b, mm);
}

// apply_controlled_1q_scalar (kernel.rs:332-358): full sweep over pairs with
// a mask test on i0.
void apply_controlled(C* amps, uint64_t len, uint64_t mask, uint64_t target,
                      const double* mm) {
  const C m0 = ld(mm, 0), m1 = ld(mm, 1), m2 = ld(mm, 2), m3 = ld(mm, 3);
  const int64_t pairs = int64_t(len / 2);
#pragma omp parallel for schedule(static) if (pairs >= (1 << 16))
  for (int64_t i = 0; i < pairs; ++i) {
    uint64_t i0, i1;
    index_pair(target, uint64_t(i), &i0, &i1);
    if ((i0 & mask) == mask) {
      const C a0 = amps[i0], a1 = amps[i1];
      amps[i0] = cadd(cmul(m0, a0), cmul(m1, a1));
      amps[i1] = cadd(cmul(m2, a0), cmul(m3, a1));
    }
  }
}

// measure_qubit (measure.rs:15-51): sequential p1 sum from 0.0, outcome =
// u < p1, scale = 1/sqrt(surviving) or 0, zero the other half.
int measure_qubit(C* amps, uint64_t len, uint64_t k, double u) {
  const uint64_t bit = uint64_t(1) << k;
  double p1 = 0.0;
  for (uint64_t j = 0; j < len; ++j)
    if (j & bit) p1 += norm_sqr(amps[j]);
  const bool outcome = u < p1;
  const double surviving = outcome ? p1 : 1.0 - p1;
  const double scale = surviving > 0.0 ? 1.0 / std::sqrt(surviving) : 0.0;
  const int64_t n = int64_t(len);
#pragma omp parallel for schedule(static) if (n >= (1 << 16))
  for (int64_t j = 0; j < n; ++j) {
    const bool keep = ((uint64_t(j) & bit) != 0) == outcome;
    amps[j] = keep ? cscale(amps[j], scale) : C{0.0, 0.0};
  }
  return outcome ? 1 : 0;
}

// State::norm_sqr: iterator sum, folded left to right from -0.0 (Rust's
// neutral element for f64 Sum) (state.rs:94-96).
double state_norm_sqr(const C* amps, uint64_t len) {
  double acc = -0.0;
  for (uint64_t j = 0; j < len; ++j) acc += norm_sqr(amps[j]);
  return acc;
}

// ---- op walk (src/backend/mod.rs:43-72, src/circuit.rs:245-306) ------------

int check_qubit(const ev_circuit* c, uint64_t q) {
  return q < c->num_qubits ? EV_OK : EV_ERR_QUBIT_OUT_OF_RANGE;
}
int check_classical(const ev_circuit* c, uint64_t b) {
  return b < c->num_classical ? EV_OK : EV_ERR_CLASSICAL_BIT_OUT_OF_RANGE;
}

// Validates the op starting at *pos (prefix-encoded IfClassic) and advances
// *pos past it.  Mirrors Circuit::validate_op (circuit.rs:252-284).
int validate_op(const ev_circuit* c, uint64_t* pos) {
  if (*pos >= c->nops) return EV_ERR_INVALID_ARGUMENT;
  const ev_op& op = c->ops[*pos];
  *pos += 1;
  int rc;
  switch (op.kind) {
    case EV_OP_APPLY1:
      return check_qubit(c, op.q0);
    case EV_OP_APPLY2:
      if ((rc = check_qubit(c, op.q0))) return rc;
      if ((rc = check_qubit(c, op.q1))) return rc;
      return op.q0 == op.q1 ? EV_ERR_DUPLICATE_QUBIT : EV_OK;
    case EV_OP_CONTROLLED:
      if ((rc = check_qubit(c, op.q0))) return rc;
      if (op.ctrl_off + op.nctrl > c->pool_len) return EV_ERR_INVALID_ARGUMENT;
      for (uint32_t j = 0; j < op.nctrl; ++j) {
        const uint64_t q = c->ctrl_pool[op.ctrl_off + j];
        if ((rc = check_qubit(c, q))) return rc;
        if (q == op.q0) return EV_ERR_DUPLICATE_QUBIT;
      }
      return EV_OK;
    case EV_OP_MEASURE:
      if ((rc = check_qubit(c, op.q0))) return rc;
      return check_classical(c, op.q1);
    case EV_OP_IF:
      if ((rc = check_classical(c, op.q0))) return rc;
      return validate_op(c, pos);
    default:
      return EV_ERR_INVALID_ARGUMENT;
  }
}

// apply_op (backend/mod.rs:51-72).  Returns the index after the op.
uint64_t run_op(const ev_circuit* c, uint64_t pos, C* amps, uint64_t len, Rng* rng,
                uint8_t* classical, bool active) {
  const ev_op& op = c->ops[pos];
  if (op.kind == EV_OP_IF) {
    const bool take = active && classical[op.q0] != 0;
    return run_op(c, pos + 1, amps, len, rng, classical, take);
  }
  if (active) {
    switch (op.kind) {
      case EV_OP_APPLY1:
        apply_1q(amps, len, op.q0, op.m);
        break;
      case EV_OP_APPLY2:
        apply_2q(amps, len, op.q0, op.q1, op.m);
        break;
      case EV_OP_CONTROLLED: {
        uint64_t mask = 0;
        for (uint32_t j = 0; j < op.nctrl; ++j) mask |= uint64_t(1) << c->ctrl_pool[op.ctrl_off + j];
        apply_controlled(amps, len, mask, op.q0, op.m);
        break;
      }
      case EV_OP_MEASURE:
        classical[op.q1] = uint8_t(measure_qubit(amps, len, op.q0, rng->next_f64()));
        break;
    }
  }
  return pos + 1;
}

}  // namespace

extern "C" {

// ---- gate constructors (src/gate.rs:54-136) ---------------------------------
// Matrices are built on the host with libm sin/cos, exactly as the reference
// builds them; the engine receives matrices, never angles.
static void put(double* m, int i, double re, double im) {
  m[2 * i] = re;
  m[2 * i + 1] = im;
}
void oracle_gate_h(double* m) {
  const double s = 0.70710678118654752440;  // FRAC_1_SQRT_2
  put(m, 0, s, 0); put(m, 1, s, 0); put(m, 2, s, 0); put(m, 3, -s, 0);
}
void oracle_gate_rx(double t, double* m) {  // gate.rs:106-110
  const double s = std::sin(t / 2.0), co = std::cos(t / 2.0);
  put(m, 0, co, 0); put(m, 1, 0, -s); put(m, 2, 0, -s); put(m, 3, co, 0);
}
void oracle_gate_ry(double t, double* m) {  // gate.rs:114-118
  const double s = std::sin(t / 2.0), co = std::cos(t / 2.0);
  put(m, 0, co, 0); put(m, 1, -s, 0); put(m, 2, s, 0); put(m, 3, co, 0);
}
void oracle_gate_rz(double t, double* m) {  // gate.rs:122-130: expi(-t/2), expi(t/2)
  put(m, 0, std::cos(-t / 2.0), std::sin(-t / 2.0)); put(m, 1, 0, 0); put(m, 2, 0, 0);
  put(m, 3, std::cos(t / 2.0), std::sin(t / 2.0));
}
void oracle_gate_phase(double l, double* m) {  // gate.rs:134-136
  put(m, 0, 1, 0); put(m, 1, 0, 0); put(m, 2, 0, 0); put(m, 3, std::cos(l), std::sin(l));
}

// ---- kernels on a caller-owned interleaved buffer ----------------------------
void oracle_apply_1q(double* amps, uint64_t len, uint64_t k, const double* m) {
  apply_1q(reinterpret_cast<C*>(amps), len, k, m);
}
void oracle_apply_2q(double* amps, uint64_t len, uint64_t a, uint64_t b, const double* m) {
  apply_2q(reinterpret_cast<C*>(amps), len, a, b, m);
}
void oracle_apply_2q_dense(double* amps, uint64_t len, uint64_t a, uint64_t b,
                           const double* m) {
  apply_2q_dense(reinterpret_cast<C*>(amps), len, a, b, m);
}
void oracle_apply_controlled_1q(double* amps, uint64_t len, const uint64_t* controls,
                                uint64_t nctrl, uint64_t target, const double* m) {
  uint64_t mask = 0;
  for (uint64_t j = 0; j < nctrl; ++j) mask |= uint64_t(1) << controls[j];
  apply_controlled(reinterpret_cast<C*>(amps), len, mask, target, m);
}
int oracle_measure_qubit(double* amps, uint64_t len, uint64_t k, double u) {
  return measure_qubit(reinterpret_cast<C*>(amps), len, k, u);
}

// ---- State observables (src/state.rs:94-185) ---------------------------------
double oracle_norm_sqr(const double* amps, uint64_t len) {
  return state_norm_sqr(reinterpret_cast<const C*>(amps), len);
}
void oracle_normalize(double* amps, uint64_t len) {  // state.rs:103-111
  C* a = reinterpret_cast<C*>(amps);
  const double norm = std::sqrt(state_norm_sqr(a, len));
  if (norm > 0.0) {
    const double inv = 1.0 / norm;
    for (uint64_t j = 0; j < len; ++j) a[j] = cscale(a[j], inv);
  }
}
// most_probable_phase's marginal (phase_estimation.rs:97-110): one pass over
// the basis in increasing order, marginal[basis & (2^m - 1)] += norm_sqr, each
// entry starting from 0.0.
void oracle_marginal_low(const double* amps, uint64_t len, uint64_t m, double* out) {
  const C* a = reinterpret_cast<const C*>(amps);
  const uint64_t count = uint64_t(1) << m;
  for (uint64_t c = 0; c < count; ++c) out[c] = 0.0;
  for (uint64_t j = 0; j < len; ++j) out[j & (count - 1)] += norm_sqr(a[j]);
}
// <other|self> = sum conj(other_j) * self_j, accumulated from ZERO (state.rs:130-138).
void oracle_overlap(const double* self, const double* other, uint64_t len, double* out) {
  const C* a = reinterpret_cast<const C*>(self);
  const C* b = reinterpret_cast<const C*>(other);
  C acc{0.0, 0.0};
  for (uint64_t j = 0; j < len; ++j) acc = cadd(acc, cmul(conj(b[j]), a[j]));
  out[0] = acc.re;
  out[1] = acc.im;
}
// PauliString::expectation (backend/stabilizer.rs:79-125): P applied to a
// copy (phase i^(#Y) times the sign, X flips, Z signs), then
// Re <P psi | psi> by State::overlap.
double oracle_pauli_expectation(const double* amps, uint64_t n, uint64_t xmask, uint64_t zmask,
                                int negative) {
  const C* a = reinterpret_cast<const C*>(amps);
  const uint64_t dim = uint64_t(1) << n;
  uint64_t ycount = 0;
  for (uint64_t q = 0; q < n; ++q)
    if (((xmask >> q) & 1) && ((zmask >> q) & 1)) ++ycount;
  C phase{1.0, 0.0};
  switch (ycount % 4) {
    case 1: phase = C{0.0, 1.0}; break;
    case 2: phase = C{-1.0, 0.0}; break;
    case 3: phase = C{0.0, -1.0}; break;
    default: break;
  }
  const double sign = negative ? -1.0 : 1.0;
  const C factor = cscale(phase, sign);
  std::vector<C> out(dim, C{0.0, 0.0});
  for (uint64_t j = 0; j < dim; ++j) {
    uint64_t target = j;
    double zsign = 1.0;
    for (uint64_t q = 0; q < n; ++q) {
      if ((xmask >> q) & 1) target ^= uint64_t(1) << q;
      if (((zmask >> q) & 1) && ((j >> q) & 1)) zsign = -zsign;
    }
    out[target] = cadd(out[target], cscale(cmul(a[j], factor), zsign));
  }
  double ov[2];
  oracle_overlap(amps, reinterpret_cast<const double*>(out.data()), dim, ov);
  return ov[0];
}
void oracle_bloch_vector(const double* amps, uint64_t len, uint64_t qubit, double* out) {
  const C* a = reinterpret_cast<const C*>(amps);
  const uint64_t bit = uint64_t(1) << qubit;
  double r00 = 0.0, r11 = 0.0;
  C r01{0.0, 0.0};
  for (uint64_t j = 0; j < len; ++j) {
    if ((j & bit) == 0) {
      r00 += norm_sqr(a[j]);
      r01 = cadd(r01, cmul(a[j], conj(a[j | bit])));
    } else {
      r11 += norm_sqr(a[j]);
    }
  }
  out[0] = 2.0 * r01.re;
  out[1] = 2.0 * r01.im;
  out[2] = r00 - r11;
}

// ---- Rng -------------------------------------------------------------------
void oracle_rng_u64(uint64_t seed, uint64_t count, uint64_t* out) {
  Rng r(seed);
  for (uint64_t j = 0; j < count; ++j) out[j] = r.next_u64();
}
void oracle_rng_f64(uint64_t seed, uint64_t count, double* out) {
  Rng r(seed);
  for (uint64_t j = 0; j < count; ++j) out[j] = r.next_f64();
}
// The generator step alone, from a raw state (no SplitMix64 seeding), and the
// four seeding words seed_from_u64 derives: the two halves of the stream that
// the tests pin to the algorithms' published output vectors.
void oracle_rng_raw(const uint64_t* state, uint64_t count, uint64_t* out) {
  Rng r(state[0], state[1], state[2], state[3]);
  for (uint64_t j = 0; j < count; ++j) out[j] = r.next_u64();
}
void oracle_rng_seed_words(uint64_t seed, uint64_t* words) {
  const Rng r(seed);
  for (int w = 0; w < 4; ++w) words[w] = r.s[w];
}

// ---- circuits ----------------------------------------------------------------
int oracle_validate(const ev_circuit* c) {
  uint64_t pos = 0;
  while (pos < c->nops) {
    const int rc = validate_op(c, &pos);
    if (rc) return rc;
  }
  return EV_OK;
}

// StateVectorBackend::run_seeded (statevector.rs:77-90): validate, |0..0>,
// Rng::seed_from_u64(seed), drive.  amps_out holds 2^n complex.
int oracle_run_seeded(const ev_circuit* c, uint64_t seed, double* amps_out,
                      uint8_t* classical_out) {
  const int rc = oracle_validate(c);
  if (rc) return rc;
  const uint64_t len = uint64_t(1) << c->num_qubits;
  C* amps = reinterpret_cast<C*>(amps_out);
  for (uint64_t j = 0; j < len; ++j) amps[j] = C{0.0, 0.0};
  amps[0] = C{1.0, 0.0};
  Rng rng(seed);
  for (uint64_t j = 0; j < c->num_classical; ++j) classical_out[j] = 0;
  uint64_t pos = 0;
  while (pos < c->nops) pos = run_op(c, pos, amps, len, &rng, classical_out, true);
  return EV_OK;
}

// Runs ops [first, last) of a circuit on an existing buffer with no
// measurement (used to time a bounded sample of a circuit).
void oracle_apply_ops(const ev_circuit* c, uint64_t first, uint64_t last, double* amps_io) {
  const uint64_t len = uint64_t(1) << c->num_qubits;
  Rng rng(0);
  std::vector<uint8_t> classical(c->num_classical + 1, 0);
  uint64_t pos = first;
  while (pos < last) pos = run_op(c, pos, reinterpret_cast<C*>(amps_io), len, &rng, classical.data(), true);
}

// ---- shot sampling -----------------------------------------------------------
// Literal form of the shot contract: for each shot, copy the state and call
// measure_qubit for qubits 0..n-1 with consecutive uniforms of one Rng.
// O(shots * n * 2^n); for small registers only.
void oracle_sample_literal(const double* amps, uint64_t n, uint64_t seed, uint64_t shots,
                           uint64_t* out) {
  const uint64_t len = uint64_t(1) << n;
  std::vector<C> work(len);
  Rng rng(seed);
  for (uint64_t s = 0; s < shots; ++s) {
    std::memcpy(work.data(), amps, len * sizeof(C));
    uint64_t bits = 0;
    for (uint64_t q = 0; q < n; ++q)
      if (measure_qubit(work.data(), len, q, rng.next_f64())) bits |= uint64_t(1) << q;
    out[s] = bits;
  }
}

// Conditional-mass form of the same contract.  mass[q][r] is the total
// probability of basis states whose low q bits equal r, built by pairwise
// sums: mass[n][j] = |a_j|^2 and mass[q][r] = mass[q+1][r] + mass[q+1][r+2^q].
// Qubit q of a shot whose earlier outcomes are r is 1 iff
// u < mass[q+1][r + 2^q] / mass[q][r]; a zero mass gives NaN and outcome 0,
// as measure_qubit's zero scale does.  Mathematically equal to the literal
// form; outcomes differ only where u lies within rounding of the boundary.
void oracle_sample_tree(const double* amps, uint64_t n, uint64_t seed, uint64_t shots,
                        uint64_t* out) {
  const uint64_t len = uint64_t(1) << n;
  const C* a = reinterpret_cast<const C*>(amps);
  std::vector<std::vector<double>> mass(n + 1);
  mass[n].resize(len);
  for (uint64_t j = 0; j < len; ++j) mass[n][j] = norm_sqr(a[j]);
  for (int64_t q = int64_t(n) - 1; q >= 0; --q) {
    const uint64_t w = uint64_t(1) << q;
    mass[q].resize(w);
    for (uint64_t r = 0; r < w; ++r) mass[q][r] = mass[q + 1][r] + mass[q + 1][r + w];
  }
  Rng rng(seed);
  for (uint64_t s = 0; s < shots; ++s) {
    uint64_t r = 0;
    for (uint64_t q = 0; q < n; ++q) {
      const double u = rng.next_f64();
      const double p1 = mass[q + 1][r + (uint64_t(1) << q)] / mass[q][r];
      if (u < p1) r |= uint64_t(1) << q;
    }
    out[s] = r;
  }
}


// ---- density matrices (src/density.rs, src/backend/density_matrix.rs) -------------
// Row-major 2^n x 2^n; every loop below follows the reference's order.

// index_group (density.rs:426-454): the 2^m indices whose non-target bits
// encode g; target bits inserted in sorted order, combinations in `targets`
// order.
static std::vector<uint64_t> dm_index_group(const std::vector<uint64_t>& targets, uint64_t g) {
  std::vector<uint64_t> sorted = targets;
  std::sort(sorted.begin(), sorted.end());
  uint64_t base = g;
  for (uint64_t t : sorted) {
    const uint64_t low = (uint64_t(1) << t) - 1;
    base = ((base >> t) << (t + 1)) | (base & low);
  }
  const uint64_t gd = uint64_t(1) << targets.size();
  std::vector<uint64_t> idx(gd);
  for (uint64_t k = 0; k < gd; ++k) {
    uint64_t v = base;
    for (size_t b = 0; b < targets.size(); ++b)
      if ((k >> b) & 1) v |= uint64_t(1) << targets[b];
    idx[k] = v;
  }
  return idx;
}

// left_multiply (density.rs:348-378): out = U rho.
static void dm_left(const std::vector<C>& rho, std::vector<C>& out, const std::vector<C>& u,
                    const std::vector<uint64_t>& targets, uint64_t n) {
  const uint64_t dim = uint64_t(1) << n, gd = uint64_t(1) << targets.size();
  for (uint64_t col = 0; col < dim; ++col)
    for (uint64_t g = 0; g < dim / gd; ++g) {
      const std::vector<uint64_t> rows = dm_index_group(targets, g);
      std::vector<C> in(gd);
      for (uint64_t c = 0; c < gd; ++c) in[c] = rho[rows[c] * dim + col];
      for (uint64_t r = 0; r < gd; ++r) {
        C acc{0.0, 0.0};
        for (uint64_t c = 0; c < gd; ++c) acc = cadd(acc, cmul(u[r * gd + c], in[c]));
        out[rows[r] * dim + col] = acc;
      }
    }
}

// right_multiply_adjoint[_add] (density.rs:381-421): out (+)= tmp U^dagger.
static void dm_right(const std::vector<C>& tmp, std::vector<C>& out, const std::vector<C>& u,
                     const std::vector<uint64_t>& targets, uint64_t n, bool add) {
  const uint64_t dim = uint64_t(1) << n, gd = uint64_t(1) << targets.size();
  for (uint64_t row = 0; row < dim; ++row)
    for (uint64_t g = 0; g < dim / gd; ++g) {
      const std::vector<uint64_t> cols = dm_index_group(targets, g);
      std::vector<C> in(gd);
      for (uint64_t c = 0; c < gd; ++c) in[c] = tmp[row * dim + cols[c]];
      for (uint64_t ci = 0; ci < gd; ++ci) {
        C acc{0.0, 0.0};
        for (uint64_t k = 0; k < gd; ++k) acc = cadd(acc, cmul(in[k], conj(u[ci * gd + k])));
        C& dst = out[row * dim + cols[ci]];
        dst = add ? cadd(dst, acc) : acc;
      }
    }
}

static void dm_unitary(std::vector<C>& rho, const std::vector<C>& u,
                       const std::vector<uint64_t>& targets, uint64_t n) {
  std::vector<C> out(rho.size(), C{0.0, 0.0});
  dm_left(rho, out, u, targets, n);
  dm_right(out, rho, u, targets, n, false);
}

// apply_channel (density.rs:195-215).
static void dm_channel(std::vector<C>& rho, const ev_channel& ch, uint64_t target, uint64_t n) {
  std::vector<C> acc(rho.size(), C{0.0, 0.0});
  for (uint32_t k = 0; k < ch.nops; ++k) {
    std::vector<C> u(4);
    for (int e = 0; e < 4; ++e) u[e] = C{ch.k[k][2 * e], ch.k[k][2 * e + 1]};
    std::vector<C> tmp(rho.size(), C{0.0, 0.0});
    dm_left(rho, tmp, u, {target}, n);
    dm_right(tmp, acc, u, {target}, n, true);
  }
  rho = acc;
}

static double dm_trace(const std::vector<C>& rho, uint64_t dim) {
  double t = 0.0;
  for (uint64_t i = 0; i < dim; ++i) t += rho[i * dim + i].re;
  return t;
}

struct DmRun {
  std::vector<C> rho;
  uint64_t n;
  const ev_noise_model* noise;
  Rng rng;
  uint8_t* classical;
};

// Backend for DensityMatrixBackend (density_matrix.rs:101-160).
static void dm_apply_op(const ev_circuit* c, uint64_t* pos, DmRun* r) {
  const ev_op& op = c->ops[*pos];
  *pos += 1;
  const uint64_t n = r->n, dim = uint64_t(1) << n;
  const ev_noise_model* nz = r->noise;
  switch (op.kind) {
    case EV_OP_APPLY1: {
      std::vector<C> u(4);
      for (int e = 0; e < 4; ++e) u[e] = ld(op.m, e);
      dm_unitary(r->rho, u, {op.q0}, n);
      if (nz && nz->after_1q.nops) dm_channel(r->rho, nz->after_1q, op.q0, n);
      return;
    }
    case EV_OP_APPLY2: {
      std::vector<C> u(16);
      for (int e = 0; e < 16; ++e) u[e] = ld(op.m, e);
      dm_unitary(r->rho, u, {op.q1, op.q0}, n);
      if (nz && nz->after_2q.nops) {
        dm_channel(r->rho, nz->after_2q, op.q0, n);
        dm_channel(r->rho, nz->after_2q, op.q1, n);
      }
      return;
    }
    case EV_OP_CONTROLLED: {
      // controlled_unitary (density_matrix.rs:195-228): the full 2^n x 2^n matrix
      uint64_t mask = 0;
      for (uint32_t j = 0; j < op.nctrl; ++j) mask |= uint64_t(1) << c->ctrl_pool[op.ctrl_off + j];
      std::vector<C> u(dim * dim, C{0.0, 0.0});
      const uint64_t t = op.q0;
      for (uint64_t col = 0; col < dim; ++col) {
        if ((col & mask) == mask) {
          const uint64_t partner = col ^ (uint64_t(1) << t);
          if (((col >> t) & 1) == 0) {
            u[col * dim + col] = ld(op.m, 0);
            u[partner * dim + col] = ld(op.m, 2);
          } else {
            u[partner * dim + col] = ld(op.m, 1);
            u[col * dim + col] = ld(op.m, 3);
          }
        } else {
          u[col * dim + col] = C{1.0, 0.0};
        }
      }
      std::vector<uint64_t> all(n);
      for (uint64_t q = 0; q < n; ++q) all[q] = q;
      dm_unitary(r->rho, u, all, n);
      if (nz && nz->after_1q.nops) {
        dm_channel(r->rho, nz->after_1q, t, n);
        for (uint32_t j = 0; j < op.nctrl; ++j)
          dm_channel(r->rho, nz->after_1q, c->ctrl_pool[op.ctrl_off + j], n);
      }
      return;
    }
    case EV_OP_MEASURE: {
      const uint64_t bit = uint64_t(1) << op.q0;
      double p1 = 0.0;  // measure_probability (density_matrix.rs:165-176)
      for (uint64_t j = 0; j < dim; ++j)
        if (j & bit) p1 += r->rho[j * dim + j].re;
      const bool raw = r->rng.next_f64() < p1;
      for (uint64_t i = 0; i < dim; ++i)  // collapse (density_matrix.rs:178-193)
        for (uint64_t j = 0; j < dim; ++j) {
          const bool im = ((i & bit) != 0) == raw, jm = ((j & bit) != 0) == raw;
          if (!im || !jm) r->rho[i * dim + j] = C{0.0, 0.0};
        }
      const double t = dm_trace(r->rho, dim);  // renormalize (density.rs:218-226)
      if (t > 0.0) {
        const double inv = 1.0 / t;
        for (C& x : r->rho) x = cscale(x, inv);
      }
      bool out = raw;
      if (nz && nz->readout_error > 0.0 && r->rng.next_f64() < nz->readout_error) out = !raw;
      r->classical[op.q1] = out ? 1 : 0;
      return;
    }
    case EV_OP_IF: {
      const bool take = r->classical[op.q0] != 0;
      if (take) {
        dm_apply_op(c, pos, r);
      } else {  // skip the inner record (and any nested IF prefixes)
        while (c->ops[*pos].kind == EV_OP_IF) *pos += 1;
        *pos += 1;
      }
      return;
    }
  }
}

int oracle_dm_run(const ev_circuit* c, const ev_noise_model* noise, uint64_t seed, double* rho_out,
                  uint8_t* classical_out) {
  const int rc = oracle_validate(c);
  if (rc) return rc;
  const uint64_t n = c->num_qubits, dim = uint64_t(1) << n;
  DmRun r{std::vector<C>(dim * dim, C{0.0, 0.0}), n, noise, Rng(seed), classical_out};
  r.rho[0] = C{1.0, 0.0};
  for (uint64_t j = 0; j < c->num_classical; ++j) classical_out[j] = 0;
  uint64_t pos = 0;
  while (pos < c->nops) dm_apply_op(c, &pos, &r);
  std::memcpy(rho_out, r.rho.data(), dim * dim * sizeof(C));
  return EV_OK;
}

void oracle_dm_from_amplitudes(const double* amps, uint64_t dim, double* rho_out) {
  const C* a = reinterpret_cast<const C*>(amps);
  C* rho = reinterpret_cast<C*>(rho_out);
  for (uint64_t i = 0; i < dim; ++i)
    for (uint64_t j = 0; j < dim; ++j) rho[i * dim + j] = cmul(a[i], conj(a[j]));
}

// trace, purity, expectation_pauli, partial_trace_1q (density.rs:117-295).
void oracle_dm_observables(const double* rho_in, uint64_t n, uint64_t qubit, double* out) {
  const C* rho = reinterpret_cast<const C*>(rho_in);
  const uint64_t dim = uint64_t(1) << n, bit = uint64_t(1) << qubit;
  std::vector<C> v(rho, rho + dim * dim);
  out[0] = dm_trace(v, dim);
  double pur = 0.0;
  for (uint64_t i = 0; i < dim; ++i)
    for (uint64_t j = 0; j < dim; ++j) pur += norm_sqr(rho[i * dim + j]);
  out[1] = pur;
  const char ops[4] = {'I', 'X', 'Y', 'Z'};
  for (int o = 0; o < 4; ++o) {
    C res{0.0, 0.0};
    for (uint64_t i = 0; i < dim; ++i)
      for (uint64_t j = 0; j < dim; ++j) {
        if ((i & ~bit) != (j & ~bit)) continue;
        const uint64_t iq = (i & bit) >> qubit, jq = (j & bit) >> qubit;
        C p{0.0, 0.0};
        switch (ops[o]) {
          case 'I': p = iq == jq ? C{1.0, 0.0} : C{0.0, 0.0}; break;
          case 'X': p = iq == jq ? C{0.0, 0.0} : C{1.0, 0.0}; break;
          case 'Y': p = (iq == 0 && jq == 1) ? C{0.0, -1.0} : (iq == 1 && jq == 0) ? C{0.0, 1.0} : C{0.0, 0.0}; break;
          default: p = (iq == 0 && jq == 0) ? C{1.0, 0.0} : (iq == 1 && jq == 1) ? C{-1.0, 0.0} : C{0.0, 0.0}; break;
        }
        if (p.re != 0.0 || p.im != 0.0) res = cadd(res, cmul(p, rho[j * dim + i]));
      }
    out[2 + o] = res.re;
  }
  C red[4] = {C{0, 0}, C{0, 0}, C{0, 0}, C{0, 0}};
  for (uint64_t i = 0; i < dim; ++i)
    for (uint64_t j = 0; j < dim; ++j) {
      if ((i & ~bit) != (j & ~bit)) continue;
      const uint64_t iq = (i & bit) >> qubit, jq = (j & bit) >> qubit;
      red[iq * 2 + jq] = cadd(red[iq * 2 + jq], rho[i * dim + j]);
    }
  for (int e = 0; e < 4; ++e) {
    out[6 + 2 * e] = red[e].re;
    out[7 + 2 * e] = red[e].im;
  }
}


// ---- stabilizer tableau (src/backend/stabilizer.rs) ---------------------------

enum StPrim { SP_H, SP_S, SP_SDG, SP_X, SP_Y, SP_Z, SP_CNOT };
struct StOp {
  StPrim k;
  uint64_t a, b;
};

struct Tableau {
  uint64_t n;
  std::vector<std::vector<uint8_t>> x, z;
  std::vector<uint8_t> r;
  Rng rng;
  int error = 0;
  Tableau(uint64_t n_, uint64_t seed) : n(n_), rng(seed) {  // identity (stabilizer.rs:231-250)
    const uint64_t rows = 2 * n + 1;
    x.assign(rows, std::vector<uint8_t>(n, 0));
    z.assign(rows, std::vector<uint8_t>(n, 0));
    r.assign(rows, 0);
    for (uint64_t i = 0; i < n; ++i) {
      x[i][i] = 1;
      z[n + i][i] = 1;
    }
  }
  void prim(const StOp& p) {  // stabilizer.rs:254-320
    const uint64_t a = p.a, b = p.b;
    for (uint64_t i = 0; i < 2 * n; ++i) {
      switch (p.k) {
        case SP_H: {
          r[i] ^= x[i][a] & z[i][a];
          std::swap(x[i][a], z[i][a]);
          break;
        }
        case SP_S:
          r[i] ^= x[i][a] & z[i][a];
          z[i][a] ^= x[i][a];
          break;
        case SP_SDG:
          r[i] ^= x[i][a] & z[i][a];
          z[i][a] ^= x[i][a];
          r[i] ^= x[i][a];
          break;
        case SP_X: r[i] ^= z[i][a]; break;
        case SP_Y: r[i] ^= x[i][a] ^ z[i][a]; break;
        case SP_Z: r[i] ^= x[i][a]; break;
        case SP_CNOT:
          r[i] ^= x[i][a] & z[i][b] & (x[i][b] ^ z[i][a] ^ 1);
          x[i][b] ^= x[i][a];
          z[i][a] ^= z[i][b];
          break;
      }
    }
  }
  static int g(int x1, int z1, int x2, int z2) {  // stabilizer.rs:381-390
    if (!x1 && !z1) return 0;
    if (x1 && z1) return z2 - x2;
    if (x1) return z2 * (2 * x2 - 1);
    return x2 * (1 - 2 * z2);
  }
  void rowsum(uint64_t h, uint64_t j) {  // stabilizer.rs:366-378
    int sum = 2 * r[h] + 2 * r[j];
    for (uint64_t q = 0; q < n; ++q) sum += g(x[j][q], z[j][q], x[h][q], z[h][q]);
    r[h] = (((sum % 4) + 4) % 4) == 2;
    for (uint64_t q = 0; q < n; ++q) {
      x[h][q] ^= x[j][q];
      z[h][q] ^= z[j][q];
    }
  }
  bool measure(uint64_t q) {  // stabilizer.rs:322-364
    uint64_t p = 2 * n;
    for (uint64_t i = n; i < 2 * n; ++i)
      if (x[i][q]) {
        p = i;
        break;
      }
    if (p < 2 * n) {
      for (uint64_t i = 0; i < 2 * n; ++i)
        if (i != p && x[i][q]) rowsum(i, p);
      x[p - n] = x[p];
      z[p - n] = z[p];
      r[p - n] = r[p];
      std::fill(x[p].begin(), x[p].end(), 0);
      std::fill(z[p].begin(), z[p].end(), 0);
      const bool outcome = (rng.next_u64() & 1) == 1;
      r[p] = outcome;
      z[p][q] = 1;
      return outcome;
    }
    const uint64_t s = 2 * n;
    std::fill(x[s].begin(), x[s].end(), 0);
    std::fill(z[s].begin(), z[s].end(), 0);
    r[s] = 0;
    for (uint64_t i = 0; i < n; ++i)
      if (x[i][q]) rowsum(s, n + i);
    return r[s] != 0;
  }
};

// up to global phase (stabilizer.rs:540-563), EPS = 1e-9
static bool st_phase_aligned(const C* a, const C* b, int len) {
  const double eps = 1e-9;
  int p = -1;
  for (int i = 0; i < len; ++i)
    if (std::hypot(b[i].re, b[i].im) > eps) {
      p = i;
      break;
    }
  if (p < 0) {
    for (int i = 0; i < len; ++i)
      if (std::hypot(a[i].re, a[i].im) > eps) return false;
    return true;
  }
  if (std::hypot(a[p].re, a[p].im) <= eps) return false;
  const double ns = norm_sqr(b[p]);
  const C num = cmul(a[p], conj(b[p]));
  const C phase{num.re / ns, num.im / ns};
  if (std::fabs(std::hypot(phase.re, phase.im) - 1.0) > eps) return false;
  for (int i = 0; i < len; ++i) {
    const C pb = cmul(phase, b[i]);
    if (std::hypot(a[i].re - pb.re, a[i].im - pb.im) > eps) return false;
  }
  return true;
}

static bool st_is1(const double* m, const double* ref) {
  C a[4], b[4];
  for (int e = 0; e < 4; ++e) {
    a[e] = ld(m, e);
    b[e] = ld(ref, e);
  }
  return st_phase_aligned(a, b, 4);
}

void oracle_gate_h(double* m);
static const double kStI[8] = {1, 0, 0, 0, 0, 0, 1, 0}, kStX[8] = {0, 0, 1, 0, 1, 0, 0, 0},
                    kStY[8] = {0, 0, 0, -1, 0, 1, 0, 0}, kStZ[8] = {1, 0, 0, 0, 0, 0, -1, 0},
                    kStS[8] = {1, 0, 0, 0, 0, 0, 0, 1}, kStSdg[8] = {1, 0, 0, 0, 0, 0, 0, -1};

// clifford1 (stabilizer.rs:497-515); returns false if not Clifford
static bool st_clifford1(const double* m, uint64_t t, std::vector<StOp>* out) {
  double h[8];
  oracle_gate_h(h);
  if (st_is1(m, kStI)) return true;
  if (st_is1(m, h)) return out->push_back({SP_H, t, 0}), true;
  if (st_is1(m, kStS)) return out->push_back({SP_S, t, 0}), true;
  if (st_is1(m, kStSdg)) return out->push_back({SP_SDG, t, 0}), true;
  if (st_is1(m, kStX)) return out->push_back({SP_X, t, 0}), true;
  if (st_is1(m, kStY)) return out->push_back({SP_Y, t, 0}), true;
  if (st_is1(m, kStZ)) return out->push_back({SP_Z, t, 0}), true;
  return false;
}

static bool st_clifford2(const double* m, uint64_t a, uint64_t b, std::vector<StOp>* out) {
  static const double cnot[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                                  0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0};
  static const double cz[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                                0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, -1, 0};
  static const double swp[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0,
                                 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0};
  C g[16], ref[16];
  for (int e = 0; e < 16; ++e) g[e] = ld(m, e);
  auto eq = [&](const double* r) {
    for (int e = 0; e < 16; ++e) ref[e] = ld(r, e);
    return st_phase_aligned(g, ref, 16);
  };
  if (eq(cnot)) return out->push_back({SP_CNOT, a, b}), true;
  if (eq(cz)) {
    out->push_back({SP_H, b, 0});
    out->push_back({SP_CNOT, a, b});
    out->push_back({SP_H, b, 0});
    return true;
  }
  if (eq(swp)) {
    out->push_back({SP_CNOT, a, b});
    out->push_back({SP_CNOT, b, a});
    out->push_back({SP_CNOT, a, b});
    return true;
  }
  return false;
}

struct StRun {
  Tableau t;
  uint8_t* classical;
  const char* poison = nullptr;
};

static void st_apply(const ev_circuit* c, uint64_t* pos, StRun* s) {
  const ev_op& op = c->ops[*pos];
  *pos += 1;
  std::vector<StOp> prims;
  switch (op.kind) {
    case EV_OP_APPLY1:
      if (s->poison) return;
      if (st_clifford1(op.m, op.q0, &prims))
        for (const StOp& p : prims) s->t.prim(p);
      else
        s->poison = "non-Clifford 1-qubit gate";
      return;
    case EV_OP_APPLY2:
      if (s->poison) return;
      if (st_clifford2(op.m, op.q0, op.q1, &prims))
        for (const StOp& p : prims) s->t.prim(p);
      else
        s->poison = "non-Clifford 2-qubit gate";
      return;
    case EV_OP_CONTROLLED: {
      if (s->poison) return;
      bool ok = false;
      if (op.nctrl == 1) {  // controlled_clifford (stabilizer.rs:529-546)
        const uint64_t ctl = c->ctrl_pool[op.ctrl_off], t = op.q0;
        if (st_is1(op.m, kStX)) {
          prims.push_back({SP_CNOT, ctl, t});
          ok = true;
        } else if (st_is1(op.m, kStZ)) {
          prims.push_back({SP_H, t, 0});
          prims.push_back({SP_CNOT, ctl, t});
          prims.push_back({SP_H, t, 0});
          ok = true;
        } else if (st_is1(op.m, kStI)) {
          ok = true;
        }
      }
      if (ok)
        for (const StOp& p : prims) s->t.prim(p);
      else
        s->poison = "non-Clifford controlled gate";
      return;
    }
    case EV_OP_MEASURE:
      s->classical[op.q1] = s->poison ? 0 : (s->t.measure(op.q0) ? 1 : 0);
      return;
    case EV_OP_IF:
      if (s->classical[op.q0]) {
        st_apply(c, pos, s);
      } else {
        while (c->ops[*pos].kind == EV_OP_IF) *pos += 1;
        *pos += 1;
      }
      return;
  }
}

// StabilizerBackend::run_seeded (stabilizer.rs:207-229): returns
// EV_ERR_NON_CLIFFORD if any gate was outside the Clifford set.
int oracle_stab_run(const ev_circuit* c, uint64_t seed, uint8_t* x_out, uint8_t* z_out,
                    uint8_t* neg_out, uint8_t* classical_out) {
  const int rc = oracle_validate(c);
  if (rc) return rc;
  const uint64_t n = c->num_qubits;
  StRun s{Tableau(n, seed), classical_out};
  for (uint64_t j = 0; j < c->num_classical; ++j) classical_out[j] = 0;
  uint64_t pos = 0;
  while (pos < c->nops) st_apply(c, &pos, &s);
  if (s.poison) return EV_ERR_NON_CLIFFORD;
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t q = 0; q < n; ++q) {
      x_out[i * n + q] = s.t.x[n + i][q];
      z_out[i * n + q] = s.t.z[n + i][q];
    }
    neg_out[i] = s.t.r[n + i];
  }
  return EV_OK;
}

}  // extern "C"
