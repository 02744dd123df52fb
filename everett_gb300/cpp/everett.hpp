// everett.hpp -- the C++ host side of the engine: everett's public Rust
// surface (hz2/everett src/lib.rs) restated over the C ABI of
// include/everett_cuda.h.
//
// Same names, argument meanings and errors as the reference:
//   Complex64 (src/complex.rs), Gate1 / Gate2 (src/gate.rs), Op and Circuit
//   (src/op.rs, src/circuit.rs), State (src/state.rs), Execution and
//   StateVectorBackend::run / run_seeded (src/backend/statevector.rs), Rng
//   (src/rng.rs), the circuit generators (src/algorithms), and the error
//   variants (src/error.rs).  Where Rust returns Result<T, Error> this header
//   throws everett::Error carrying the same variant; state and run calls go to
//   the GB300 engine, and the state lives in HBM.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <variant>
#include <vector>

#include "../../include/everett_cuda.h"

namespace everett {

// ---- errors (src/error.rs) -------------------------------------------------------

enum class ErrorKind {
  QubitOutOfRange = EV_ERR_QUBIT_OUT_OF_RANGE,
  ClassicalBitOutOfRange = EV_ERR_CLASSICAL_BIT_OUT_OF_RANGE,
  DuplicateQubit = EV_ERR_DUPLICATE_QUBIT,
  DimensionMismatch = EV_ERR_DIMENSION_MISMATCH,
  NonClifford = EV_ERR_NON_CLIFFORD,
  Qasm = EV_ERR_QASM,
  InvalidArgument = EV_ERR_INVALID_ARGUMENT,
  DeviceOutOfMemory = EV_ERR_OOM,
  Cuda = EV_ERR_CUDA,
  Timeout = EV_ERR_TIMEOUT,
  Other = -1,
};

class Error : public std::runtime_error {
 public:
  Error(ErrorKind k, const std::string& msg) : std::runtime_error(msg), kind_(k) {}
  ErrorKind kind() const { return kind_; }

 private:
  ErrorKind kind_;
};

// Throws the engine's last error as an everett::Error when rc != EV_OK.
inline void check(int rc) {
  if (rc == EV_OK) return;
  const char* m = ev_last_error();
  ErrorKind k = ErrorKind::Other;
  switch (rc) {
    case EV_ERR_QUBIT_OUT_OF_RANGE:
    case EV_ERR_CLASSICAL_BIT_OUT_OF_RANGE:
    case EV_ERR_DUPLICATE_QUBIT:
    case EV_ERR_DIMENSION_MISMATCH:
    case EV_ERR_NON_CLIFFORD:
    case EV_ERR_QASM:
    case EV_ERR_INVALID_ARGUMENT:
    case EV_ERR_OOM:
    case EV_ERR_CUDA:
    case EV_ERR_TIMEOUT:
      k = static_cast<ErrorKind>(rc);
      break;
    default:
      break;
  }
  throw Error(k, (m && *m) ? m : ("error code " + std::to_string(rc)));
}

// ---- Complex64 (src/complex.rs:22-133) -------------------------------------------

struct Complex64 {
  double re = 0.0, im = 0.0;
  static constexpr Complex64 make(double r, double i) { return Complex64{r, i}; }
  static Complex64 expi(double theta) { return {std::cos(theta), std::sin(theta)}; }
  Complex64 conj() const { return {re, -im}; }
  // re.mul_add(re, im * im)
  double norm_sqr() const { return std::fma(re, re, im * im); }
  double norm() const { return std::hypot(re, im); }
  // the reference's FMA-form product
  friend Complex64 operator*(Complex64 a, Complex64 b) {
    return {std::fma(a.re, b.re, -(a.im * b.im)), std::fma(a.re, b.im, a.im * b.re)};
  }
  friend Complex64 operator*(Complex64 a, double s) { return {a.re * s, a.im * s}; }
  friend Complex64 operator+(Complex64 a, Complex64 b) { return {a.re + b.re, a.im + b.im}; }
  friend Complex64 operator-(Complex64 a, Complex64 b) { return {a.re - b.re, a.im - b.im}; }
  friend Complex64 operator-(Complex64 a) { return {-a.re, -a.im}; }
  friend bool operator==(Complex64 a, Complex64 b) { return a.re == b.re && a.im == b.im; }
};
inline constexpr Complex64 ZERO{0.0, 0.0};
inline constexpr Complex64 ONE{1.0, 0.0};
inline constexpr Complex64 I{0.0, 1.0};

// ---- gates (src/gate.rs:44-247) --------------------------------------------------

struct Gate1 {
  std::array<Complex64, 4> m{};  // row-major 2x2
  static Gate1 make(Complex64 a, Complex64 b, Complex64 c, Complex64 d) { return Gate1{{a, b, c, d}}; }
  static Gate1 id() { return make(ONE, ZERO, ZERO, ONE); }
  static Gate1 x() { return make(ZERO, ONE, ONE, ZERO); }
  static Gate1 y() { return make(ZERO, {0.0, -1.0}, {0.0, 1.0}, ZERO); }
  static Gate1 z() { return make(ONE, ZERO, ZERO, {-1.0, 0.0}); }
  static Gate1 h() {
    const double s = 0.7071067811865476;  // FRAC_1_SQRT_2
    return make({s, 0.0}, {s, 0.0}, {s, 0.0}, {-s, 0.0});
  }
  static Gate1 s() { return make(ONE, ZERO, ZERO, I); }
  static Gate1 t() { return make(ONE, ZERO, ZERO, Complex64::expi(0.7853981633974483)); }
  static Gate1 rx(double theta) {
    const double sn = std::sin(theta / 2.0), cs = std::cos(theta / 2.0);
    return make({cs, 0.0}, {0.0, -sn}, {0.0, -sn}, {cs, 0.0});
  }
  static Gate1 ry(double theta) {
    const double sn = std::sin(theta / 2.0), cs = std::cos(theta / 2.0);
    return make({cs, 0.0}, {-sn, 0.0}, {sn, 0.0}, {cs, 0.0});
  }
  static Gate1 rz(double theta) {
    return make(Complex64::expi(-theta / 2.0), ZERO, ZERO, Complex64::expi(theta / 2.0));
  }
  static Gate1 phase(double lambda) { return make(ONE, ZERO, ZERO, Complex64::expi(lambda)); }
  Gate1 adjoint() const { return make(m[0].conj(), m[2].conj(), m[1].conj(), m[3].conj()); }
  friend bool operator==(const Gate1& a, const Gate1& b) { return a.m == b.m; }
};

struct Gate2 {
  std::array<Complex64, 16> m{};  // basis |q_a q_b>, a the more significant operand
  static Gate2 cnot() {
    Gate2 g;
    g.m[0] = g.m[5] = g.m[11] = g.m[14] = ONE;
    return g;
  }
  static Gate2 cz() {
    Gate2 g;
    g.m[0] = g.m[5] = g.m[10] = ONE;
    g.m[15] = {-1.0, 0.0};
    return g;
  }
  static Gate2 swap() {
    Gate2 g;
    g.m[0] = g.m[6] = g.m[9] = g.m[15] = ONE;
    return g;
  }
  static Gate2 controlled(const Gate1& u) {
    Gate2 g;
    g.m[0] = g.m[5] = ONE;
    g.m[10] = u.m[0];
    g.m[11] = u.m[1];
    g.m[14] = u.m[2];
    g.m[15] = u.m[3];
    return g;
  }
  friend bool operator==(const Gate2& a, const Gate2& b) { return a.m == b.m; }
};

// ---- ops and circuits (src/op.rs, src/circuit.rs) ----------------------------------

struct Op;
struct Apply1 {
  Gate1 gate;
  size_t target;
};
struct Apply2 {
  Gate2 gate;
  size_t a, b;
};
struct Controlled {
  std::vector<size_t> controls;
  Gate1 gate;
  size_t target;
};
struct Measure {
  size_t qubit, into;
};
struct IfClassic {
  size_t bit;
  std::shared_ptr<Op> then;
};
struct Op {
  std::variant<Apply1, Apply2, Controlled, Measure, IfClassic> v;
};

// op records and control pool in the C ABI's layout (IfClassic as a prefix)
struct Encoded {
  std::vector<ev_op> ops;
  std::vector<uint64_t> pool;
};

class Circuit {
 public:
  explicit Circuit(size_t num_qubits = 0, size_t num_classical = 0)
      : n_(num_qubits), ncl_(num_classical) {}
  static Circuit new_(size_t n) { return Circuit(n); }
  static Circuit with_classical(size_t n, size_t c) { return Circuit(n, c); }

  size_t num_qubits() const { return n_; }
  size_t num_classical() const { return ncl_; }
  const std::vector<Op>& ops() const { return ops_; }
  size_t len() const { return ops_.size(); }
  bool is_empty() const { return ops_.empty(); }

  Circuit& push_op(Op op) {
    ops_.push_back(std::move(op));
    return *this;
  }
  Circuit& gate1(const Gate1& g, size_t t) { return push_op(Op{Apply1{g, t}}); }
  Circuit& gate2(const Gate2& g, size_t a, size_t b) { return push_op(Op{Apply2{g, a, b}}); }
  Circuit& controlled(std::vector<size_t> cs, const Gate1& g, size_t t) {
    return push_op(Op{Controlled{std::move(cs), g, t}});
  }
  Circuit& measure(size_t q, size_t into) { return push_op(Op{Measure{q, into}}); }
  Circuit& if_classic(size_t bit, Op then) {
    return push_op(Op{IfClassic{bit, std::make_shared<Op>(std::move(then))}});
  }
  Circuit& h(size_t q) { return gate1(Gate1::h(), q); }
  Circuit& x(size_t q) { return gate1(Gate1::x(), q); }
  Circuit& y(size_t q) { return gate1(Gate1::y(), q); }
  Circuit& z(size_t q) { return gate1(Gate1::z(), q); }
  Circuit& s(size_t q) { return gate1(Gate1::s(), q); }
  Circuit& t(size_t q) { return gate1(Gate1::t(), q); }
  Circuit& rx(size_t q, double th) { return gate1(Gate1::rx(th), q); }
  Circuit& ry(size_t q, double th) { return gate1(Gate1::ry(th), q); }
  Circuit& rz(size_t q, double th) { return gate1(Gate1::rz(th), q); }
  Circuit& phase(size_t q, double l) { return gate1(Gate1::phase(l), q); }
  Circuit& cnot(size_t c, size_t t) { return gate2(Gate2::cnot(), c, t); }
  Circuit& cz(size_t a, size_t b) { return gate2(Gate2::cz(), a, b); }
  Circuit& swap(size_t a, size_t b) { return gate2(Gate2::swap(), a, b); }
  Circuit& x_if(size_t bit, size_t q) { return if_classic(bit, Op{Apply1{Gate1::x(), q}}); }
  Circuit& z_if(size_t bit, size_t q) { return if_classic(bit, Op{Apply1{Gate1::z(), q}}); }
  Circuit& compose(const Circuit& other) {
    for (const Op& op : other.ops_) ops_.push_back(op);
    return *this;
  }

  Encoded encode() const {
    Encoded e;
    for (const Op& op : ops_) emit(op, &e);
    return e;
  }
  // a view for the C ABI; `e` must outlive its use
  ev_circuit view(const Encoded& e) const {
    ev_circuit c;
    c.num_qubits = n_;
    c.num_classical = ncl_;
    c.ops = e.ops.empty() ? nullptr : e.ops.data();
    c.nops = e.ops.size();
    c.ctrl_pool = e.pool.empty() ? nullptr : e.pool.data();
    c.pool_len = e.pool.size();
    return c;
  }

  // Circuit::validate (circuit.rs:245-306): the first error in op order
  void validate() const {
    const Encoded e = encode();
    const ev_circuit c = view(e);
    check(ev_validate(&c));
  }

  // OpenQASM 3 (circuit.rs:308-326)
  std::string to_qasm() const {
    const Encoded e = encode();
    const ev_circuit c = view(e);
    uint64_t len = 0;
    check(ev_qasm_emit(&c, nullptr, 0, &len));
    std::string s(len + 1, '\0');
    check(ev_qasm_emit(&c, &s[0], len + 1, &len));
    s.resize(len);
    return s;
  }
  static Circuit from_qasm(const std::string& src) {
    ev_program* p = nullptr;
    check(ev_qasm_parse(src.data(), src.size(), &p, nullptr, nullptr));
    std::unique_ptr<ev_program, int (*)(ev_program*)> own(p, ev_program_free);
    ev_circuit v;
    check(ev_program_circuit(p, &v));
    Circuit c(v.num_qubits, v.num_classical);
    uint64_t pos = 0;
    while (pos < v.nops) c.ops_.push_back(decode(v, &pos));
    return c;
  }

 private:
  static void put_m1(ev_op* r, const Gate1& g) {
    for (int e = 0; e < 4; ++e) {
      r->m[2 * e] = g.m[e].re;
      r->m[2 * e + 1] = g.m[e].im;
    }
  }
  static void emit(const Op& op, Encoded* e) {
    ev_op r;
    std::memset(&r, 0, sizeof(r));
    if (auto* a = std::get_if<Apply1>(&op.v)) {
      r.kind = EV_OP_APPLY1;
      r.q0 = a->target;
      put_m1(&r, a->gate);
    } else if (auto* b = std::get_if<Apply2>(&op.v)) {
      r.kind = EV_OP_APPLY2;
      r.q0 = b->a;
      r.q1 = b->b;
      for (int k = 0; k < 16; ++k) {
        r.m[2 * k] = b->gate.m[k].re;
        r.m[2 * k + 1] = b->gate.m[k].im;
      }
    } else if (auto* c = std::get_if<Controlled>(&op.v)) {
      r.kind = EV_OP_CONTROLLED;
      r.q0 = c->target;
      r.nctrl = uint32_t(c->controls.size());
      r.ctrl_off = e->pool.size();
      for (size_t q : c->controls) e->pool.push_back(q);
      put_m1(&r, c->gate);
    } else if (auto* m = std::get_if<Measure>(&op.v)) {
      r.kind = EV_OP_MEASURE;
      r.q0 = m->qubit;
      r.q1 = m->into;
    } else {
      const auto& f = std::get<IfClassic>(op.v);
      r.kind = EV_OP_IF;
      r.q0 = f.bit;
      e->ops.push_back(r);
      emit(*f.then, e);
      return;
    }
    e->ops.push_back(r);
  }
  static Gate1 m1(const ev_op& r) {
    Gate1 g;
    for (int k = 0; k < 4; ++k) g.m[k] = {r.m[2 * k], r.m[2 * k + 1]};
    return g;
  }
  static Op decode(const ev_circuit& v, uint64_t* pos) {
    const ev_op& r = v.ops[(*pos)++];
    switch (r.kind) {
      case EV_OP_APPLY1: return Op{Apply1{m1(r), size_t(r.q0)}};
      case EV_OP_APPLY2: {
        Gate2 g;
        for (int k = 0; k < 16; ++k) g.m[k] = {r.m[2 * k], r.m[2 * k + 1]};
        return Op{Apply2{g, size_t(r.q0), size_t(r.q1)}};
      }
      case EV_OP_CONTROLLED: {
        std::vector<size_t> cs(v.ctrl_pool + r.ctrl_off, v.ctrl_pool + r.ctrl_off + r.nctrl);
        return Op{Controlled{cs, m1(r), size_t(r.q0)}};
      }
      case EV_OP_MEASURE: return Op{Measure{size_t(r.q0), size_t(r.q1)}};
      default: return Op{IfClassic{size_t(r.q0), std::make_shared<Op>(decode(v, pos))}};
    }
  }

  size_t n_, ncl_;
  std::vector<Op> ops_;
};

// ---- Rng (src/rng.rs:10-58) -------------------------------------------------------

class Rng {
 public:
  static Rng seed_from_u64(uint64_t seed) { return Rng(seed); }
  uint64_t next_u64() {
    const uint64_t result = rotl(s_[0] + s_[3], 23) + s_[0];
    const uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return result;
  }
  double next_f64() { return double(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

 private:
  explicit Rng(uint64_t seed) {
    for (int w = 0; w < 4; ++w) {  // SplitMix64
      seed += 0x9E3779B97F4A7C15ULL;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      s_[w] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
  uint64_t s_[4];
};

// ---- State (src/state.rs:24-185), resident in HBM -----------------------------------

class State {
 public:
  static State zero(size_t n) {
    ev_state* s = nullptr;
    check(ev_state_create(n, EV_C128, &s));
    return State(s);
  }
  static State from_amplitudes(const std::vector<Complex64>& amps) {
    const uint64_t len = amps.size();
    if (len == 0 || (len & (len - 1))) {
      uint64_t next = 1;
      while (next < len) next <<= 1;
      throw Error(ErrorKind::DimensionMismatch,
                  "amplitude buffer has length " + std::to_string(len) + ", expected " +
                      std::to_string(next));
    }
    size_t n = 0;
    while ((uint64_t(1) << n) < len) ++n;
    State s = zero(n);
    check(ev_state_upload(s.h_.get(), reinterpret_cast<const double*>(amps.data()), len));
    return s;
  }
  size_t num_qubits() const {
    uint64_t n = 0;
    check(ev_state_num_qubits(h_.get(), &n));
    return n;
  }
  size_t dim() const { return size_t(1) << num_qubits(); }
  std::vector<Complex64> amplitudes() const {
    std::vector<Complex64> out(dim());
    check(ev_state_download(h_.get(), reinterpret_cast<double*>(out.data()), out.size()));
    return out;
  }
  double probability(size_t basis) const {
    double p = 0;
    check(ev_probability(h_.get(), basis, &p));
    return p;
  }
  double norm_sqr() const {
    double v = 0;
    check(ev_norm_sqr(h_.get(), &v));
    return v;
  }
  void normalize() { check(ev_normalize(h_.get())); }
  Complex64 overlap(const State& other) const {
    double r[2];
    check(ev_overlap(h_.get(), other.h_.get(), r));
    return {r[0], r[1]};
  }
  double fidelity(const State& other) const {
    double f = 0;
    check(ev_fidelity(h_.get(), other.h_.get(), &f));
    return f;
  }
  std::array<double, 3> bloch_vector(size_t qubit) const {
    std::array<double, 3> b{};
    check(ev_bloch_vector(h_.get(), qubit, b.data()));
    return b;
  }
  // probabilities of the low m qubits summed over the others, in basis order
  // (the marginal of phase_estimation.rs:97-110)
  std::vector<double> marginal_low(size_t m) const {
    std::vector<double> out(size_t(1) << m);
    check(ev_marginal_low(h_.get(), m, out.data()));
    return out;
  }
  // full-register shots (bit q of a shot = qubit q); no reference counterpart
  std::vector<uint64_t> sample(uint64_t shots, uint64_t seed) {
    std::vector<uint64_t> out(shots);
    check(ev_sample(h_.get(), seed, shots, out.data()));
    return out;
  }
  ev_state* handle() const { return h_.get(); }
  explicit State(ev_state* s) : h_(s, ev_state_destroy) {}

 private:
  std::shared_ptr<ev_state> h_;
};

// ---- Execution and the backend (src/backend/statevector.rs:25-106) -------------------

class Execution {
 public:
  Execution(State s, std::vector<bool> classical) : state_(std::move(s)), classical_(std::move(classical)) {}
  const State& state() const { return state_; }
  const std::vector<bool>& classical() const { return classical_; }
  State into_state() && { return std::move(state_); }

 private:
  State state_;
  std::vector<bool> classical_;
};

class StateVectorBackend {
 public:
  static Execution run(const Circuit& c) { return run_seeded(c, 0); }
  static Execution run_seeded(const Circuit& c, uint64_t seed) {
    const Encoded e = c.encode();
    const ev_circuit v = c.view(e);
    check(ev_validate(&v));  // validation runs before any compute
    ev_state* s = nullptr;
    std::vector<uint8_t> bits(c.num_classical() + 1, 0);
    check(ev_run_seeded(&v, seed, nullptr, &s, bits.data()));
    std::vector<bool> classical(c.num_classical());
    for (size_t i = 0; i < classical.size(); ++i) classical[i] = bits[i] != 0;
    return Execution(State(s), std::move(classical));
  }
};

// ---- circuit generators (src/algorithms) -------------------------------------------

namespace algorithms {

inline Circuit bell() {  // prep.rs:23-30
  Circuit c(2);
  c.h(0).cnot(0, 1);
  return c;
}

inline Circuit ghz(size_t n) {  // prep.rs:51-59
  if (n < 2) throw std::invalid_argument("GHZ state requires at least 2 qubits");
  Circuit c(n);
  c.h(0);
  for (size_t k = 0; k + 1 < n; ++k) c.cnot(k, k + 1);
  return c;
}

inline Circuit qft(size_t n) {  // qft.rs:54-79
  Circuit c(n);
  for (size_t jj = n; jj-- > 0;) {
    c.h(jj);
    for (size_t kk = jj; kk-- > 0;) {
      const size_t m = jj - kk + 1;
      c.controlled({kk}, Gate1::phase(6.283185307179586 / double(uint64_t(1) << m)), jj);
    }
  }
  for (size_t i = 0; i < n / 2; ++i) c.swap(i, n - 1 - i);
  return c;
}

inline Circuit iqft(size_t n) {  // qft.rs:81-118
  Circuit c(n);
  for (size_t i = 0; i < n / 2; ++i) c.swap(i, n - 1 - i);
  for (size_t jj = 0; jj < n; ++jj) {
    for (size_t kk = 0; kk < jj; ++kk) {
      const size_t m = jj - kk + 1;
      c.controlled({kk}, Gate1::phase(-6.283185307179586 / double(uint64_t(1) << m)), jj);
    }
    c.h(jj);
  }
  return c;
}

inline Circuit trotter_tfim(size_t n, double jzz, double hx, double t, size_t steps) {
  // hamiltonian.rs:91-118: per step an Rx layer, then ZZ terms as CNOT-Rz-CNOT
  Circuit c(n);
  const double dt = t / double(steps);
  for (size_t s = 0; s < steps; ++s) {
    const double rx_angle = -2.0 * hx * dt;
    for (size_t i = 0; i < n; ++i) c.rx(i, rx_angle);
    const double zz_angle = -2.0 * jzz * dt;
    for (size_t i = 0; i + 1 < n; ++i) c.cnot(i, i + 1).rz(i + 1, zz_angle).cnot(i, i + 1);
  }
  return c;
}

inline Circuit teleport_circuit() {  // teleport.rs:45-77
  Circuit c = Circuit::with_classical(3, 2);
  c.h(1).cnot(1, 2);
  c.cnot(0, 1).h(0);
  c.measure(0, 0).measure(1, 1);
  c.x_if(1, 2).z_if(0, 2);
  return c;
}

inline Circuit teleport_state(Complex64 alpha, Complex64 beta) {  // teleport.rs:79-85
  const Gate1 prep = Gate1::make(alpha, -beta.conj(), beta, alpha.conj());
  Circuit c = Circuit::with_classical(3, 2);
  c.gate1(prep, 0);
  c.compose(teleport_circuit());
  return c;
}

inline Circuit superdense_circuit(bool bit0, bool bit1) {  // superdense.rs:35-50
  Circuit c = Circuit::with_classical(2, 2);
  c.h(0).cnot(0, 1);
  if (bit1) c.x(0);
  if (bit0) c.z(0);
  c.cnot(0, 1).h(0);
  c.measure(0, 0).measure(1, 1);
  return c;
}

inline Circuit phase_estimation(size_t m, double phi) {  // phase_estimation.rs:55-87
  Circuit c(m + 1);
  c.x(m);
  for (size_t j = 0; j < m; ++j) c.h(j);
  for (size_t j = 0; j < m; ++j)
    c.controlled({j}, Gate1::phase(6.283185307179586 * phi * double(uint32_t(1) << j)), m);
  c.compose(iqft(m));
  return c;
}

// phase_estimation.rs:97-121; among equal maxima the last index wins, as
// Rust's Iterator::max_by returns it
inline double most_probable_phase(const State& state, size_t m) {
  const std::vector<double> marg = state.marginal_low(m);
  size_t best = 0;
  for (size_t i = 1; i < marg.size(); ++i)
    if (!(marg[best] > marg[i])) best = i;
  return double(best) / double(marg.size());
}

}  // namespace algorithms
}  // namespace everett
