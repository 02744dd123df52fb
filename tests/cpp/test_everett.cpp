// Tests of the C++ host surface (everett_gb300/cpp/everett.hpp), written as
// the reference's own Rust tests are (src/circuit.rs:331-384,
// src/state.rs:188-240, src/rng.rs:61-90, tests/algorithms_prep.rs,
// tests/algorithms_qft.rs, tests/algorithms_teleport.rs,
// tests/algorithms_phase_estimation.rs, tests/algorithms_superdense.rs), plus checks that
// the C++ builder encodes what the engine's own circuit records hold.
//
// Usage: test_everett host|gpu   (host cases need no GPU)
#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "everett.hpp"

using namespace everett;

static int g_failed = 0;
static int g_run = 0;

#define REQUIRE(cond)                                                          \
  do {                                                                         \
    if (!(cond)) {                                                             \
      throw std::runtime_error(std::string(__FILE__ ":") + std::to_string(__LINE__) + \
                               ": " #cond);                                    \
    }                                                                          \
  } while (0)

template <class F>
static ErrorKind error_of(F f) {
  try {
    f();
  } catch (const Error& e) {
    return e.kind();
  }
  return ErrorKind::Other;
}

struct Case {
  const char* name;
  std::function<void()> body;
};

// ---- host cases ---------------------------------------------------------------

static void fluent_chaining_records_ops() {
  Circuit c(2);
  c.h(0).cnot(0, 1);
  REQUIRE(c.len() == 2);
  c.validate();
}

static void out_of_range_qubit_is_rejected() {
  Circuit c(2);
  c.h(5);
  bool caught = false;
  try {
    c.validate();
  } catch (const Error& e) {
    caught = true;
    REQUIRE(e.kind() == ErrorKind::QubitOutOfRange);
    REQUIRE(std::string(e.what()) == "qubit q5 out of range for 2-qubit register");
  }
  REQUIRE(caught);
}

static void duplicate_qubit_in_two_qubit_gate_is_rejected() {
  Circuit c(2);
  c.cnot(1, 1);
  REQUIRE(error_of([&] { c.validate(); }) == ErrorKind::DuplicateQubit);
}

static void measure_into_missing_classical_bit_is_rejected() {
  Circuit c(1);
  c.measure(0, 0);
  REQUIRE(error_of([&] { c.validate(); }) == ErrorKind::ClassicalBitOutOfRange);
}

static void compose_inlines_ops() {
  Circuit sub(2);
  sub.h(0).cnot(0, 1);
  Circuit c(2);
  c.compose(sub).x(0);
  REQUIRE(c.len() == 3);
}

static void classical_control_validates_recursively() {
  Circuit c = Circuit::with_classical(1, 1);
  c.x_if(0, 3);
  REQUIRE(error_of([&] { c.validate(); }) == ErrorKind::QubitOutOfRange);
}

static void controlled_target_among_controls_is_rejected() {
  Circuit c(3);
  c.controlled({0, 2}, Gate1::x(), 2);
  REQUIRE(error_of([&] { c.validate(); }) == ErrorKind::DuplicateQubit);
}

static void same_seed_same_stream() {
  Rng a = Rng::seed_from_u64(42), b = Rng::seed_from_u64(42);
  for (int i = 0; i < 100; ++i) REQUIRE(a.next_u64() == b.next_u64());
}

static void different_seeds_differ() {
  Rng a = Rng::seed_from_u64(1), b = Rng::seed_from_u64(2);
  REQUIRE(a.next_u64() != b.next_u64());
}

static void f64_in_unit_interval() {
  Rng r = Rng::seed_from_u64(7);
  for (int i = 0; i < 10000; ++i) {
    const double x = r.next_f64();
    REQUIRE(x >= 0.0 && x < 1.0);
  }
}

static void gate_identities() {
  // H^2 = I and S^2 = Z, with the reference's FMA-form product
  auto mul = [](const Gate1& a, const Gate1& b) {
    Gate1 r;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        r.m[2 * i + j] = a.m[2 * i] * b.m[j] + a.m[2 * i + 1] * b.m[2 + j];
    return r;
  };
  const Gate1 hh = mul(Gate1::h(), Gate1::h());
  const Gate1 id = Gate1::id();
  for (int k = 0; k < 4; ++k) REQUIRE((hh.m[k] - id.m[k]).norm() < 1e-15);
  REQUIRE(mul(Gate1::s(), Gate1::s()) == Gate1::z());
  REQUIRE(Gate1::s().adjoint() == Gate1::make(ONE, ZERO, ZERO, {0.0, -1.0}));
  REQUIRE(Gate2::controlled(Gate1::x()) == Gate2::cnot());
  REQUIRE(Gate2::controlled(Gate1::z()) == Gate2::cz());
}

static void encoding_prefixes_if_classic() {
  Circuit c = Circuit::with_classical(3, 2);
  c.controlled({0, 1}, Gate1::t(), 2).x_if(1, 2).measure(2, 0);
  const Encoded e = c.encode();
  REQUIRE(e.ops.size() == 4);
  REQUIRE(e.ops[0].kind == EV_OP_CONTROLLED && e.ops[0].nctrl == 2 && e.ops[0].ctrl_off == 0);
  REQUIRE(e.pool.size() == 2 && e.pool[0] == 0 && e.pool[1] == 1);
  REQUIRE(e.ops[1].kind == EV_OP_IF && e.ops[1].q0 == 1);
  REQUIRE(e.ops[2].kind == EV_OP_APPLY1 && e.ops[2].q0 == 2 && e.ops[2].m[2] == 1.0);
  REQUIRE(e.ops[3].kind == EV_OP_MEASURE && e.ops[3].q0 == 2 && e.ops[3].q1 == 0);
}

static void qasm_round_trip() {
  Circuit c = Circuit::with_classical(3, 2);
  c.ry(0, 0.7).rz(0, 1.1).controlled({0, 1}, Gate1::t(), 2);
  c.compose(algorithms::teleport_circuit());
  const std::string src = c.to_qasm();
  REQUIRE(src.rfind("OPENQASM 3.0;", 0) == 0);
  const Circuit back = Circuit::from_qasm(src);
  REQUIRE(back.num_qubits() == 3 && back.num_classical() == 2);
  const Encoded a = c.encode(), b = back.encode();
  REQUIRE(a.ops.size() == b.ops.size() && a.pool == b.pool);
  for (size_t i = 0; i < a.ops.size(); ++i) {
    REQUIRE(a.ops[i].kind == b.ops[i].kind && a.ops[i].q0 == b.ops[i].q0);
    for (int k = 0; k < 32; ++k) REQUIRE(std::fabs(a.ops[i].m[k] - b.ops[i].m[k]) < 1e-15);
  }
  // a generic unitary has no OpenQASM 3 name
  Circuit g(1);
  g.gate1(Gate1::make({0.6, 0.0}, {-0.48, 0.64}, {0.48, 0.64}, {0.6, 0.0}), 0);
  REQUIRE(error_of([&] { g.to_qasm(); }) == ErrorKind::Qasm);
}

static void qasm_error_is_positioned() {
  bool caught = false;
  try {
    Circuit::from_qasm("OPENQASM 3.0;\nqubit[2] q;\nfoo q[0];\n");
  } catch (const Error& e) {
    caught = true;
    REQUIRE(e.kind() == ErrorKind::Qasm);
    REQUIRE(std::string(e.what()).rfind("OpenQASM 3 error at ", 0) == 0);
    REQUIRE(std::string(e.what()).find("unknown single-qubit gate 'foo'") != std::string::npos);
  }
  REQUIRE(caught);
}

static void from_amplitudes_rejects_non_power_of_two_host() {
  // the length check runs before any device call
  bool caught = false;
  try {
    State::from_amplitudes(std::vector<Complex64>(3));
  } catch (const Error& e) {
    caught = true;
    REQUIRE(e.kind() == ErrorKind::DimensionMismatch);
    REQUIRE(std::string(e.what()) == "amplitude buffer has length 3, expected 4");
  }
  REQUIRE(caught);
}

static void invalid_circuit_fails_before_device() {
  Circuit c(2);
  c.cnot(0, 0);
  REQUIRE(error_of([&] { StateVectorBackend::run(c); }) == ErrorKind::DuplicateQubit);
}

// ---- GPU cases -----------------------------------------------------------------

static void zero_state_is_normalized() {
  State s = State::zero(3);
  REQUIRE(std::fabs(s.norm_sqr() - 1.0) < 1e-15);
  REQUIRE(s.amplitudes()[0] == ONE);
}

static void fidelity_ignores_global_phase() {
  const double r = 0.7071067811865476;
  State a = State::from_amplitudes({{r, 0.0}, {r, 0.0}});
  State b = State::from_amplitudes({{0.0, r}, {0.0, r}});
  REQUIRE(std::fabs(a.fidelity(b) - 1.0) < 1e-12);
}

static void bloch_vector_of_zero_state_points_up() {
  State s = State::zero(1);
  const auto b = s.bloch_vector(0);
  REQUIRE(std::fabs(b[0]) < 1e-12 && std::fabs(b[1]) < 1e-12 && std::fabs(b[2] - 1.0) < 1e-12);
}

static void normalize_fixes_drift() {
  State s = State::from_amplitudes({{2.0, 0.0}, {0.0, 0.0}});
  s.normalize();
  REQUIRE(std::fabs(s.norm_sqr() - 1.0) < 1e-12);
}

static void bell_probabilities() {
  State s = StateVectorBackend::run(algorithms::bell()).into_state();
  REQUIRE(std::fabs(s.probability(0b00) - 0.5) < 1e-12);
  REQUIRE(std::fabs(s.probability(0b11) - 0.5) < 1e-12);
  REQUIRE(s.probability(0b01) < 1e-12);
  REQUIRE(s.probability(0b10) < 1e-12);
  REQUIRE(std::fabs(s.norm_sqr() - 1.0) < 1e-12);
}

static void ghz_probabilities_3_to_5() {
  for (size_t n = 3; n <= 5; ++n) {
    State s = StateVectorBackend::run(algorithms::ghz(n)).into_state();
    const size_t all = (size_t(1) << n) - 1;
    REQUIRE(std::fabs(s.probability(0) - 0.5) < 1e-12);
    REQUIRE(std::fabs(s.probability(all) - 0.5) < 1e-12);
    for (size_t b = 1; b < all; ++b) REQUIRE(s.probability(b) < 1e-12);
  }
}

static void ghz_qubits_are_maximally_mixed() {
  State s = StateVectorBackend::run(algorithms::ghz(3)).into_state();
  for (size_t q = 0; q < 3; ++q) {
    const auto b = s.bloch_vector(q);
    REQUIRE(std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) < 0.01);
  }
}

static void qft_of_zero_is_uniform_for_n_1_to_5() {
  for (size_t n = 1; n <= 5; ++n) {
    State s = StateVectorBackend::run(algorithms::qft(n)).into_state();
    const double want = 1.0 / double(size_t(1) << n);
    for (size_t b = 0; b < (size_t(1) << n); ++b) REQUIRE(std::fabs(s.probability(b) - want) < 1e-12);
  }
}

static void qft_then_iqft_is_identity_on_basis_states() {
  const size_t n = 4;
  for (size_t input : {0, 1, 3, 7, 8, 15}) {
    std::vector<Complex64> amps(size_t(1) << n, ZERO);
    amps[input] = ONE;
    State want = State::from_amplitudes(amps);
    Circuit c(n);
    for (size_t bit = 0; bit < n; ++bit)
      if (input & (size_t(1) << bit)) c.x(bit);
    c.compose(algorithms::qft(n)).compose(algorithms::iqft(n));
    State got = StateVectorBackend::run(c).into_state();
    REQUIRE(got.fidelity(want) > 1.0 - 1e-12);
  }
}

static void qft_of_basis_one_matches_closed_form() {
  const size_t n = 3, nn = size_t(1) << n;
  Circuit c(n);
  c.x(0);
  c.compose(algorithms::qft(n));
  const auto amps = StateVectorBackend::run(c).into_state().amplitudes();
  const double scale = 1.0 / std::sqrt(double(nn));
  for (size_t k = 0; k < nn; ++k) {
    const Complex64 want = Complex64::expi(6.283185307179586 * double(k) / double(nn)) * scale;
    REQUIRE((amps[k] - want).norm() < 1e-12);
  }
}

static std::array<double, 3> expected_bloch(Complex64 a, Complex64 b) {
  const Complex64 r01 = a * b.conj();
  return {2.0 * r01.re, 2.0 * r01.im, a.norm_sqr() - b.norm_sqr()};
}

static void teleport_cases() {
  const double s = 1.0 / std::sqrt(2.0);
  const double sh = std::sin(0.35), ch = std::cos(0.35);
  const std::vector<std::pair<Complex64, Complex64>> states = {
      {ONE, ZERO},
      {ZERO, ONE},
      {{s, 0.0}, {s, 0.0}},
      {{ch * std::cos(-0.55), ch * std::sin(-0.55)}, {sh * std::cos(0.55), sh * std::sin(0.55)}},
  };
  for (const auto& ab : states) {
    const auto got = StateVectorBackend::run(algorithms::teleport_state(ab.first, ab.second))
                         .state()
                         .bloch_vector(2);
    const auto want = expected_bloch(ab.first, ab.second);
    for (int i = 0; i < 3; ++i) REQUIRE(std::fabs(got[i] - want[i]) < 1e-10);
  }
}

static void teleport_is_seed_independent() {
  const double s = 1.0 / std::sqrt(2.0);
  const Complex64 a{s, 0.0}, b{0.0, s};
  const Circuit c = algorithms::teleport_state(a, b);
  const auto want = expected_bloch(a, b);
  std::vector<int> seen(4, 0);
  for (uint64_t seed = 0; seed < 8; ++seed) {
    Execution ex = StateVectorBackend::run_seeded(c, seed);
    const auto got = ex.state().bloch_vector(2);
    for (int i = 0; i < 3; ++i) REQUIRE(std::fabs(got[i] - want[i]) < 1e-10);
    seen[int(ex.classical()[0]) + 2 * int(ex.classical()[1])] = 1;
  }
  // at least two measurement branches were exercised
  REQUIRE(seen[0] + seen[1] + seen[2] + seen[3] >= 2);
}

// tests/algorithms_phase_estimation.rs:12-36
static void phase_estimation_recovers_phases() {
  const std::vector<std::pair<size_t, double>> dyadic = {
      {1, 0.5}, {2, 0.25}, {2, 0.75}, {3, 0.125}, {3, 0.875}, {4, 0.0}};
  for (const auto& mp : dyadic) {
    Execution ex = StateVectorBackend::run(algorithms::phase_estimation(mp.first, mp.second));
    REQUIRE(std::fabs(algorithms::most_probable_phase(ex.state(), mp.first) - mp.second) < 1e-10);
  }
  Execution ex = StateVectorBackend::run(algorithms::phase_estimation(4, 0.3));
  REQUIRE(std::fabs(algorithms::most_probable_phase(ex.state(), 4) - 0.3) <= 1.0 / 16.0 + 1e-10);
}

// tests/algorithms_superdense.rs:5-36
static void superdense_decodes_both_bits() {
  for (int b = 0; b < 4; ++b) {
    const bool bit0 = b & 1, bit1 = b & 2;
    Execution ex = StateVectorBackend::run(algorithms::superdense_circuit(bit0, bit1));
    REQUIRE(ex.classical()[0] == bit0);
    REQUIRE(ex.classical()[1] == bit1);
  }
}

static void measurement_uses_the_seeded_uniforms() {
  // One measurement of |+>: the outcome is 1 exactly when the seed's first
  // uniform is below P(1) = |1/sqrt 2|^2 (measure.rs measure_qubit).
  Circuit c = Circuit::with_classical(1, 1);
  c.h(0).measure(0, 0);
  int ones = 0;
  for (uint64_t seed = 0; seed < 16; ++seed) {
    Rng r = Rng::seed_from_u64(seed);
    const double u = r.next_f64();
    const Execution ex = StateVectorBackend::run_seeded(c, seed);
    const double p1 = Complex64{0.7071067811865476, 0.0}.norm_sqr();
    REQUIRE(ex.classical()[0] == (u < p1));
    ones += ex.classical()[0];
  }
  REQUIRE(ones > 0 && ones < 16);
}

static void trotter_norm_is_kept() {
  State s = StateVectorBackend::run(algorithms::trotter_tfim(10, 1.0, 0.7, 1.0, 5)).into_state();
  REQUIRE(std::fabs(s.norm_sqr() - 1.0) < 1e-12);
}

static void gpu_run_errors_are_typed() {
  Circuit c(2);
  c.h(7);
  REQUIRE(error_of([&] { StateVectorBackend::run(c); }) == ErrorKind::QubitOutOfRange);
  State s = State::zero(2);
  REQUIRE(error_of([&] { s.bloch_vector(9); }) != ErrorKind::Other);
}

int main(int argc, char** argv) {
  const std::string which = argc > 1 ? argv[1] : "host";
  if (which == "rng" && argc == 4) {  // rng SEED COUNT: the u64 stream, then the f64 stream
    const uint64_t seed = std::stoull(argv[2]), count = std::stoull(argv[3]);
    Rng a = Rng::seed_from_u64(seed), b = Rng::seed_from_u64(seed);
    for (uint64_t i = 0; i < count; ++i) std::printf("%llu\n", (unsigned long long)a.next_u64());
    for (uint64_t i = 0; i < count; ++i) std::printf("%a\n", b.next_f64());
    return 0;
  }
  const std::vector<Case> host = {
      {"fluent_chaining_records_ops", fluent_chaining_records_ops},
      {"out_of_range_qubit_is_rejected", out_of_range_qubit_is_rejected},
      {"duplicate_qubit_in_two_qubit_gate_is_rejected", duplicate_qubit_in_two_qubit_gate_is_rejected},
      {"measure_into_missing_classical_bit_is_rejected", measure_into_missing_classical_bit_is_rejected},
      {"compose_inlines_ops", compose_inlines_ops},
      {"classical_control_validates_recursively", classical_control_validates_recursively},
      {"controlled_target_among_controls_is_rejected", controlled_target_among_controls_is_rejected},
      {"same_seed_same_stream", same_seed_same_stream},
      {"different_seeds_differ", different_seeds_differ},
      {"f64_in_unit_interval", f64_in_unit_interval},
      {"gate_identities", gate_identities},
      {"encoding_prefixes_if_classic", encoding_prefixes_if_classic},
      {"qasm_round_trip", qasm_round_trip},
      {"qasm_error_is_positioned", qasm_error_is_positioned},
      {"from_amplitudes_rejects_non_power_of_two", from_amplitudes_rejects_non_power_of_two_host},
      {"invalid_circuit_fails_before_device", invalid_circuit_fails_before_device},
  };
  const std::vector<Case> gpu = {
      {"zero_state_is_normalized", zero_state_is_normalized},
      {"fidelity_ignores_global_phase", fidelity_ignores_global_phase},
      {"bloch_vector_of_zero_state_points_up", bloch_vector_of_zero_state_points_up},
      {"normalize_fixes_drift", normalize_fixes_drift},
      {"bell_probabilities", bell_probabilities},
      {"ghz_probabilities_3_to_5", ghz_probabilities_3_to_5},
      {"ghz_qubits_are_maximally_mixed", ghz_qubits_are_maximally_mixed},
      {"qft_of_zero_is_uniform_for_n_1_to_5", qft_of_zero_is_uniform_for_n_1_to_5},
      {"qft_then_iqft_is_identity_on_basis_states", qft_then_iqft_is_identity_on_basis_states},
      {"qft_of_basis_one_matches_closed_form", qft_of_basis_one_matches_closed_form},
      {"teleport_cases", teleport_cases},
      {"teleport_is_seed_independent", teleport_is_seed_independent},
      {"phase_estimation_recovers_phases", phase_estimation_recovers_phases},
      {"superdense_decodes_both_bits", superdense_decodes_both_bits},
      {"measurement_uses_the_seeded_uniforms", measurement_uses_the_seeded_uniforms},
      {"trotter_norm_is_kept", trotter_norm_is_kept},
      {"gpu_run_errors_are_typed", gpu_run_errors_are_typed},
  };
  const std::vector<Case>& cases = which == "gpu" ? gpu : host;
  for (const Case& c : cases) {
    ++g_run;
    try {
      c.body();
      std::printf("ok   %s\n", c.name);
    } catch (const std::exception& e) {
      ++g_failed;
      std::printf("FAIL %s: %s\n", c.name, e.what());
    }
  }
  std::printf("%d run, %d failed\n", g_run, g_failed);
  return g_failed == 0 ? 0 : 1;
}
