"""Pins the CPU oracle against the reference's own known-answer tests.

Each test re-expresses an assertion of the reference crate (file:line given)
against oracle/ev_oracle.cpp, so that the oracle the GPU parity tests trust
is itself checked against what the reference asserts.  CPU only.
"""
import math

import numpy as np
import pytest

import oracle as O
from everett_gb300 import Circuit, Gate1, Gate2, Rng, algorithms, workloads

GATES_1Q = [Gate1.h(), Gate1.x(), Gate1.y(), Gate1.z(), Gate1.s(), Gate1.t(), Gate1.rx(0.7),
            Gate1.ry(-1.3), Gate1.rz(2.1), Gate1.phase(0.9)]


def naive_apply_1q(amps, k, gate):
    """properties.rs:397-412: bit-test loop without index insertion."""
    m = gate.m
    out = amps.copy()
    for i in range(len(amps)):
        if (i >> k) & 1 == 0:
            p = i | (1 << k)
            a0, a1 = amps[i], amps[p]
            out[i] = m[0] * a0 + m[1] * a1
            out[p] = m[2] * a0 + m[3] * a1
    return out


# ---- kernel.rs:520-596 ------------------------------------------------------

def test_x_gate_flips_single_qubit():  # kernel.rs:541-547
    a = np.array([1, 0], dtype=np.complex128)
    O.apply_1q(a, 0, Gate1.x())
    assert np.array_equal(a, np.array([0, 1], dtype=np.complex128))


def test_hadamard_then_hadamard_is_identity():  # kernel.rs:549-556
    a = np.array([1, 0], dtype=np.complex128)
    O.apply_1q(a, 0, Gate1.h())
    O.apply_1q(a, 0, Gate1.h())
    assert abs(a[0] - 1) < 1e-12 and abs(a[1]) < 1e-12


def test_index_pair_and_quad_partition():  # kernel.rs:520-539, 558-568
    # a permutation gate applied through the pair/quad loops moves every
    # amplitude exactly once
    for n in range(1, 7):
        for k in range(n):
            a = np.arange(1 << n).astype(np.complex128)
            O.apply_1q(a, k, Gate1.x())
            assert sorted(a.real.astype(int)) == list(range(1 << n))
            assert all(int(a[j].real) == j ^ (1 << k) for j in range(1 << n))
    a = np.arange(8).astype(np.complex128)
    O.apply_2q(a, 0, 2, Gate2.swap())
    assert sorted(a.real.astype(int)) == list(range(8))


def test_cnot_flips_target_when_control_set():  # kernel.rs:570-579
    a = np.zeros(4, dtype=np.complex128)
    a[2] = 1
    O.apply_2q(a, 1, 0, Gate2.cnot())
    assert abs(a[3] - 1) < 1e-12


def test_controlled_x_matches_cnot():  # kernel.rs:581-596
    base = np.array([0.5 + 0.1j, 0.2 - 0.3j, -0.4 + 0.2j, 0.1 + 0.6j])
    a, b = base.copy(), base.copy()
    O.apply_2q(a, 1, 0, Gate2.cnot())
    O.apply_controlled_1q(b, [1], 0, Gate1.x())
    assert np.max(np.abs(a - b)) < 1e-12


def test_norm_preserved_small():  # kernel.rs:598-628
    for n in range(1, 5):
        for k in range(n):
            a = np.zeros(1 << n, dtype=np.complex128)
            a[0] = 1
            O.apply_1q(a, k, Gate1.h())
            assert abs(O.norm_sqr(a) - 1) < 1e-12
    for n in range(2, 5):
        a = np.zeros(1 << n, dtype=np.complex128)
        a[0] = 1
        O.apply_1q(a, 0, Gate1.h())
        O.apply_2q(a, 0, 1, Gate2.cnot())
        O.apply_controlled_1q(a, [0], 1, Gate1.z())
        assert abs(O.norm_sqr(a) - 1) < 1e-12


def test_specialized_2q_matches_dense():  # kernel.rs:637-690
    for n in range(2, 11):
        base = O.sample_state(n)
        for a in range(n):
            for b in range(n):
                if a == b:
                    continue
                for g in (Gate2.cnot(), Gate2.cz(), Gate2.swap()):
                    x, y = base.copy(), base.copy()
                    O.apply_2q(x, a, b, g)
                    O.apply_2q_dense(y, a, b, g)
                    assert np.max(np.abs(x - y)) < 1e-12, (n, a, b)


def test_controlled_matches_naive_all_placements():  # kernel.rs:692-730
    gates = [Gate1.x(), Gate1.y(), Gate1.z(), Gate1.h(), Gate1.s(), Gate1.rx(1.1),
             Gate1.ry(-0.7), Gate1.rz(2.3)]
    for n in range(2, 8):
        for t in range(n):
            for c in range(n):
                if c == t:
                    continue
                base = O.sample_state(n)
                for g in gates:
                    x = base.copy()
                    O.apply_controlled_1q(x, [c], t, g)
                    ref = naive_apply_1q(base, t, g)
                    mask = ((np.arange(1 << n) >> c) & 1).astype(bool)
                    want = np.where(mask, ref, base)
                    assert np.max(np.abs(x - want)) < 1e-12


def test_1q_matches_naive():  # kernel.rs:731-769, properties.rs:415-440
    for n in range(1, 9):
        for k in range(n):
            for g in GATES_1Q:
                x = O.sample_state(n)
                ref = naive_apply_1q(x, k, g)
                O.apply_1q(x, k, g)
                assert np.max(np.abs(x - ref)) < 1e-12


# ---- measure.rs:59-106, properties.rs:331-389 -------------------------------

def test_measuring_zero_state_yields_zero():
    c = Circuit.with_classical(1, 1)
    c.measure(0, 0)
    amps, bits, rc = O.run_seeded(c, 0)
    assert rc == 0 and bits == [False] and abs(abs(amps[0]) ** 2 - 1) < 1e-12


def test_measurement_collapses_and_renormalizes():
    c = Circuit.with_classical(1, 1)
    c.h(0).measure(0, 0)
    amps, bits, _ = O.run_seeded(c, 99)
    assert abs(O.norm_sqr(amps) - 1) < 1e-12
    assert abs(abs(amps[int(bits[0])]) ** 2 - 1) < 1e-12


def test_plus_state_statistics_are_balanced():
    u = O.rng_f64(2024, 4000)
    ones = 0
    for x in u:
        a = np.array([1, 0], dtype=np.complex128)
        O.apply_1q(a, 0, Gate1.h())
        ones += O.measure_qubit(a, 0, float(x))
    assert abs(ones / 4000 - 0.5) < 0.05


def test_deterministic_after_measurement():
    c = Circuit.with_classical(2, 2)
    c.h(0).measure(0, 0).measure(0, 1)
    _, bits, _ = O.run_seeded(c, 5)
    assert bits[0] == bits[1]


def test_measurement_collapses_to_basis_state():
    for seed in range(0, 10000, 157):
        c = Circuit.with_classical(2, 2)
        c.h(0).ry(1, 0.37 * seed).measure(0, 0).measure(1, 1)
        amps, _, _ = O.run_seeded(c, seed)
        p = np.abs(amps) ** 2
        assert np.sum(np.abs(p - 1) < 1e-10) == 1 and np.sum(p < 1e-10) == 3


# ---- state.rs:192-234 -------------------------------------------------------

def test_state_observables():
    for n in range(6):
        a = np.zeros(1 << n, dtype=np.complex128)
        a[0] = 1
        assert abs(O.norm_sqr(a) - 1) < 1e-12
    a = np.array([1, 0, 0, 0], dtype=np.complex128)
    b = a * complex(math.cos(0.7), math.sin(0.7))
    assert abs(abs(O.overlap(a, b)) ** 2 - 1) < 1e-12
    x, y, z = O.bloch_vector(np.array([1, 0], dtype=np.complex128), 0)
    assert abs(x) < 1e-12 and abs(y) < 1e-12 and abs(z - 1) < 1e-12
    d = np.array([2, 2j])
    O.normalize(d)
    assert abs(O.norm_sqr(d) - 1) < 1e-12


# ---- tests/algorithms_*.rs ---------------------------------------------------

def test_qft_of_zero_is_uniform():  # algorithms_qft.rs:11-23
    for n in range(1, 6):
        amps, _, _ = O.run_seeded(algorithms.qft(n))
        assert np.max(np.abs(np.abs(amps) ** 2 - 1 / (1 << n))) < 1e-12


def test_qft_then_iqft_is_identity():  # algorithms_qft.rs:25-48
    n = 4
    for basis in [0, 1, 3, 7, 8, 15]:
        c = Circuit(n)
        for bit in range(n):
            if basis >> bit & 1:
                c.x(bit)
        c.compose(algorithms.qft(n)).compose(algorithms.iqft(n))
        amps, _, _ = O.run_seeded(c)
        want = np.zeros(1 << n, dtype=np.complex128)
        want[basis] = 1
        assert abs(abs(O.overlap(amps, want)) ** 2 - 1) < 1e-12


def test_qft_of_basis_one_matches_closed_form():  # algorithms_qft.rs:50-74
    n, nn = 3, 8
    c = Circuit(n)
    c.x(0).compose(algorithms.qft(n))
    amps, _, _ = O.run_seeded(c)
    for k in range(nn):
        want = complex(math.cos(math.tau * k / nn), math.sin(math.tau * k / nn)) / math.sqrt(nn)
        assert abs(amps[k] - want) < 1e-12


def test_bell_and_ghz():  # algorithms_prep.rs:5-65
    amps, _, _ = O.run_seeded(algorithms.bell())
    p = np.abs(amps) ** 2
    assert abs(p[0] - 0.5) < 1e-12 and abs(p[3] - 0.5) < 1e-12 and p[1] < 1e-12 and p[2] < 1e-12
    for n in (3, 4, 5):
        amps, _, _ = O.run_seeded(algorithms.ghz(n))
        p = np.abs(amps) ** 2
        assert abs(p[0] - 0.5) < 1e-12 and abs(p[-1] - 0.5) < 1e-12
        assert np.all(p[1:-1] < 1e-12)
        for q in range(n):
            assert np.linalg.norm(O.bloch_vector(amps, q)) < 0.01


def test_tfim():  # algorithms_hamiltonian.rs:10-58
    amps, _, _ = O.run_seeded(algorithms.trotter_tfim(4, 1.0, 0.5, 1.0, 100))
    assert abs(O.norm_sqr(amps) - 1) < 1e-12
    hx, t = 0.8, 0.4
    a, _, _ = O.run_seeded(algorithms.trotter_tfim(1, 0.0, hx, t, 500))
    e = Circuit(1)
    e.rx(0, -2.0 * hx * t)
    b, _, _ = O.run_seeded(e)
    assert abs(O.overlap(a, b)) ** 2 > 0.9999
    coarse, _, _ = O.run_seeded(algorithms.trotter_tfim(2, 1.0, 0.5, 0.5, 10))
    fine, _, _ = O.run_seeded(algorithms.trotter_tfim(2, 1.0, 0.5, 0.5, 1000))
    assert abs(O.overlap(coarse, fine)) ** 2 > 0.99


@pytest.mark.parametrize("alpha,beta", [
    (1, 0), (0, 1), (1 / math.sqrt(2), 1 / math.sqrt(2)),
    (math.cos(0.35) * complex(math.cos(-0.55), math.sin(-0.55)),
     math.sin(0.35) * complex(math.cos(0.55), math.sin(0.55))),
])
def test_teleport_bloch(alpha, beta):  # algorithms_teleport.rs:40-91
    alpha, beta = complex(alpha), complex(beta)
    r01 = alpha * beta.conjugate()
    want = [2 * r01.real, 2 * r01.imag, abs(alpha) ** 2 - abs(beta) ** 2]
    c = algorithms.teleport_state(alpha, beta)
    for seed in range(8):
        amps, _, rc = O.run_seeded(c, seed)
        assert rc == 0
        got = O.bloch_vector(amps, 2)
        assert max(abs(g - w) for g, w in zip(got, want)) < 1e-10


@pytest.mark.parametrize("m,phi", [(1, 0.5), (2, 0.25), (2, 0.75), (3, 0.125), (3, 0.875),
                                   (4, 0.0)])
def test_phase_estimation_dyadic(m, phi):  # algorithms_phase_estimation.rs:12-36
    amps, _, rc = O.run_seeded(algorithms.phase_estimation(m, phi), 0)
    assert rc == 0
    assert abs(O.most_probable_phase(amps, m) - phi) < 1e-10


def test_phase_estimation_non_dyadic():  # algorithms_phase_estimation.rs:22-29
    amps, _, _ = O.run_seeded(algorithms.phase_estimation(4, 0.3), 0)
    assert abs(O.most_probable_phase(amps, 4) - 0.3) <= 1.0 / 16.0 + 1e-10


def test_most_probable_phase_ties_take_last():
    """Iterator::max_by keeps the later of equal elements: a uniform
    marginal gives the last index."""
    amps = np.full(8, 1 / math.sqrt(8), dtype=np.complex128)
    assert O.most_probable_phase(amps, 2) == 3 / 4


@pytest.mark.parametrize("bit0,bit1", [(False, False), (False, True), (True, False), (True, True)])
def test_superdense(bit0, bit1):  # algorithms_superdense.rs:5-36
    for seed in range(4):
        _, cl, rc = O.run_seeded(algorithms.superdense_circuit(bit0, bit1), seed)
        assert rc == 0
        assert list(cl) == [bit0, bit1]


# ---- rng.rs:62-95 plus cross-implementation agreement ------------------------

def test_rng_properties_and_agreement():
    a = O.rng_u64(42, 100)
    assert np.array_equal(a, O.rng_u64(42, 100))
    assert O.rng_u64(1, 1)[0] != O.rng_u64(2, 1)[0]
    x = O.rng_f64(7, 10000)
    assert np.all((x >= 0) & (x < 1))
    assert abs(O.rng_f64(123, 100000).mean() - 0.5) < 0.01
    r = Rng.seed_from_u64(42)
    assert [r.next_u64() for _ in range(100)] == [int(v) for v in a]
    r = Rng.seed_from_u64(0xFFFFFFFFFFFFFFFF)
    assert [r.next_f64() for _ in range(10)] == list(O.rng_f64(0xFFFFFFFFFFFFFFFF, 10))


# Published output vectors of the two algorithms behind rng.rs:18-58, which
# the reference's own tests (rng.rs:62-95) never pin:
#  - SplitMix64 (Steele, Lea, Flood, OOPSLA 2014; the reference code is
#    splitmix64.c by S. Vigna, prng.di.unimi.it) started from x = 0;
#  - xoshiro256++ (Blackman, Vigna, ACM TOMS 2021; xoshiro256plusplus.c)
#    started from the state {1, 2, 3, 4}, the vector its Rust port
#    (rand_xoshiro) checks against the C code.  The first value can be
#    checked by hand: rotl(1 + 4, 23) + 1 = 41943041.
SPLITMIX64_FROM_0 = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F,
                     0xF88BB8A8724C81EC]
XOSHIRO256PP_FROM_1234 = [41943041, 58720359, 3588806011781223, 3591011842654386,
                          9228616714210784205, 9973669472204895162, 14011001112246962877,
                          12406186145184390807, 15849039046786891736, 10450023813501588000]


def test_rng_pinned_to_published_vectors():
    """Rng::seed_from_u64 fills the state with four SplitMix64 outputs and
    steps it with xoshiro256++ (rng.rs:18-58): both halves equal the
    algorithms' published vectors, in the oracle and in the engine's Python
    restatement.  The engine's C++ and device restatements are held equal to
    the oracle's stream by test_rng_properties_and_agreement, the C++ host
    tests and the GPU measurement tests."""
    assert [int(v) for v in O.rng_seed_words(0)] == SPLITMIX64_FROM_0
    assert [int(v) for v in O.rng_raw([1, 2, 3, 4], 10)] == XOSHIRO256PP_FROM_1234
    assert Rng.seed_from_u64(0).s == SPLITMIX64_FROM_0
    r = Rng([1, 2, 3, 4])
    assert [r.next_u64() for _ in range(10)] == XOSHIRO256PP_FROM_1234
    # seeding then stepping: the oracle's stream from seed 0 is xoshiro256++
    # run from the SplitMix64 words
    r = Rng(list(SPLITMIX64_FROM_0))
    assert [r.next_u64() for _ in range(20)] == [int(v) for v in O.rng_u64(0, 20)]


def test_gate_constructors_match_oracle():  # gate.rs:106-136
    m = np.zeros(8)
    for t in (0.0, 0.3, -1.7, 2 * math.pi, 123.456):
        for name, g in (("rx", Gate1.rx), ("ry", Gate1.ry), ("rz", Gate1.rz),
                        ("phase", Gate1.phase)):
            getattr(O.lib(), "oracle_gate_" + name)(t, m.ctypes.data)
            assert np.array_equal(m, g(t).as_f64()), (name, t)
    O.lib().oracle_gate_h(m.ctypes.data)
    assert np.array_equal(m, Gate1.h().as_f64())


# ---- circuit.rs:245-306 validation --------------------------------------------

def test_validation_errors():
    c = Circuit(2)
    c.h(5)
    assert O.validate(c) == 1
    c = Circuit(2)
    c.cnot(1, 1)
    assert O.validate(c) == 3
    c = Circuit(1)
    c.measure(0, 0)
    assert O.validate(c) == 2
    c = Circuit.with_classical(1, 1)
    c.x_if(0, 3)
    assert O.validate(c) == 1
    c = Circuit(3)
    c.controlled([0, 2], Gate1.x(), 2)
    assert O.validate(c) == 3
    c = Circuit(2)
    c.h(0).cnot(0, 1)
    assert O.validate(c) == 0


# ---- shot sampling: literal collapse vs conditional-mass tree ---------------

def test_sample_tree_matches_literal():
    for n, seed in ((1, 3), (3, 4), (6, 5), (9, 6)):
        amps, _, _ = O.run_seeded(workloads.random_layers(n, 4, seed))
        lit = O.sample_literal(amps, 11, 500)
        tree = O.sample_tree(amps, 11, 500)
        assert np.array_equal(lit, tree), n
    # a state with zero-probability branches (GHZ) and a basis state
    amps, _, _ = O.run_seeded(algorithms.ghz(5))
    assert np.array_equal(O.sample_literal(amps, 2, 300), O.sample_tree(amps, 2, 300))
    assert set(O.sample_tree(amps, 2, 300).tolist()) <= {0, 31}


def test_oracle_pauli_expectation_pins():
    """PauliString::expectation (backend/stabilizer.rs:79-125): eigenstates of
    X, Y and Z give +1, the wrong basis 0, a negative sign flips the value;
    GHZ(3) is stabilised by XXX, ZZI and IZZ (tests/stabilizer.rs:13-25)."""
    s2 = 1 / np.sqrt(2)
    plus = np.array([s2, s2], dtype=complex)
    y_plus = np.array([s2, 1j * s2], dtype=complex)
    zero = np.array([1, 0], dtype=complex)
    assert abs(O.pauli_expectation(plus, 1, 0) - 1) < 1e-15
    assert abs(O.pauli_expectation(y_plus, 1, 1) - 1) < 1e-15
    assert abs(O.pauli_expectation(zero, 0, 1) - 1) < 1e-15
    assert abs(O.pauli_expectation(zero, 1, 0)) < 1e-15
    assert abs(O.pauli_expectation(zero, 0, 1, True) + 1) < 1e-15
    ghz = np.zeros(8, dtype=complex)
    ghz[0] = ghz[7] = s2
    for x, z in ((0b111, 0), (0, 0b011), (0, 0b110)):
        assert abs(O.pauli_expectation(ghz, x, z) - 1) < 1e-15
    assert abs(O.pauli_expectation(ghz, 0b111, 0b001)) < 1e-15  # <YXX> = 0 on GHZ(3)


def test_oracle_density_matrix_pins():
    """density.rs / density_matrix.rs / noise.rs tests, re-expressed: |0><0|
    has trace 1 and purity 1; X flips it; the Bell state's diagonal matches
    the statevector probabilities; noise keeps the trace at 1 and lowers the
    purity; Kraus sets are complete."""
    from everett_gb300 import Circuit
    from everett_gb300.density import Channel, NoiseModel
    c = Circuit(2)
    c.h(0).cnot(0, 1)
    rho, _ = O.dm_run(c)
    ob = O.dm_observables(rho, 0)
    assert abs(ob["trace"] - 1) < 1e-12 and abs(ob["purity"] - 1) < 1e-12
    amps, _, _ = O.run_seeded(c)
    assert np.max(np.abs(np.diag(rho).real - np.abs(amps) ** 2)) < 1e-12
    x = Circuit(1)
    x.x(0)
    rx, _ = O.dm_run(x)
    assert rx[1, 1] == 1 and rx[0, 0] == 0
    noisy, _ = O.dm_run(c, NoiseModel.uniform_depolarizing(0.1).ev_struct())
    ob = O.dm_observables(noisy, 1)
    assert abs(ob["trace"] - 1) < 1e-10 and ob["purity"] < 1
    for ch in (Channel.depolarizing(0.3), Channel.amplitude_damping(0.5),
               Channel.phase_damping(0.9), Channel.bit_flip(0.2), Channel.dephasing(0.4)):
        s = sum(np.conj(k.m.reshape(2, 2)).T @ k.m.reshape(2, 2) for k in ch.kraus_ops())
        assert np.max(np.abs(s - np.eye(2))) < 1e-12
