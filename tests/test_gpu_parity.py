"""GPU parity: the engine's kernels, called through the C ABI, against the
CPU oracle on the same seeded inputs.

Bars (written per test):
  complex128 gate arithmetic   bit-identical to the oracle (== on every
                               component; only the sign of a zero may differ)
  reductions (p1, norm, ...)   1e-12 absolute (the GPU sums in a different
                               order)
  measurement outcomes         identical for the same uniforms
  shot sampling                identical to the oracle's conditional-mass tree
                               (same pairwise sums, same uniforms)
  complex64                    fidelity >= 1 - 1e-6 against the complex128 oracle
"""
import math

import numpy as np
import pytest

import oracle as O
from everett_gb300 import (Apply1, Circuit, CudaStateVectorBackend, DuplicateQubit, Gate1, Gate2,
                           IfClassic, Measure, QubitOutOfRange, State, algorithms, workloads)
from everett_gb300.error import DimensionMismatch

pytestmark = pytest.mark.gpu

GATES_1Q = [Gate1.h(), Gate1.x(), Gate1.y(), Gate1.z(), Gate1.s(), Gate1.t(), Gate1.rx(0.7),
            Gate1.ry(-1.3), Gate1.rz(2.1), Gate1.phase(0.9), Gate1.id(),
            Gate1(0.6 + 0.1j, -0.3 + 0.2j, 0.25 - 0.7j, 0.1 + 0.05j)]


def rand_gate2(rng):
    return Gate2(rng.normal(size=16) + 1j * rng.normal(size=16))


def gates_2q(rng):
    return [Gate2.cnot(), Gate2.cz(), Gate2.swap(), Gate2.rzz(0.77), Gate2.controlled(Gate1.ry(0.4)),
            rand_gate2(rng)]


def exact(a, b):
    return np.array_equal(a, b)


def test_apply_1q_bit_exact(gpu):  # kernel.rs:76-119
    for n in range(1, 11):
        base = O.sample_state(n)
        st = State.from_amplitudes(base)
        for k in range(n):
            for g in GATES_1Q:
                st.upload(base)
                st.apply_1q(k, g)
                want = base.copy()
                O.apply_1q(want, k, g)
                assert exact(st.amplitudes(), want), (n, k, g)


def test_apply_2q_bit_exact(gpu):  # kernel.rs:192-289
    rng = np.random.default_rng(1)
    gs = gates_2q(rng)
    for n in range(2, 9):
        base = O.sample_state(n)
        st = State.from_amplitudes(base)
        for a in range(n):
            for b in range(n):
                if a == b:
                    continue
                for g in gs:
                    st.upload(base)
                    st.apply_2q(a, b, g)
                    want = base.copy()
                    O.apply_2q(want, a, b, g)
                    assert exact(st.amplitudes(), want), (n, a, b, g)


def test_controlled_bit_exact(gpu):  # kernel.rs:299-358
    rng = np.random.default_rng(2)
    for n in range(2, 9):
        base = O.sample_state(n)
        st = State.from_amplitudes(base)
        for t in range(n):
            for _ in range(6):
                nc = int(rng.integers(1, min(3, n - 1) + 1))
                ctrls = [int(c) for c in rng.choice([q for q in range(n) if q != t], nc,
                                                    replace=False)]
                for g in GATES_1Q:
                    st.upload(base)
                    st.apply_controlled_1q(ctrls, t, g)
                    want = base.copy()
                    O.apply_controlled_1q(want, ctrls, t, g)
                    assert exact(st.amplitudes(), want), (n, t, ctrls, g)


def test_large_state_gates_bit_exact(gpu):
    n = 22
    rng = np.random.default_rng(3)
    base = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) / math.sqrt(2 << n)
    g = rand_gate2(rng)
    st = State.from_amplitudes(base)
    want = base.copy()
    for k in (0, 1, 4, 5, 11, 21):
        st.apply_1q(k, Gate1.rx(0.3 + k))
        O.apply_1q(want, k, Gate1.rx(0.3 + k))
    st.apply_2q(21, 0, Gate2.cnot())
    O.apply_2q(want, 21, 0, Gate2.cnot())
    st.apply_2q(3, 17, g)
    O.apply_2q(want, 3, 17, g)
    st.apply_controlled_1q([2, 20], 9, Gate1.phase(0.123))
    O.apply_controlled_1q(want, [2, 20], 9, Gate1.phase(0.123))
    assert exact(st.amplitudes(), want)


def test_measure_matches_oracle(gpu):  # measure.rs:15-51
    n = 12
    amps, _, _ = O.run_seeded(workloads.random_layers(n, 6, seed=7))
    for k in (0, 3, 11):
        for u in (0.01, 0.37, 0.5, 0.93):
            st = State.from_amplitudes(amps)
            got = st.measure_qubit(k, u)
            want_amps = amps.copy()
            want = O.measure_qubit(want_amps, k, u)
            assert got == want
            assert np.max(np.abs(st.amplitudes() - want_amps)) < 1e-12


def test_observables_match_oracle(gpu):  # state.rs:94-185
    n = 14
    amps, _, _ = O.run_seeded(workloads.random_layers(n, 5, seed=8))
    other, _, _ = O.run_seeded(workloads.random_layers(n, 5, seed=9))
    st, so = State.from_amplitudes(amps), State.from_amplitudes(other)
    assert abs(st.norm_sqr() - O.norm_sqr(amps)) < 1e-12
    assert abs(st.overlap(so) - O.overlap(amps, other)) < 1e-12
    assert abs(st.fidelity(so) - abs(O.overlap(amps, other)) ** 2) < 1e-12
    for q in (0, 7, 13):
        assert np.max(np.abs(np.array(st.bloch_vector(q)) - O.bloch_vector(amps, q))) < 1e-12
    for b in (0, 5, (1 << n) - 1):
        assert abs(st.probability(b) - abs(amps[b]) ** 2) < 1e-15
    d = State.from_amplitudes(np.array([2, 2j]))
    d.normalize()
    assert abs(d.norm_sqr() - 1) < 1e-12


def test_complex64_reductions_match_oracle(gpu):
    """complex64 norms, p1, overlaps and measurement (double-float sums on
    the FP32 pipe, FP64 results) against the oracle evaluated in f64 on the
    same complex64 amplitudes: 1e-12, at sizes that exercise the pair and
    odd-tail paths (n = 1, 2, 3) and multi-block grids."""
    for n in (1, 2, 3, 9, 17, 21):
        amps, _, _ = O.run_seeded(workloads.random_layers(n, 3, seed=n))
        other, _, _ = O.run_seeded(workloads.random_layers(n, 3, seed=n + 50))
        a32 = amps.astype(np.complex64).astype(np.complex128)
        o32 = other.astype(np.complex64).astype(np.complex128)
        st = State.from_amplitudes(amps, dtype="complex64")
        so = State.from_amplitudes(other, dtype="complex64")
        assert abs(st.norm_sqr() - O.norm_sqr(a32)) < 1e-12, n
        assert abs(st.overlap(so) - O.overlap(a32, o32)) < 1e-12, n
        for k in sorted({0, min(1, n - 1), n - 1}):
            st.upload(a32)
            u = 0.37
            got = st.measure_qubit(k, u)
            p1 = float(np.sum(np.abs(a32[(np.arange(1 << n) >> k) & 1 == 1]) ** 2))
            assert got == (u < p1), (n, k)
    # a state concentrated on one amplitude: relative accuracy must hold
    a = np.zeros(1 << 12, dtype=np.complex128)
    a[77] = np.float32(0.999)
    a[5] = np.float32(1e-3) * 1j
    st = State.from_amplitudes(a, dtype="complex64")
    want = O.norm_sqr(a.astype(np.complex64).astype(np.complex128))
    assert abs(st.norm_sqr() - want) < 1e-14


def test_max_abs_diff_matches_host(gpu):
    """ev_max_abs_diff (either amplitude type) equals the host maximum to
    1e-15 relative (the device and host hypot may differ in the last bit)."""
    def close(x, y):
        return abs(x - y) <= 1e-15 * max(abs(y), 1e-300)

    for n in (1, 5, 13):
        amps, _, _ = O.run_seeded(workloads.random_layers(n, 3, seed=n))
        other, _, _ = O.run_seeded(workloads.random_layers(n, 3, seed=n + 1))
        a, b = State.from_amplitudes(amps), State.from_amplitudes(other)
        assert close(a.max_abs_diff(b), np.max(np.abs(amps - other)))
        c = State.from_amplitudes(amps, dtype="complex64")
        c32 = c.amplitudes()
        assert close(a.max_abs_diff(c), np.max(np.abs(amps - c32)))
        assert close(c.max_abs_diff(a), np.max(np.abs(c32 - amps)))
        assert a.max_abs_diff(a) == 0.0


def test_complex64_shots_match_tree(gpu):
    """complex64 sampling: the tree's leaves are double-float sums rounded to
    f64 once, so shots equal the oracle's tree on the same amplitudes except
    where a uniform falls within ~1e-14 of a conditional probability (none
    at these sizes and seeds)."""
    for n, seed in ((1, 3), (5, 4), (16, 5)):
        amps, _, _ = O.run_seeded(workloads.random_layers(n, 4, seed=n))
        st = State.from_amplitudes(amps, dtype="complex64")
        a32 = np.ascontiguousarray(st.amplitudes())
        assert np.array_equal(st.sample(2000, seed=seed), O.sample_tree(a32, seed, 2000)), n


@pytest.mark.parametrize("mode", ["exact", "tiled"])
def test_run_random_layers_bit_exact(gpu, mode):
    for n, depth, seed in ((5, 6, 1), (12, 10, 2), (16, 8, 3)):
        c = workloads.random_layers(n, depth, seed)
        want, _, _ = O.run_seeded(c, 0, parallel=True)
        ex = CudaStateVectorBackend.run(c, mode=mode)
        assert exact(ex.state().amplitudes(), want), (n, mode)


@pytest.mark.parametrize("tile_bits", [4, 6, 9, 12])
def test_tiled_mixed_ops_bit_exact(gpu, tile_bits):
    """Every op kind through the shared-memory tile path, including controls
    inside and outside the tile."""
    rng = np.random.default_rng(tile_bits)
    n = 14
    c = Circuit(n)
    for _ in range(120):
        kind = int(rng.integers(0, 4))
        qs = [int(v) for v in rng.choice(n, 4, replace=False)]
        if kind == 0:
            c.gate1(GATES_1Q[int(rng.integers(0, len(GATES_1Q)))], qs[0])
        elif kind == 1:
            c.gate2(gates_2q(rng)[int(rng.integers(0, 6))], qs[0], qs[1])
        elif kind == 2:
            c.controlled(qs[1:1 + int(rng.integers(1, 4))], GATES_1Q[int(rng.integers(0, 12))], qs[0])
        else:
            c.controlled([qs[1]], Gate1.phase(float(rng.uniform(0, 6))), qs[0])
    want, _, _ = O.run_seeded(c, 0)
    got = CudaStateVectorBackend.run(c, mode="tiled", tile_bits=tile_bits).state().amplitudes()
    assert exact(got, want)


def test_cfg0_random20_and_shots(gpu):
    """The plain-method small config: 20 qubits, depth 20, complex128, then
    10000 full-register shots from seed-derived uniforms."""
    c = workloads.random_layers(20, 20, seed=1)
    want, _, _ = O.run_seeded(c, 0, parallel=True)
    for mode in ("exact", "tiled"):
        ex = CudaStateVectorBackend.run(c, mode=mode)
        st = ex.state()
        assert exact(st.amplitudes(), want), mode
    shots = st.sample(10000, seed=2024)
    assert np.array_equal(shots, O.sample_tree(want, 2024, 10000))


def test_sample_matches_literal_collapse(gpu):
    for n in (1, 4, 9):
        amps, _, _ = O.run_seeded(workloads.random_layers(n, 5, seed=n))
        st = State.from_amplitudes(amps)
        assert np.array_equal(st.sample(400, seed=5), O.sample_literal(amps, 5, 400))


def test_midcircuit_measurement_and_classical_control(gpu):  # backend/mod.rs:51-72
    for seed in range(24):
        for c in (workloads.ghz_midmeasure(6), algorithms.teleport_state(0.6, 0.8j)):
            want, wbits, _ = O.run_seeded(c, seed)
            ex = CudaStateVectorBackend.run_seeded(c, seed)
            assert ex.classical() == wbits, seed
            assert np.max(np.abs(ex.state().amplitudes() - want)) < 1e-12
    # nested IfClassic, a conditional measurement that must not consume a uniform
    c = Circuit.with_classical(3, 3)
    c.h(0).h(1).measure(0, 0).measure(1, 1)
    c.if_classic(0, IfClassic(1, Apply1(Gate1.x(), 2)))
    c.if_classic(0, Measure(2, 2))
    c.h(2).measure(2, 2)
    for seed in range(32):
        want, wbits, _ = O.run_seeded(c, seed)
        ex = CudaStateVectorBackend.run_seeded(c, seed)
        assert ex.classical() == wbits, seed
        assert np.max(np.abs(ex.state().amplitudes() - want)) < 1e-12


def test_qft20_closed_form(gpu):
    n, j = 20, 0x5A5A5
    ex = CudaStateVectorBackend.run(workloads.qft_on_basis(n, j), mode="tiled")
    assert np.max(np.abs(ex.state().amplitudes() - workloads.qft_closed_form(n, j))) < 1e-12


@pytest.mark.parametrize("mode", ["exact", "tiled"])
def test_complex64_fidelity(gpu, mode):
    """complex64 runs (FP32 gate arithmetic, FP64 reductions and final
    renormalisation) against the complex128 oracle: fidelity >= 1 - 1e-6."""
    for n, depth in ((12, 20), (16, 10)):
        c = workloads.random_layers(n, depth, seed=4)
        want, _, _ = O.run_seeded(c, 0, parallel=True)
        st = CudaStateVectorBackend.run(c, dtype="complex64", mode=mode).state()
        got = st.amplitudes()
        fid = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
        assert fid >= 1 - 1e-6, (n, fid)
        assert abs(np.vdot(got, got).real - 1) < 1e-6
        assert np.max(np.abs(got - want)) < 1e-5
        ref = State.from_amplitudes(want, dtype="complex64")
        assert abs(st.fidelity(ref) - fid) < 1e-5


def test_errors_through_c_abi(gpu):
    st = State.zero(3)
    with pytest.raises(QubitOutOfRange):
        st.apply_1q(3, Gate1.h())
    with pytest.raises(DuplicateQubit):
        st.apply_2q(1, 1, Gate2.cnot())
    with pytest.raises(DuplicateQubit):
        st.apply_controlled_1q([0, 2], 2, Gate1.x())
    with pytest.raises(DimensionMismatch):
        st.upload(np.zeros(5, dtype=np.complex128))
    with pytest.raises(DimensionMismatch):
        State.from_amplitudes(np.zeros(3, dtype=np.complex128))
    c = Circuit(2)
    c.h(2)
    with pytest.raises(QubitOutOfRange):
        CudaStateVectorBackend.run(c)


def test_edge_sizes(gpu):
    # 0-qubit and 1-qubit registers
    c = Circuit(0)
    ex = CudaStateVectorBackend.run(c)
    assert ex.state().amplitudes().tolist() == [1 + 0j]
    assert ex.state().sample(5).tolist() == [0] * 5
    c = Circuit.with_classical(1, 1)
    c.h(0).measure(0, 0)
    for seed in range(10):
        want, bits, _ = O.run_seeded(c, seed)
        ex = CudaStateVectorBackend.run_seeded(c, seed, mode="tiled")
        assert ex.classical() == bits
        assert np.max(np.abs(ex.state().amplitudes() - want)) < 1e-12
    # empty circuit on many qubits, zero shots
    ex = CudaStateVectorBackend.run(Circuit(10))
    assert ex.state().probability(0) == 1.0
    assert ex.state().sample(0).shape == (0,)


def test_integer_pipe_product_matches_fp64_pipe(gpu):
    """The tile passes' integer-pipe double product is bit-identical to the
    FP64 pipe's on 2^30 operand pairs per seed, drawn to reach every
    rounding case (exact products, exact ties, carries into the exponent,
    the edges of the fast path's exponent range)."""
    import ctypes as C
    from everett_gb300 import _native as N
    for seed in (1, 2):
        bad = C.c_uint64(7)
        N.check(N.lib().ev_softfp_check(seed, 1 << 30, C.byref(bad)))
        assert bad.value == 0, (seed, bad.value)


def test_integer_pipe_add_matches_fp64(gpu):
    """The integer-pipe double add (softfp::add) gives the FP64 add's bits on
    2^28 operand pairs per seed: the product check's families, cancellation
    (opposite signs, changed low bits) and exponent gaps of 50..66 with random
    or empty fractions (the alignment's edges, exact ties)."""
    import ctypes as C
    from everett_gb300 import _native as N
    for seed in (1, 2):
        bad = C.c_uint64(7)
        N.check(N.lib().ev_softfp_add_check(seed, 1 << 28, C.byref(bad)))
        assert bad.value == 0, (seed, bad.value)
    rate = C.c_double()
    N.check(N.lib().ev_probe_softadd(C.byref(rate)))
    assert rate.value > 0


def test_double_float_rounding_matches_fp64_add(gpu):
    """The complex64 sampling tree rounds each leaf's double-float pair to
    f64 on the integer pipes; on 2^28 pairs per seed (exponent gaps 0..80,
    ties, cancellations) it gives the FP64 add's bits."""
    import ctypes as C
    from everett_gb300 import _native as N
    for seed in (1, 2):
        bad = C.c_uint64(7)
        N.check(N.lib().ev_ff_check(seed, 1 << 28, C.byref(bad)))
        assert bad.value == 0, (seed, bad.value)


@pytest.mark.parametrize("level", ["00", "11", "22", "21", "12", "32", "42", "62"])
def test_tiled_integer_pipe_levels_bit_exact(gpu, monkeypatch, level):
    """Every level of the complex128 tile passes' integer-pipe products
    (none, one amplitude per pair, both) and of real records' adds (one, two
    or all four output parts of a pair) gives the oracle's bits, including
    pairs that leave the fast path: zeros of the initial state, gate entries
    and amplitudes below 2^-511."""
    monkeypatch.setenv("EV_TILE_SOFT", level)
    rng = np.random.default_rng(17)
    n = 13
    c = Circuit(n)
    tiny = Gate1.ry(1e-160)  # entries and amplitudes far below the fast path's range
    for layer in range(6):
        for q in range(n):
            c.gate1(GATES_1Q[int(rng.integers(0, len(GATES_1Q)))], q)
            c.rz(q, float(rng.uniform(0, 6.3)))
        c.gate1(tiny, layer % n)
        c.controlled([int((layer + 3) % n)], Gate1.ry(float(rng.uniform(0, 6.3))), layer % n)
        for i in range(layer % 2, n - 1, 2):
            c.cnot(i, i + 1)
    want, _, _ = O.run_seeded(c, 0)
    for tb in (6, 10):
        got = CudaStateVectorBackend.run(c, mode="tiled", tile_bits=tb).state().amplitudes()
        assert exact(got, want), (level, tb)
    rl = workloads.random_layers(14, 6, 5)
    want, _, _ = O.run_seeded(rl, 0, parallel=True)
    assert exact(CudaStateVectorBackend.run(rl, mode="tiled").state().amplitudes(), want), level


@pytest.mark.parametrize("chain,shape", [("0", ""), ("1", ""), ("2", ""), ("3", ""),
                                         ("3", "256"), ("3", "1x512"), ("0", "256")])
def test_tiled_chains_bit_exact(gpu, monkeypatch, chain, shape):
    """The tile pass applies runs of records in registers: 1-qubit runs on
    one target with the same controls (pair chains), uncontrolled 1-qubit
    runs over two targets (quad chains) and runs of diagonal records (Rz,
    phase, Rzz: diagonal chains, which CZ and controlled phases break).  Every chaining
    level (none, pair, pair and quad, pair, quad and diagonal) and every
    block shape of the pass (two blocks of 512 threads, three of 256 reading
    their records through L1, one of 512) gives the oracle's bits, with every
    1-qubit kind, controls inside and outside the tile, and tiles of 4 to 12
    qubits."""
    monkeypatch.setenv("EV_TILE_CHAIN", chain)
    if shape:
        monkeypatch.setenv("EV_TILE_THREADS", shape)
    else:
        monkeypatch.delenv("EV_TILE_THREADS", raising=False)
    rng = np.random.default_rng(31)
    n = 13
    c = Circuit(n)
    for layer in range(5):
        for q in range(n):
            for _ in range(int(rng.integers(1, 4))):
                c.gate1(GATES_1Q[int(rng.integers(0, len(GATES_1Q)))], q)
            if rng.random() < 0.3:
                ctrl = [(q + int(rng.integers(1, n))) % n]
                for _ in range(int(rng.integers(1, 3))):
                    c.controlled(ctrl, GATES_1Q[int(rng.integers(0, len(GATES_1Q)))], q)
        for i in range(layer % 2, n - 1, 2):
            c.cnot(i, i + 1)
        # a run of diagonal records: Rz, phase, controlled phase, CZ, Rzz
        for i in range(n - 1):
            [lambda: c.gate1(Gate1.rz(0.3 + i), i),
             lambda: c.controlled([(i + 5) % n], Gate1.phase(0.2 * i), i),
             lambda: c.gate2(Gate2.cz(), i, i + 1),
             lambda: c.gate2(Gate2.rzz(0.1 + 0.05 * i), i, i + 1),
             lambda: c.gate1(Gate1.t(), i)][(i + layer) % 5]()
    want, _, _ = O.run_seeded(c, 0)
    for tb in (4, 6, 9, 12):
        got = CudaStateVectorBackend.run(c, mode="tiled", tile_bits=tb).state().amplitudes()
        assert exact(got, want), (chain, tb)
    rl = workloads.random_layers(16, 6, 9)
    want, _, _ = O.run_seeded(rl, 0, parallel=True)
    assert exact(CudaStateVectorBackend.run(rl, mode="tiled").state().amplitudes(), want), chain


def test_gates_on_mixed_range_amplitudes_bit_exact(gpu):
    """The complex128 gate kernels form plain products on the integer pipes
    for operands in a normal range and fall back pair by pair otherwise: a
    state mixing zeros, signed zeros, tiny (1e-200) and huge (1e200) parts and
    ordinary values gives the oracle's bits for every 1-qubit kind, plain and
    controlled."""
    rng = np.random.default_rng(23)
    n = 9
    base = O.sample_state(n)
    pick = rng.integers(0, 6, size=(1 << n, 2))
    parts = base.view(np.float64).reshape(-1, 2).copy()
    parts[pick == 1] = 0.0
    parts[pick == 2] = -0.0
    parts[pick == 3] *= 1e-200
    parts[pick == 4] *= 1e200
    mixed = parts.reshape(-1).view(np.complex128).copy()
    st = State.from_amplitudes(mixed)
    for k in range(n):
        for g in GATES_1Q:
            st.upload(mixed)
            st.apply_1q(k, g)
            want = mixed.copy()
            O.apply_1q(want, k, g)
            assert exact(st.amplitudes(), want), (k, g)
            st.upload(mixed)
            st.apply_controlled_1q([(k + 1) % n], k, g)
            want = mixed.copy()
            O.apply_controlled_1q(want, [(k + 1) % n], k, g)
            assert exact(st.amplitudes(), want), ("ctrl", k, g)
