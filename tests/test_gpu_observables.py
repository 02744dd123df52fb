"""Pauli-string expectations on the device against the oracle's restatement
of PauliString::expectation (apply P to a copy, then Re <P psi|psi>,
backend/stabilizer.rs:79-125).

Bars: 1e-12 absolute in complex128 and, in complex64, against the oracle on
the same complex64 amplitudes (double-float sums on the FP32 pipe); the
stabilizer generators of a Clifford state have expectation 1 to 1e-12
(tests/stabilizer.rs:13-25 uses the statevector the same way)."""
import numpy as np
import pytest

import oracle as O
from everett_gb300 import Circuit, algorithms, CudaStateVectorBackend, PauliString, State, workloads
from everett_gb300.error import QubitOutOfRange

pytestmark = pytest.mark.gpu


def random_paulis(rng, n, count):
    out = []
    for _ in range(count):
        x = rng.integers(0, 2, n).astype(bool)
        z = rng.integers(0, 2, n).astype(bool)
        out.append(PauliString(x, z, bool(rng.integers(0, 2))))
    return out


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_pauli_expectation_matches_oracle(gpu, dtype):
    rng = np.random.default_rng(11)
    for n in (1, 2, 3, 7, 12, 17):
        amps, _, _ = O.run_seeded(workloads.random_layers(n, 3, seed=n + 3))
        st = State.from_amplitudes(amps, dtype=dtype)
        ref = np.ascontiguousarray(st.amplitudes())
        ps = random_paulis(rng, n, 40)
        # plus diagonal strings sharing x = 0 and strings sharing one X part
        ps += [PauliString([False] * n, rng.integers(0, 2, n).astype(bool)) for _ in range(10)]
        x = rng.integers(0, 2, n).astype(bool)
        ps += [PauliString(x, rng.integers(0, 2, n).astype(bool), bool(rng.integers(0, 2)))
               for _ in range(19)]
        # X parts within qubits 0..2: each index's partner lies in its own
        # aligned block of 8
        for low in ((True,), (False, True), (True, False, True)):
            if len(low) > n:
                continue
            xl = np.zeros(n, dtype=bool)
            xl[:len(low)] = low
            ps += [PauliString(xl, rng.integers(0, 2, n).astype(bool), bool(rng.integers(0, 2)))
                   for _ in range(6)]
        got = st.pauli_expectation(ps)
        for p, g in zip(ps, got):
            xm, zm = p.masks()
            want = O.pauli_expectation(ref, xm, zm, p.neg)
            assert abs(g - want) < 1e-12, (n, dtype, str(p), g, want)
        # grouped evaluation equals one string at a time
        single = np.array([p.expectation(st) for p in ps[:12]])
        assert np.max(np.abs(single - got[:12])) < 1e-13


def test_clifford_state_stabilizers(gpu):
    n = 5
    c = Circuit(n)
    c.h(0)
    for q in range(n - 1):
        c.cnot(q, q + 1)
    c.s(2).h(3)
    st = CudaStateVectorBackend.run(c).state()
    # GHZ stabilizers XXXXX, Z_q Z_{q+1}, conjugated by S on qubit 2 and H on 3
    gens = ["+XXYZX", "+ZZIII", "+IZZII", "+IIZXI", "+IIIXZ"]
    vals = st.pauli_expectation(gens)
    assert np.max(np.abs(vals - 1.0)) < 1e-12, vals
    assert abs(st.pauli_expectation(["-XXYZX"])[0] + 1.0) < 1e-12
    assert abs(st.pauli_expectation(["+ZIIII"])[0]) < 1e-12


def test_pauli_expectation_rejects_foreign_qubits(gpu):
    st = State.zero(3)
    with pytest.raises(ValueError):
        PauliString.parse("+XXXX").expectation(st)
    import ctypes as C
    from everett_gb300 import _native as N
    xm = np.array([1 << 5], dtype=np.uint64)
    zm = np.zeros(1, dtype=np.uint64)
    out = np.zeros(1)
    rc = N.lib().ev_pauli_expectation(st.handle, xm.ctypes.data, zm.ctypes.data, None, 1,
                                      out.ctypes.data)
    assert rc == N.ERR_QUBIT_OUT_OF_RANGE


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_marginal_low_and_phase_estimation(gpu, dtype):
    """most_probable_phase's marginal as a device reduction: identical to the
    oracle's basis-order sums in complex128 (1e-12 in complex64, against the
    oracle on the same complex64 amplitudes), and the reference's
    phase-estimation and superdense assertions hold on the GPU
    (algorithms_phase_estimation.rs:12-36, algorithms_superdense.rs:5-36)."""
    for n, m in [(1, 0), (6, 3), (12, 12), (17, 5)]:
        amps = O.sample_state(n) if n > 1 else np.array([0.6, 0.8j])
        st = State.from_amplitudes(amps, dtype=dtype)
        got = st.marginal_low(m)
        want = O.marginal_low(np.ascontiguousarray(st.amplitudes(), dtype=np.complex128), m)
        if dtype == "complex128":
            assert np.array_equal(got, want), (n, m)
        else:
            assert np.max(np.abs(got - want)) < 1e-12, (n, m)
    for m, phi in [(1, 0.5), (2, 0.25), (2, 0.75), (3, 0.125), (3, 0.875), (4, 0.0)]:
        ex = CudaStateVectorBackend.run(algorithms.phase_estimation(m, phi))
        assert abs(algorithms.most_probable_phase(ex.state(), m) - phi) < 1e-10
    ex = CudaStateVectorBackend.run(algorithms.phase_estimation(4, 0.3))
    assert abs(algorithms.most_probable_phase(ex.state(), 4) - 0.3) <= 1.0 / 16.0 + 1e-10
    for b0 in (False, True):
        for b1 in (False, True):
            ex = CudaStateVectorBackend.run(algorithms.superdense_circuit(b0, b1))
            assert list(ex.classical()) == [b0, b1]
