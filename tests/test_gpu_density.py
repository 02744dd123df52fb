"""Density matrices on the GPU against the oracle's restatement of
DensityMatrixBackend (src/density.rs, src/noise.rs,
src/backend/density_matrix.rs).

Bars: gates and noise channels bit-identical to the oracle (== on every
element; the engine fuses U rho U^dagger into one pass but keeps every
product and sum); after a measurement 1e-12 (the probability sums run in a
different order) with identical classical bits; observables 1e-12.
The oracle's controlled gates go through the reference's full 2^n x 2^n
unitary, so circuits with controls stay at n <= 6."""
import numpy as np
import pytest

import oracle as O
from everett_gb300 import Circuit, Gate1, Gate2, workloads
from everett_gb300.density import (Channel, DensityMatrix, DensityMatrixBackend, KrausOp,
                                   NoiseModel)
from everett_gb300.error import DimensionMismatch, QubitOutOfRange

pytestmark = pytest.mark.gpu

NOISES = {
    "ideal": NoiseModel.ideal(),
    "depolarizing": NoiseModel.uniform_depolarizing(0.03),
    "amplitude_damping": NoiseModel.amplitude_damping(0.07),
    "phase_damping": NoiseModel.phase_damping(0.2),
    "bit_flip": NoiseModel.bit_flip(0.05),
    "dephasing": NoiseModel.dephasing(0.11),
    "custom": NoiseModel(Channel.custom([[0.6, 0, 0, 0.8], [0, 0.8, 0.6, 0]]),
                         Channel.custom([[1, 0, 0, 0.9], [0, 0.1, 0, 0], [0, 0, 0.3, 0]])),
}


def mixed_circuit(n, seed, measure=False):
    rng = np.random.default_rng(seed)
    c = Circuit.with_classical(n, 2) if measure else Circuit(n)
    gates1 = [Gate1.h(), Gate1.x(), Gate1.y(), Gate1.s(), Gate1.t(), Gate1.rx(0.7), Gate1.ry(-1.1),
              Gate1.rz(2.3), Gate1.phase(0.4), Gate1(0.6 + 0.1j, -0.3 + 0.2j, 0.25 - 0.7j, 0.1)]
    for _ in range(4 * n):
        kind = int(rng.integers(0, 4))
        qs = [int(v) for v in rng.choice(n, min(n, 3), replace=False)]
        if kind == 0 or n < 2:
            c.gate1(gates1[int(rng.integers(0, len(gates1)))], qs[0])
        elif kind == 1:
            g = [Gate2.cnot(), Gate2.cz(), Gate2.swap(), Gate2.rzz(0.3),
                 Gate2(rng.normal(size=16) + 1j * rng.normal(size=16))][int(rng.integers(0, 5))]
            c.gate2(g, qs[0], qs[1])
        elif kind == 2:
            c.controlled(qs[1:], gates1[int(rng.integers(0, len(gates1)))], qs[0])
        else:
            c.gate1(gates1[int(rng.integers(0, len(gates1)))], qs[-1])
    if measure:
        c.measure(0, 0).x_if(0, n - 1)
        c.gate1(Gate1.h(), 0).measure(n - 1, 1)
        c.if_classic(1, workloads_controlled_x(n))
    return c


def workloads_controlled_x(n):
    from everett_gb300.circuit import Controlled
    return Controlled((0,), Gate1.x(), n - 1)


@pytest.mark.parametrize("noise", list(NOISES))
def test_noisy_gates_bit_exact(gpu, noise):
    for n in (1, 2, 3, 5):
        c = mixed_circuit(n, 10 * n + len(noise))
        nm = NOISES[noise]
        want, _ = O.dm_run(c, nm.ev_struct())
        got = DensityMatrixBackend.run_with_noise(c, nm).density_matrix().data()
        assert np.array_equal(got, want), (noise, n)


@pytest.mark.parametrize("noise", ["ideal", "depolarizing", "amplitude_damping"])
def test_measurement_and_readout(gpu, noise):
    nm = NOISES[noise]
    nm_ro = NoiseModel(nm.after_1q, nm.after_2q, readout_error=0.2)
    for n in (2, 4):
        c = mixed_circuit(n, 3 + n, measure=True)
        for seed in range(12):
            for model in (nm, nm_ro):
                want, wbits = O.dm_run(c, model.ev_struct(), seed)
                ex = DensityMatrixBackend.run_with_noise_seeded(c, model, seed)
                assert ex.classical() == wbits, (noise, n, seed)
                got = ex.density_matrix().data()
                assert np.max(np.abs(got - want)) < 1e-12, (noise, n, seed)


def test_larger_registers_without_controls(gpu):
    """Gate-only circuits (no full-register unitaries in the oracle) at sizes
    with multi-block grids."""
    for n in (7, 9):
        c = workloads.random_layers(n, 2, seed=n)
        nm = NoiseModel.uniform_depolarizing(0.01)
        want, _ = O.dm_run(c, nm.ev_struct())
        got = DensityMatrixBackend.run_with_noise(c, nm).density_matrix().data()
        assert np.array_equal(got, want), n


def test_observables_match_oracle(gpu):
    n = 5
    c = mixed_circuit(n, 77)
    nm = NoiseModel.uniform_depolarizing(0.05)
    want, _ = O.dm_run(c, nm.ev_struct())
    rho = DensityMatrixBackend.run_with_noise(c, nm).density_matrix()
    for q in range(n):
        ob = O.dm_observables(want, q)
        assert abs(rho.trace() - ob["trace"]) < 1e-12
        assert abs(rho.purity() - ob["purity"]) < 1e-12
        for p in "IXYZ":
            assert abs(rho.expectation_pauli(q, p) - ob[p]) < 1e-12, (q, p)
        red = rho.partial_trace_1q(q)
        assert np.max(np.abs(np.array(red) - ob["reduced"])) < 1e-12
    for b in (0, 7, 31):
        assert rho.probability(b) == want[b, b].real
    assert rho.get(3, 17) == want[3, 17]


def test_from_statevector_and_reference_properties(gpu):
    amps, _, _ = O.run_seeded(workloads.random_layers(4, 3, seed=2))
    rho = DensityMatrix.from_statevector(amps)
    assert np.array_equal(rho.data(), O.dm_from_amplitudes(amps))
    assert abs(rho.purity() - 1.0) < 1e-12                           # pure state
    with pytest.raises(DimensionMismatch):
        DensityMatrix.from_statevector(np.ones(3))
    # density_matrix.rs tests: ideal Bell probabilities, purity, trace under noise,
    # amplitude damping decays |1>, dephasing kills coherences
    bell = Circuit(2)
    bell.h(0).cnot(0, 1)
    ideal = DensityMatrixBackend.run(bell).density_matrix()
    assert abs(ideal.probability(0) - 0.5) < 1e-12 and abs(ideal.probability(3) - 0.5) < 1e-12
    assert abs(ideal.purity() - 1.0) < 1e-10
    noisy = DensityMatrixBackend.run_with_noise(bell, NoiseModel.uniform_depolarizing(0.1))
    assert noisy.density_matrix().purity() < 1.0
    assert abs(noisy.density_matrix().trace() - 1.0) < 1e-10
    x = Circuit(1)
    x.x(0)
    assert DensityMatrixBackend.run_with_noise(
        x, NoiseModel.amplitude_damping(0.99)).density_matrix().probability(0) > 0.9
    h = Circuit(1)
    h.h(0)
    r = DensityMatrixBackend.run_with_noise(h, NoiseModel.dephasing(0.5)).density_matrix()
    assert abs(r.get(0, 1)) < 1e-12 and abs(r.get(1, 0)) < 1e-12
    with pytest.raises(QubitOutOfRange):
        r.partial_trace_1q(1)
