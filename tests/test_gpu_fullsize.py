"""Full-size checks at the benchmark's 30 qubits (16 GiB complex128,
8 GiB complex64), where the oracle cannot follow, through properties that
do not depend on size:

  QFT|j>        every sampled amplitude equals the closed form
                e^{2 pi i jk / 2^30} / 2^15 (jk reduced mod 2^30 first)
  IQFT QFT|j>   returns |j>: amplitude 1 at j, 0 elsewhere (sampled)
  random layers depth 20 keeps the norm at 1; the complex64 fused run has
                fidelity >= 1 - 1e-6 against complex128 and its max amplitude
                error is at the FP32 level
  GHZ(30)       every shot is all-zeros or all-ones; measuring qubit 0
                collapses every other qubit to the same value

Tolerances are written per check.  Together these take ~40 s and ~28 GiB of
HBM."""
import math

import numpy as np
import pytest

from everett_gb300 import Circuit, CudaStateVectorBackend, State, algorithms, workloads

pytestmark = pytest.mark.gpu

N30 = 30


def sampled_indices(rng, n, count, must=()):
    idx = set(int(v) for v in rng.integers(0, 1 << n, size=count))
    idx.update(must)
    return sorted(idx)


def test_qft_closed_form_30q(gpu):
    rng = np.random.default_rng(30)
    j = int(rng.integers(0, 1 << N30))
    st = State.zero(N30, "complex128")
    CudaStateVectorBackend.run_into(st, workloads.qft_on_basis(N30, j), 0, mode="tiled")
    dim = 1 << N30
    worst = 0.0
    for k in sampled_indices(rng, N30, 512, must=(0, 1, dim - 1, j)):
        ph = (j * k) % dim
        ang = math.tau * ph / dim
        want = complex(math.cos(ang), math.sin(ang)) / math.sqrt(dim)
        worst = max(worst, abs(st.amplitude(k) - want))
    assert worst < 1e-12, worst
    assert abs(st.norm_sqr() - 1.0) < 1e-12


def test_qft_round_trip_30q(gpu):
    rng = np.random.default_rng(31)
    j = int(rng.integers(0, 1 << N30))
    c = workloads.qft_on_basis(N30, j)
    c.compose(algorithms.iqft(N30))
    st = State.zero(N30, "complex128")
    CudaStateVectorBackend.run_into(st, c, 0, mode="tiled")
    assert abs(st.amplitude(j) - 1.0) < 1e-12
    for k in sampled_indices(rng, N30, 256):
        if k != j:
            assert abs(st.amplitude(k)) < 1e-12, k
    assert st.probability(j) > 1 - 1e-12


def test_random_layers_norm_and_complex64_fidelity_30q(gpu):
    c = workloads.random_layers(N30, 20, seed=1)
    ref = State.zero(N30, "complex128")
    CudaStateVectorBackend.run_into(ref, c, 0, mode="tiled")
    assert abs(ref.norm_sqr() - 1.0) < 1e-12
    st = State.zero(N30, "complex64")
    CudaStateVectorBackend.run_into(st, c, 0, mode="fused", variant="bf16x3", tile_bits=5)
    ov = ref.overlap(st)
    fid = abs(ov) ** 2 / (ref.norm_sqr() * st.norm_sqr())
    assert fid >= 1 - 1e-6, fid
    # amplitudes are ~2^-15 in size; FP32 storage alone is ~2^-39 absolute
    assert ref.max_abs_diff(st) < 1e-6
    # The run ends with an FP64 renormalisation applied with one rounding per
    # amplitude; the norm of the FP32-stored result is then 1 to ~1e-10 at
    # every size (a factor within one ulp of 1 rounds each amplitude in a
    # direction tied to its mantissa, so the errors do not average out).
    assert abs(st.norm_sqr() - 1.0) < 1e-9
    del st
    # complex128 fused on the tensor cores (digit slicing) against the
    # bit-exact tiled complex128 result, to the complex128 bar of 1e-12
    oz = State.zero(N30, "complex128")
    CudaStateVectorBackend.run_into(oz, c, 0, mode="fused", variant="ozaki")
    assert ref.max_abs_diff(oz) <= 1e-12
    ov = ref.overlap(oz)
    assert abs(ov) ** 2 >= 1 - 1e-12


def test_ghz_shots_and_collapse_30q(gpu):
    g = algorithms.ghz(N30)
    st = State.zero(N30, "complex64")
    CudaStateVectorBackend.run_into(st, g, 0, mode="tiled")
    shots = st.sample(2000, seed=3)
    full = (1 << N30) - 1
    assert set(np.unique(shots).tolist()) <= {0, full}
    ones = int(np.sum(shots == full))
    assert 850 < ones < 1150  # Binomial(2000, 1/2): 6.7 sigma either side
    c = Circuit.with_classical(N30, 2)
    c.compose(g)
    c.measure(0, 0).measure(N30 - 1, 1)
    for seed in range(4):
        ex = CudaStateVectorBackend.run_seeded(c, seed, dtype="complex64", mode="tiled")
        bits = ex.classical()
        assert bits[0] == bits[1]
        want = full if bits[0] else 0
        assert abs(ex.state().probability(want) - 1.0) < 1e-6


def test_ghz_pauli_expectations_30q(gpu):
    """GHZ(30) = (|0...0> + |1...1>)/sqrt 2 in complex64: <Z^30> = <Z0 Z29> =
    <X^30> = 1 and <Z0> = <X0 X2> = 0, whatever the size.  One call covers the
    Z-only pass, a shared X mask on the top qubit and an X mask inside the
    low three qubits.  The amplitudes are fl32(1/sqrt 2), whose doubled square
    is 1 - 6e-8: the bar is 1e-6 for the unit values, 1e-12 for the zeros
    (the two contributions cancel exactly)."""
    st = State.zero(N30, "complex64")
    CudaStateVectorBackend.run_into(st, algorithms.ghz(N30), 0, mode="tiled")
    strings = ["+" + "Z" * N30, "+Z" + "I" * (N30 - 1), "+Z" + "I" * (N30 - 2) + "Z",
               "+" + "X" * N30, "-" + "X" * N30, "+XIX" + "I" * (N30 - 3)]
    got = st.pauli_expectation(strings)
    want = [1.0, 0.0, 1.0, 1.0, -1.0, 0.0]
    for s, g, w in zip(strings, got, want):
        assert abs(g - w) < (1e-6 if w else 1e-12), (s[:6], g, w)
