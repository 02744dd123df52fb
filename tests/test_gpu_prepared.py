"""Prepared runs: a circuit planned once and replayed as one CUDA graph.

Bar: every launch gives exactly what ``run_into`` (ev_state_run) gives for
the same circuit, options and seed -- amplitudes compared with == (both paths
run the same kernels on the same records) and the classical register equal.
"""
import gc

import numpy as np
import pytest

import oracle as O
from everett_gb300 import (Apply1, Circuit, CudaStateVectorBackend, Gate1, Gate2, IfClassic,
                           Measure, PreparedRun, State, algorithms, workloads)
from everett_gb300 import _native as N
from everett_gb300.error import DimensionMismatch, EverettError

pytestmark = pytest.mark.gpu


def control_flow_circuit(n: int, seed: int) -> Circuit:
    """Gates, mid-circuit measurements, single and nested classical control."""
    rng = np.random.default_rng(seed)
    c = Circuit.with_classical(n, 4)
    for q in range(n):
        c.h(q)
    for layer in range(3):
        for q in range(n):
            c.ry(q, float(rng.uniform(0, 6.3)))
        for q in range(layer % 2, n - 1, 2):
            c.cnot(q, q + 1)
        c.measure(layer, layer)
        c.x_if(layer, (layer + 2) % n)
    c.controlled([1, 3], Gate1.rx(0.4), 0)
    c.gate2(Gate2.rzz(0.3), 2, n - 1)
    c.if_classic(0, IfClassic(1, Apply1(Gate1.h(), n - 2)))
    c.measure(n - 1, 3)
    return c


def plain(state, c, seed, **kw):
    cl = CudaStateVectorBackend.run_into(state, c, seed, **kw)
    return state.amplitudes(), cl


@pytest.mark.parametrize("dtype,mode,kw", [
    ("complex128", "exact", {}),
    ("complex128", "tiled", {}),
    ("complex64", "tiled", {}),
    ("complex64", "fused", {"variant": "bf16x3"}),
    ("complex64", "fused", {"variant": "tf32x3"}),
    ("complex64", "fused", {"variant": "fp32", "tile_bits": 4}),
    ("complex128", "fused", {"variant": "ozaki"}),
    ("complex128", "fused", {"variant": "ozaki6"}),
])
def test_prepared_equals_run(gpu, dtype, mode, kw):
    n = 14
    c = workloads.ghz_midmeasure(n).compose(workloads.random_layers(n, 4, 3))
    c.measure(2, 0)
    st = State.zero(n, dtype)
    ref = State.zero(n, dtype)
    prep = CudaStateVectorBackend.prepare(st, c, mode=mode, **kw)
    assert prep.kernels() > 0
    for seed in (0, 1, 7, 12345):
        got_cl = prep.launch(seed)
        want, want_cl = plain(ref, c, seed, mode=mode, **kw)
        assert got_cl == want_cl, (seed, dtype, mode)
        assert np.array_equal(st.amplitudes(), want), (seed, dtype, mode)
    prep.close()


def test_prepared_control_flow_matches_oracle(gpu):
    """Single and nested IfClassic chains, a conditional measurement and
    several measurements: the classical register equals the oracle's and the
    amplitudes agree to 1e-12 (a collapse divides by the square root of a
    probability the GPU sums in a different order), while replay and
    ``run_into`` agree bit for bit."""
    n = 8
    c = control_flow_circuit(n, 5)
    c.if_classic(3, Measure(0, 1))
    st = State.zero(n)
    ref = State.zero(n)
    prep = PreparedRun(st, c)
    for seed in range(8):
        cl = prep.launch(seed)
        want, want_cl, _ = O.run_seeded(c, seed)
        assert cl == [bool(b) for b in want_cl], seed
        got = st.amplitudes()
        assert np.max(np.abs(got - want)) < 1e-12, seed
        assert CudaStateVectorBackend.run_into(ref, c, seed) == cl
        assert np.array_equal(ref.amplitudes(), got), seed


def test_prepared_outlives_circuit_and_repeats(gpu):
    n = 10
    st = State.zero(n)
    c = workloads.ghz_midmeasure(n)
    prep = PreparedRun(st, c, mode="tiled")
    del c
    gc.collect()
    first = prep.launch(3)
    a1 = st.amplitudes()
    st.upload(np.ones(1 << n) / np.sqrt(1 << n))  # the launch resets the state
    assert prep.launch(3) == first
    assert np.array_equal(st.amplitudes(), a1)


def test_prepared_counts_launches(gpu):
    n = 12
    st = State.zero(n)
    c = workloads.random_layers(n, 3, 1)
    prep = PreparedRun(st, c, mode="exact")
    k = prep.kernels()
    before = C_launches(st)
    prep.launch(0)
    prep.launch(1)
    assert C_launches(st) - before == 2 * k
    # exact mode: one kernel per gate plus the reset
    assert k >= len(c)
    # the default (tiled) mode: one kernel per tile pass
    assert PreparedRun(st, c).kernels() < len(c) // 4


def C_launches(st):
    import ctypes as C
    out = C.c_uint64()
    N.check(N.lib().ev_state_launch_count(st.handle, C.byref(out)))
    return out.value


def test_prepare_rejects_mismatches(gpu):
    st = State.zero(6)
    with pytest.raises(DimensionMismatch):
        PreparedRun(st, algorithms.ghz(7))
    with pytest.raises(EverettError):  # a complex64 arithmetic on a complex128 state
        PreparedRun(st, algorithms.ghz(6), mode="fused", variant="bf16x3")
