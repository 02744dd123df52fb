"""GPU parity of the fused paths: dense k-qubit unitaries applied on tensor
cores (complex64: TF32x3, BF16x3; complex128: 8-bit digit slices, the Ozaki
scheme) or CUDA cores (complex64 FP32), against the complex128 oracle.
Bars: complex64 fidelity >= 1 - 1e-6 and max |amplitude error| <= 1e-5 (the
complex64 storage alone rounds at ~6e-8 relative per pass); complex128
max |amplitude error| <= 1e-12 and identical measurement outcomes."""
import numpy as np
import pytest

import oracle as O
from everett_gb300 import Circuit, CudaStateVectorBackend, Gate1, Gate2, algorithms, workloads

pytestmark = pytest.mark.gpu

VARIANTS = [("tf32x3", 5), ("bf16x3", 5), ("bf16x3", 6), ("fp32", 5), ("fp32", 3)]


def fidelity(a, b):
    return abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)


def check(c, variant, k, seed=0, fid_bar=1 - 1e-6, err_bar=1e-5):
    want, wbits, rc = O.run_seeded(c, seed, parallel=True)
    assert rc == 0
    ex = CudaStateVectorBackend.run_seeded(c, seed, dtype="complex64", mode="fused",
                                           tile_bits=k, variant=variant)
    got = ex.state().amplitudes()
    f = fidelity(want, got)
    err = float(np.max(np.abs(got - want)))
    assert f >= fid_bar, (variant, k, f)
    assert err <= err_bar, (variant, k, err)
    return ex, wbits, f, err


@pytest.mark.parametrize("variant,k", VARIANTS)
def test_fused_random_layers(gpu, variant, k):
    check(workloads.random_layers(14, 12, seed=5), variant, k)


@pytest.mark.parametrize("variant,k", VARIANTS)
def test_fused_haar_cz(gpu, variant, k):
    check(workloads.haar_layers(15, 10, seed=6), variant, k)


@pytest.mark.parametrize("variant,k", VARIANTS)
def test_fused_qft_and_controls(gpu, variant, k):
    n, j = 13, 4321
    c = workloads.qft_on_basis(n, j)
    ex, _, _, _ = check(c, variant, k)
    got = ex.state().amplitudes()
    assert np.max(np.abs(got - workloads.qft_closed_form(n, j))) < 1e-5
    # multi-controlled gates and dense 2-qubit gates across fused blocks
    rng = np.random.default_rng(k)
    c = Circuit(14)
    for _ in range(80):
        qs = [int(x) for x in rng.choice(14, 4, replace=False)]
        c.ry(qs[0], float(rng.uniform(0, 6)))
        c.controlled(qs[1:3], Gate1.rx(float(rng.uniform(0, 6))), qs[0])
        c.gate2(Gate2.rzz(float(rng.uniform(0, 6))), qs[2], qs[3])
    check(c, variant, k)


@pytest.mark.parametrize("variant,k", VARIANTS[:3])
def test_fused_midcircuit_measurement(gpu, variant, k):
    c = workloads.ghz_midmeasure(16)
    c.compose(workloads.random_layers(16, 3, seed=2))
    for seed in range(6):
        ex, wbits, _, _ = check(c, variant, k, seed=seed)
        assert ex.classical() == wbits


def test_fused_small_registers_use_tile_pass(gpu):
    for n in (1, 3, 7, 11):
        check(workloads.random_layers(n, 6, seed=n), "tf32x3", 5)


@pytest.mark.parametrize("variant", ["bf16x3", "tf32x3"])
def test_fused_tma_staging(gpu, variant, monkeypatch):
    """The warp-specialised TMA-staged pipeline gives the same results."""
    monkeypatch.setenv("EV_FUSED_STAGING", "tma")
    check(workloads.random_layers(15, 10, seed=12), variant, 5)
    check(workloads.haar_layers(16, 6, seed=13), variant, 5)
    c = workloads.ghz_midmeasure(14)
    c.compose(workloads.random_layers(14, 3, seed=2))
    ex, wbits, _, _ = check(c, variant, 5, seed=3)
    assert ex.classical() == wbits


OZAKI = pytest.mark.parametrize("variant", ["ozaki", "ozaki6"])


def check128(c, seed=0, variant="ozaki"):
    want, wbits, rc = O.run_seeded(c, seed, parallel=True)
    assert rc == 0
    ex = CudaStateVectorBackend.run_seeded(c, seed, dtype="complex128", mode="fused",
                                           variant=variant)
    got = ex.state().amplitudes()
    err = float(np.max(np.abs(got - want)))
    assert err <= 1e-12, err
    assert ex.classical() == wbits
    return ex, err


@OZAKI
def test_ozaki_complex128_circuits(gpu, variant):
    """Random layers, Haar layers with CZ bricks, QFT (closed form), multi-
    controlled and dense 2-qubit gates across blocks: max error <= 1e-12,
    with seven digits and with six."""
    check128(workloads.random_layers(14, 12, seed=5), variant=variant)
    check128(workloads.random_layers(18, 20, seed=8), variant=variant)
    check128(workloads.haar_layers(15, 10, seed=6), variant=variant)
    n, j = 13, 4321
    ex, _ = check128(workloads.qft_on_basis(n, j), variant=variant)
    assert np.max(np.abs(ex.state().amplitudes() - workloads.qft_closed_form(n, j))) < 1e-12
    rng = np.random.default_rng(3)
    c = Circuit(14)
    for _ in range(80):
        qs = [int(x) for x in rng.choice(14, 4, replace=False)]
        c.ry(qs[0], float(rng.uniform(0, 6)))
        c.controlled(qs[1:3], Gate1.rx(float(rng.uniform(0, 6))), qs[0])
        c.gate2(Gate2.rzz(float(rng.uniform(0, 6))), qs[2], qs[3])
    check128(c, variant=variant)


@OZAKI
def test_ozaki_complex128_measurement_and_small_registers(gpu, variant):
    """Mid-circuit measurement and classical control between fused runs give
    the oracle's outcomes; registers below 12 qubits take the tile pass."""
    c = workloads.ghz_midmeasure(16)
    c.compose(workloads.random_layers(16, 3, seed=2))
    for seed in range(6):
        check128(c, seed=seed, variant=variant)
    for n in (1, 3, 7, 11, 12):
        check128(workloads.random_layers(n, 6, seed=n), variant=variant)


@OZAKI
def test_ozaki_complex128_rows_of_mixed_scale(gpu, variant):
    """Each row of a step is scaled by its own largest exponent: on an
    uploaded state whose rows differ in scale by up to 1e-30 (and hold exact
    zeros), one fused block on each qubit window matches the oracle row by
    row to 1e-14 of the row's largest amplitude with seven digits (2^-39,
    the six-digit form's proven bound, with six), and to 1e-12 absolute."""
    from everett_gb300 import State
    rng = np.random.default_rng(4)
    n = 13
    for lo in (0, 3, 8):
        mask = 31 << lo
        idx = np.arange(1 << n)
        key = idx & ~mask
        # one scale per row (the 32 amplitudes that agree outside the window)
        scale = np.exp(rng.uniform(-69, 0, size=1 << n))[key]
        amps = O.sample_state(n) * scale
        amps[rng.integers(0, 1 << n, size=200)] = 0
        amps /= np.linalg.norm(amps)
        c = Circuit(n)
        for q in range(lo, lo + 5):
            c.rx(q, 0.3 + q).rz(q, 1.1 * q)
        c.cnot(lo, lo + 4).cz(lo + 1, lo + 3)
        want = amps.copy()
        O.apply_ops(c, want, 0, len(c))
        st = State.from_amplitudes(amps)
        CudaStateVectorBackend.drive(st, c, 0, mode="fused", variant=variant)
        got = st.amplitudes()
        assert np.max(np.abs(got - want)) <= 1e-12, lo
        order = np.argsort(key, kind="stable")
        g, w = got[order].reshape(-1, 32), want[order].reshape(-1, 32)
        rowmax = np.abs(w).max(axis=1)
        rel = np.abs(g - w).max(axis=1) / np.where(rowmax > 0, rowmax, 1)
        assert rel.max() <= (1e-14 if variant == "ozaki" else 2.0 ** -39), (lo, rel.max())


@OZAKI
def test_ozaki_reports_non_finite_amplitudes(gpu, variant):
    """Fixed-point digits cannot carry a NaN or an infinity: a fused
    complex128 pass over a state holding one reports it as an invalid
    argument instead of returning finite numbers, and the next run on the
    same state is unaffected."""
    import everett_gb300.error as E
    from everett_gb300 import State
    n = 13
    c = workloads.random_layers(n, 2, seed=4)
    for bad in (float("nan"), float("inf")):
        amps = O.sample_state(n) / np.sqrt(float(1 << n))
        amps[777] = complex(bad, 0.0)
        st = State.from_amplitudes(amps)
        with pytest.raises(E.InvalidArgument):
            CudaStateVectorBackend.drive(st, c, 0, mode="fused", variant=variant)
        CudaStateVectorBackend.run_into(st, c, 0, mode="fused", variant=variant)
        want, _, _ = O.run_seeded(c, 0)
        assert np.max(np.abs(st.amplitudes() - want)) <= 1e-12


def test_ozaki_rejects_complex64_and_complex64_variants_reject_complex128(gpu):
    import everett_gb300.error as E
    c = workloads.random_layers(13, 2, seed=1)
    for v in ("ozaki", "ozaki6"):
        with pytest.raises(E.EverettError):
            CudaStateVectorBackend.run(c, dtype="complex64", mode="fused", variant=v)
    with pytest.raises(E.EverettError):
        CudaStateVectorBackend.run(c, dtype="complex128", mode="fused", variant="bf16x3")
