"""GPU parity of the complex64 fused path: dense k-qubit unitaries applied on
tensor cores (TF32x3, BF16x3) or CUDA cores (FP32), against the complex128
oracle.  Bar: fidelity >= 1 - 1e-6 and max |amplitude error| <= 1e-5 (the
complex64 storage alone rounds at ~6e-8 relative per pass)."""
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
