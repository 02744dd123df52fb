"""GPU parity of the batched runner against the oracle.

complex128 batches: every final state bit-identical to the oracle's run,
<Z_0> within 1e-12, shots identical to the oracle's conditional-mass tree.
complex64 batches: fidelity >= 1 - 1e-6 against the oracle, shots identical
to the tree of the batch's own final state.  Small tiles force the larger
circuits through the multi-pass (tile, dependency-counter) queue items.
Circuits with mid-circuit measurement and classical control
(backend/mod.rs:51-72, measure.rs:15-51): classical registers identical to
the oracle's run with the same seed, amplitudes within 1e-12 (complex128:
the p1 sums are taken in another order), shots identical to the tree of the
batch's own final state."""
import os

import numpy as np
import pytest

import oracle as O
from everett_gb300 import (Apply1, Circuit, Gate1, IfClassic, Measure, Rng, algorithms, batch,
                           workloads)
from everett_gb300.error import DeviceTimeout, InvalidArgument

pytestmark = pytest.mark.gpu


def tfim_mix(count, nmin, nmax, seed, smin=2, smax=6):
    rng = Rng.seed_from_u64(seed)
    return [workloads.tfim_instance(rng, nmin, nmax, smin, smax) for _ in range(count)]


def oracle_expz(amps):
    b = O.bloch_vector(amps, 0)
    return b[2] / O.norm_sqr(amps)


@pytest.mark.parametrize("tile_bits,chain", [(6, ""), (8, ""), (12, ""), (8, "0"), (6, "pqd"),
                                             (12, "pq")])
def test_batch_c128_bit_exact(gpu, monkeypatch, tile_bits, chain):
    """Batched complex128 runs give the oracle's bits at every tile size and
    with every kind of chain (TFIM steps chain their Rzz records as diagonal
    chains, their Rx records as quad chains); records reach the kernel
    through shared-memory windows, so long circuits span many windows."""
    if chain:
        monkeypatch.setenv("EV_BATCH_CHAIN", chain)
    else:
        monkeypatch.delenv("EV_BATCH_CHAIN", raising=False)
    circs = tfim_mix(24, 2, 13, seed=tile_bits)
    circs.append(workloads.random_layers(11, 4, seed=9))
    circs.append(workloads.qft_on_basis(9, 300))
    circs += [Circuit(3), Circuit(14)]  # no ops: the state stays |0...0>
    res, stats = batch.run_batch(circs, seeds=range(100, 100 + len(circs)), shots=300,
                                 dtype="complex128", tile_bits=tile_bits, threads=256,
                                 return_states=True)
    assert stats["tile_bits"] == tile_bits
    for c, r, seed in zip(circs, res, range(100, 100 + len(circs))):
        want, _, _ = O.run_seeded(c, 0)
        assert np.array_equal(r.amplitudes, want), c.num_qubits()
        assert abs(r.expz - oracle_expz(want)) < 1e-12
        assert np.array_equal(r.shots, O.sample_tree(want, seed, 300))


@pytest.mark.parametrize("threads", [256, 512])
def test_batch_c64_fidelity_and_shots(gpu, threads):
    circs = tfim_mix(40, 3, 16, seed=7, smin=3, smax=8)
    res, stats = batch.run_batch(circs, seeds=range(len(circs)), shots=200, dtype="complex64",
                                 tile_bits=10, threads=threads, return_states=True)
    for i, (c, r) in enumerate(zip(circs, res)):
        want, _, _ = O.run_seeded(c, 0)
        got = r.amplitudes
        fid = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
        assert fid >= 1 - 1e-6
        assert abs(r.expz - oracle_expz(want)) < 1e-5
        assert np.array_equal(r.shots, O.sample_tree(np.ascontiguousarray(got), i, 200))


def test_batch_matches_single_runs(gpu):
    """A circuit gives the same final state alone and inside a batch."""
    circs = tfim_mix(12, 4, 14, seed=3)
    alone = [batch.run_batch([c], shots=50, dtype="complex128", tile_bits=9, threads=256,
                             return_states=True)[0][0] for c in circs]
    mixed, _ = batch.run_batch(circs, shots=50, dtype="complex128", tile_bits=9, threads=256,
                               return_states=True)
    for a, m in zip(alone, mixed):
        assert np.array_equal(a.amplitudes, m.amplitudes)


def classical_mix(seed):
    """Circuits that measure mid-run and gate ops on the outcomes: GHZ with
    a measurement and a controlled X (the serving mix's kind),
    teleportation of a prepared state with both corrections, random layers
    with measurements in between, a nested IfClassic and a conditional
    measurement, and a gate-only circuit beside them."""
    out = [workloads.ghz_midmeasure(n) for n in (3, 7, 10)]
    out.append(algorithms.teleport_state(0.6 + 0.0j, 0.48 + 0.64j))
    for n in (6, 9):
        c = Circuit.with_classical(n, 3)
        c.compose(workloads.random_layers(n, 3, seed + n))
        c.measure(1, 0).measure(n - 1, 1)
        c.x_if(0, 2)
        c.if_classic(1, IfClassic(0, Apply1(Gate1.ry(0.9), 3)))
        c.compose(workloads.random_layers(n, 2, seed + 2 * n))
        c.if_classic(1, Measure(2, 2))
        c.z_if(2, 0)
        out.append(c)
    out.append(workloads.random_layers(8, 3, seed))
    return out


def window_edge_circuits():
    """Circuits whose measurements and IfClassic prefixes fall on the edges
    of the batch kernel's 16-record windows: a prefix as the last record of
    a window with the op it gates in the next one, a measurement as the
    first record of a window, nested prefixes across an edge."""
    out = []
    for pad in (14, 15, 16, 30, 31):
        c = Circuit.with_classical(6, 2)
        c.h(0).cnot(0, 1)
        c.measure(0, 0)
        for j in range(pad):
            c.rz(2 + j % 4, 0.1 * (j + 1))
        c.x_if(0, 3)
        c.if_classic(0, IfClassic(0, Apply1(Gate1.ry(0.7), 4)))
        c.measure(3, 1)
        c.z_if(1, 5)
        out.append(c)
    return out


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_batch_classical_records_across_windows(gpu, dtype):
    """Measurements and IfClassic prefixes give the oracle's classical bits
    and amplitudes wherever they fall relative to the record windows."""
    circs = window_edge_circuits()
    run_seeds = [5 + 3 * i for i in range(len(circs))]
    res, _ = batch.run_batch(circs, seeds=range(len(circs)), shots=50, dtype=dtype,
                             tile_bits=10, threads=256, return_states=True,
                             run_seeds=run_seeds)
    for i, (c, r) in enumerate(zip(circs, res)):
        want, bits, rc = O.run_seeded(c, run_seeds[i])
        assert rc == 0
        assert r.classical == bits, i
        got = r.amplitudes
        if dtype == "complex128":
            assert np.max(np.abs(got - want)) < 1e-12, i
        else:
            fid = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
            assert fid >= 1 - 1e-6, i


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_batch_measurement_and_classical_control(gpu, dtype):
    circs = classical_mix(4)
    run_seeds = [11 + 7 * i for i in range(len(circs))]
    res, _ = batch.run_batch(circs, seeds=range(len(circs)), shots=200, dtype=dtype,
                             tile_bits=10, threads=256, return_states=True,
                             run_seeds=run_seeds)
    for i, (c, r) in enumerate(zip(circs, res)):
        want, bits, rc = O.run_seeded(c, run_seeds[i])
        assert rc == 0
        assert r.classical == bits, i
        got = r.amplitudes
        if dtype == "complex128":
            assert np.max(np.abs(got - want)) < 1e-12, i
        else:
            fid = abs(np.vdot(want, got)) ** 2 / (np.vdot(got, got).real * np.vdot(want, want).real)
            assert fid >= 1 - 1e-6, i
        assert np.array_equal(r.shots, O.sample_tree(np.ascontiguousarray(got), i, 200)), i
    # each circuit's result is the same alone
    for i in (0, 4):
        alone, _ = batch.run_batch([circs[i]], seeds=[i], shots=200, dtype=dtype, tile_bits=10,
                                   threads=256, return_states=True, run_seeds=[run_seeds[i]])
        assert alone[0].classical == res[i].classical
        assert np.array_equal(alone[0].amplitudes, res[i].amplitudes)
        assert np.array_equal(alone[0].shots, res[i].shots)


def test_batch_rejects_oversize_classical_and_autotunes(gpu, tmp_path):
    c = workloads.ghz_midmeasure(9)
    with pytest.raises(InvalidArgument):  # measurement needs the whole state in one CTA
        batch.run_batch([c], tile_bits=8)
    os.environ["EV_AUTOTUNE_CACHE"] = str(tmp_path / "tune.txt")
    try:
        circs = tfim_mix(30, 8, 16, seed=5)
        _, s1 = batch.run_batch(circs, shots=10, autotune=True)
        assert not s1["from_cache"] and s1["tile_bits"] in (12, 13, 14)
        _, s2 = batch.run_batch(circs, shots=10, autotune=True)
        assert s2["from_cache"] and (s2["tile_bits"], s2["threads"]) == (s1["tile_bits"], s1["threads"])
    finally:
        del os.environ["EV_AUTOTUNE_CACHE"]


def test_batch_bounded_wait_reports_timeout(gpu):
    """A queue item whose dependency is never met: the device wait gives up
    after its bound, the call reports EV_ERR_TIMEOUT, and the context stays
    usable for the next batch (no fault, no trap, no hang)."""
    circs = tfim_mix(4, 3, 8, seed=1)
    with pytest.raises(DeviceTimeout):
        batch.run_batch(circs, shots=10, dtype="complex128", tile_bits=6, threads=256,
                        test_stall=True)
    res, _ = batch.run_batch(circs, shots=10, dtype="complex128", tile_bits=6, threads=256,
                             return_states=True)
    for c, r in zip(circs, res):
        want, _, _ = O.run_seeded(c, 0)
        assert np.array_equal(r.amplitudes, want)
