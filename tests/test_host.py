"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared entry point, the op encoding matches the header's layout,
circuit validation (pure host code in the engine) mirrors the reference's
errors, and the workload generators build the configured circuits."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from everett_gb300 import (Circuit, ClassicalBitOutOfRange, DuplicateQubit, Gate1, Gate2,
                           QubitOutOfRange, _native, algorithms, workloads)
from everett_gb300.error import InvalidArgument

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(ev_[a-z0-9_]+)\s*\(",
                            text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(engine):
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(engine, name), name
    # every entry point has a ctypes signature (an unsigned 64-bit size passed
    # without one is silently truncated to a C int)
    assert set(names) == set(_native.exported_symbols())


def test_version_and_device_count(engine):
    assert b"sm_103a" in engine.ev_version()
    assert _native.device_count() >= 0


def test_op_record_layout():
    assert _native.OP_DTYPE.itemsize == 288
    assert [_native.OP_DTYPE.fields[f][1] for f in ("kind", "nctrl", "ctrl_off", "q0", "q1", "m")] \
        == [0, 4, 8, 16, 24, 32]
    assert C.sizeof(_native.EvCircuit) == 48 and C.sizeof(_native.EvRunOptions) == 16


def test_encoding_prefix_ifclassic():
    c = Circuit.with_classical(3, 2)
    c.h(0).controlled([1, 2], Gate1.x(), 0).measure(0, 1).x_if(1, 2)
    ops, pool, npool = c.to_ev()
    assert list(ops["kind"]) == [1, 3, 4, 5, 1]
    assert npool == 2 and list(pool[:2]) == [1, 2]
    assert ops[1]["ctrl_off"] == 0 and ops[1]["nctrl"] == 2
    assert ops[3]["q0"] == 1 and ops[4]["q0"] == 2


def test_validation_mirrors_reference(engine):  # circuit.rs:333-382
    c = Circuit(2)
    c.h(0).cnot(0, 1)
    c.validate()
    c = Circuit(2)
    c.h(5)
    with pytest.raises(QubitOutOfRange, match="q5 out of range for 2-qubit register"):
        c.validate()
    c = Circuit(2)
    c.cnot(1, 1)
    with pytest.raises(DuplicateQubit, match="q1 used more than once"):
        c.validate()
    c = Circuit(1)
    c.measure(0, 0)
    with pytest.raises(ClassicalBitOutOfRange, match="c0 out of range for 0-bit register"):
        c.validate()
    c = Circuit.with_classical(1, 1)
    c.x_if(0, 3)
    with pytest.raises(QubitOutOfRange):
        c.validate()
    # first error in op order wins; within Controlled the target is checked first
    c = Circuit(3)
    c.controlled([7, 2], Gate1.x(), 2)
    with pytest.raises(QubitOutOfRange, match="q7"):
        c.validate()
    # an IF record with no body is malformed
    ops = np.zeros(1, dtype=_native.OP_DTYPE)
    ops[0]["kind"] = _native.OP_IF
    st = _native.EvCircuit(1, 1, ops.ctypes.data, 1, None, 0)
    with pytest.raises(InvalidArgument):
        _native.check(engine.ev_validate(C.byref(st)))


def test_validation_agrees_with_oracle(engine):
    import oracle as O
    rng = np.random.default_rng(5)
    for _ in range(200):
        n, ncl = int(rng.integers(1, 5)), int(rng.integers(0, 3))
        c = Circuit.with_classical(n, ncl)
        for _ in range(4):
            kind = rng.integers(0, 5)
            q = [int(v) for v in rng.integers(0, n + 1, size=3)]
            if kind == 0:
                c.h(q[0])
            elif kind == 1:
                c.cnot(q[0], q[1])
            elif kind == 2:
                c.controlled([q[1], q[2]], Gate1.z(), q[0])
            elif kind == 3:
                c.measure(q[0], q[1] % 3)
            else:
                c.x_if(q[1] % 3, q[0])
        st = c.ev_struct()
        assert engine.ev_validate(C.byref(st)) == O.validate(c)


def test_workload_shapes():
    c = workloads.random_layers(20, 20, seed=1)
    assert len(c) == 20 * 20 * 3 + 10 * 10 + 10 * 9  # 1390
    c = workloads.random_layers(30, 20, seed=1)
    assert len(c) == 1800 + 290
    q = algorithms.qft(30)
    assert len(q) == 30 + 435 + 15
    h = workloads.haar_layers(28, 40, seed=3)
    assert len(h) == 1120 + 540
    for op in h.ops()[:28]:
        u = op.gate.m.reshape(2, 2)
        assert np.allclose(u.conj().T @ u, np.eye(2), atol=1e-12)
    g = workloads.ghz_midmeasure(5)
    assert g.num_classical() == 1 and len(g) == 1 + 4 + 1 + 1


def test_qft_closed_form_matches_oracle():
    import oracle as O
    for n, j in ((3, 1), (6, 45), (10, 777)):
        amps, _, _ = O.run_seeded(workloads.qft_on_basis(n, j))
        assert np.max(np.abs(amps - workloads.qft_closed_form(n, j))) < 1e-12


def test_gate_bytes_counts():
    c = Circuit(10)
    c.h(0).phase(1, 0.3).cnot(0, 1).cz(2, 3).controlled([0], Gate1.phase(0.2), 4)
    dim = 1024
    assert workloads.gate_bytes(c) == 2 * 16 * (dim + dim // 2 + dim // 2 + dim // 4 + dim // 4)
