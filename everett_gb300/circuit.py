"""The circuit builder and instruction set, mirroring everett's Circuit
(src/circuit.rs:26-306) and Op (src/op.rs:14-58).

Builder methods record ops without validating and return ``self`` so they
chain; ``validate()`` (run automatically by the backend) reports the first
bad index in op order.  ``to_ev()`` encodes the ops into the C ABI's record
array (IfClassic in prefix form).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Union

import numpy as np

from . import _native as N
from .gate import Gate1, Gate2


@dataclass(frozen=True)
class Apply1:
    gate: Gate1
    target: int


@dataclass(frozen=True)
class Apply2:
    gate: Gate2
    a: int
    b: int


@dataclass(frozen=True)
class Controlled:
    controls: tuple
    gate: Gate1
    target: int


@dataclass(frozen=True)
class Measure:
    qubit: int
    into: int


@dataclass(frozen=True)
class IfClassic:
    bit: int
    then: "Op"


Op = Union[Apply1, Apply2, Controlled, Measure, IfClassic]


def _gate1(m) -> Gate1:
    return Gate1(complex(m[0], m[1]), complex(m[2], m[3]), complex(m[4], m[5]), complex(m[6], m[7]))


class Circuit:
    def __init__(self, num_qubits: int, num_classical: int = 0):
        self._n = int(num_qubits)
        self._nc = int(num_classical)
        self._ops: list = []
        self._enc = None

    @classmethod
    def new(cls, num_qubits: int) -> "Circuit":
        return cls(num_qubits)

    @classmethod
    def with_classical(cls, num_qubits: int, num_classical: int) -> "Circuit":
        return cls(num_qubits, num_classical)

    def num_qubits(self) -> int:
        return self._n

    def num_classical(self) -> int:
        return self._nc

    def ops(self) -> list:
        return self._ops

    def __len__(self) -> int:
        return len(self._ops)

    def is_empty(self) -> bool:
        return not self._ops

    def _push(self, op) -> "Circuit":
        self._ops.append(op)
        self._enc = None
        return self

    # generic builders (circuit.rs:91-127)
    def gate1(self, gate: Gate1, target: int) -> "Circuit":
        return self._push(Apply1(gate, int(target)))

    def gate2(self, gate: Gate2, a: int, b: int) -> "Circuit":
        return self._push(Apply2(gate, int(a), int(b)))

    def controlled(self, controls, gate: Gate1, target: int) -> "Circuit":
        return self._push(Controlled(tuple(int(c) for c in controls), gate, int(target)))

    def compose(self, sub: "Circuit") -> "Circuit":
        self._ops.extend(sub._ops)
        self._enc = None
        return self

    # named gates (circuit.rs:131-185)
    def h(self, q):
        return self.gate1(Gate1.h(), q)

    def x(self, q):
        return self.gate1(Gate1.x(), q)

    def y(self, q):
        return self.gate1(Gate1.y(), q)

    def z(self, q):
        return self.gate1(Gate1.z(), q)

    def s(self, q):
        return self.gate1(Gate1.s(), q)

    def t(self, q):
        return self.gate1(Gate1.t(), q)

    def rx(self, q, theta):
        return self.gate1(Gate1.rx(theta), q)

    def ry(self, q, theta):
        return self.gate1(Gate1.ry(theta), q)

    def rz(self, q, theta):
        return self.gate1(Gate1.rz(theta), q)

    def phase(self, q, lam):
        return self.gate1(Gate1.phase(lam), q)

    def cnot(self, control, target):
        return self.gate2(Gate2.cnot(), control, target)

    def cz(self, a, b):
        return self.gate2(Gate2.cz(), a, b)

    def swap(self, a, b):
        return self.gate2(Gate2.swap(), a, b)

    # measurement and classical control (circuit.rs:190-228)
    def measure(self, qubit, into):
        return self._push(Measure(int(qubit), int(into)))

    def x_if(self, bit, q):
        return self.if_classic(bit, Apply1(Gate1.x(), int(q)))

    def z_if(self, bit, q):
        return self.if_classic(bit, Apply1(Gate1.z(), int(q)))

    def if_classic(self, bit, op) -> "Circuit":
        return self._push(IfClassic(int(bit), op))

    # encoding for the C ABI
    def to_ev(self):
        """(ops record array, control pool) for include/everett_cuda.h."""
        if self._enc is not None:
            return self._enc
        recs = []
        pool: list[int] = []

        def emit(op):
            r = np.zeros((), dtype=N.OP_DTYPE)
            if isinstance(op, Apply1):
                r["kind"] = N.OP_APPLY1
                r["q0"] = op.target
                r["m"][:8] = op.gate.as_f64()
            elif isinstance(op, Apply2):
                r["kind"] = N.OP_APPLY2
                r["q0"], r["q1"] = op.a, op.b
                r["m"][:] = op.gate.as_f64()
            elif isinstance(op, Controlled):
                r["kind"] = N.OP_CONTROLLED
                r["q0"] = op.target
                r["nctrl"] = len(op.controls)
                r["ctrl_off"] = len(pool)
                pool.extend(op.controls)
                r["m"][:8] = op.gate.as_f64()
            elif isinstance(op, Measure):
                r["kind"] = N.OP_MEASURE
                r["q0"], r["q1"] = op.qubit, op.into
            elif isinstance(op, IfClassic):
                r["kind"] = N.OP_IF
                r["q0"] = op.bit
                recs.append(r)
                emit(op.then)
                return
            else:
                raise TypeError(f"not an op: {op!r}")
            recs.append(r)

        for op in self._ops:
            emit(op)
        ops = np.array(recs, dtype=N.OP_DTYPE) if recs else np.zeros(0, dtype=N.OP_DTYPE)
        ctrl = np.array(pool, dtype=np.uint64) if pool else np.zeros(1, dtype=np.uint64)
        self._enc = (ops, ctrl, len(pool))
        return self._enc

    def ev_struct(self) -> N.EvCircuit:
        ops, ctrl, npool = self.to_ev()
        c = N.EvCircuit()
        c.num_qubits = self._n
        c.num_classical = self._nc
        c.ops = ops.ctypes.data if len(ops) else None
        c.nops = len(ops)
        c.ctrl_pool = ctrl.ctypes.data
        c.pool_len = npool
        return c

    # OpenQASM 3 (src/circuit.rs:308-326)
    @classmethod
    def from_qasm(cls, src: str) -> "Circuit":
        """Circuit::from_qasm: the engine's reader (ev_qasm_parse), the same
        subset, circuit and errors as src/qasm/parse.rs; raises QasmError."""
        import ctypes as C
        data = src.encode("utf-8")
        h = C.c_void_p()
        N.check(N.lib().ev_qasm_parse(data, len(data), C.byref(h), None, None))
        try:
            view = N.EvCircuit()
            N.check(N.lib().ev_program_circuit(h, C.byref(view)))
            recs = np.zeros(0, dtype=N.OP_DTYPE)
            pool = np.zeros(0, dtype=np.uint64)
            if view.nops:
                raw = (C.c_char * (view.nops * N.OP_DTYPE.itemsize)).from_address(view.ops)
                recs = np.frombuffer(raw, dtype=N.OP_DTYPE).copy()
            if view.pool_len:
                raw = (C.c_char * (view.pool_len * 8)).from_address(view.ctrl_pool)
                pool = np.frombuffer(raw, dtype=np.uint64).copy()
            c = cls(view.num_qubits, view.num_classical)
        finally:
            N.lib().ev_program_free(h)
        pos = 0

        def take():
            nonlocal pos
            r = recs[pos]
            pos += 1
            kind = int(r["kind"])
            m = r["m"]
            if kind == N.OP_APPLY1:
                return Apply1(_gate1(m), int(r["q0"]))
            if kind == N.OP_APPLY2:
                return Apply2(Gate2(m[0::2] + 1j * m[1::2]), int(r["q0"]), int(r["q1"]))
            if kind == N.OP_CONTROLLED:
                off, k = int(r["ctrl_off"]), int(r["nctrl"])
                return Controlled(tuple(int(q) for q in pool[off:off + k]), _gate1(m), int(r["q0"]))
            if kind == N.OP_MEASURE:
                return Measure(int(r["q0"]), int(r["q1"]))
            return IfClassic(int(r["q0"]), take())

        while pos < len(recs):
            c._push(take())
        return c

    def to_qasm(self) -> str:
        """Circuit::to_qasm: the engine's writer (ev_qasm_emit, emit.rs:17);
        raises QasmError for a gate without a stdgates.inc name."""
        import ctypes as C
        c = self.ev_struct()
        n = C.c_uint64()
        N.check(N.lib().ev_qasm_emit(C.byref(c), None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        N.check(N.lib().ev_qasm_emit(C.byref(c), buf, n.value + 1, C.byref(n)))
        return buf.raw[:n.value].decode("utf-8")

    def validate(self) -> None:
        """Circuit::validate (circuit.rs:245-306), via the engine's check."""
        c = self.ev_struct()
        N.check(N.lib().ev_validate(c))
