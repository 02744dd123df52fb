"""OpenQASM 3 ingress and egress (no GPU: parsing and emitting are host code).

The oracle (oracle/qasm.py, a restatement of src/qasm/{parse,emit,gates}.rs)
is pinned first against the reference's own assertions (src/qasm/mod.rs
tests, tests/qasm_corpus.rs, properties.rs:458-517, error.rs:145-153),
re-expressed on snippets of this file.  The engine's C++ reader and writer
(ev_qasm_parse / ev_qasm_emit) must then give exactly the oracle's result on
every input: the same circuit (gate matrices bit for bit) or the same error
(message, line and column), over a corpus and seeded mutations of it, and
the same text when emitting.
"""
import math
import random

import numpy as np
import pytest

import oracle.qasm as Q
from everett_gb300 import Circuit, Gate1, Gate2, Rng, algorithms
from everett_gb300.circuit import Apply1, Apply2, Controlled, IfClassic, Measure
from everett_gb300.error import QasmError


def lib_parse(src):
    """The engine's result in the oracle's tuple form, or its error."""
    try:
        c = Circuit.from_qasm(src)
    except QasmError as e:
        return ("error", e.line, e.col, e.message)

    def conv(op):
        if isinstance(op, Apply1):
            return ("apply1", tuple(complex(z) for z in op.gate.m), op.target)
        if isinstance(op, Apply2):
            m = tuple(complex(z) for z in op.gate.m)
            name = {Q.CNOT16: "cx", Q.CZ16: "cz", Q.SWAP16: "swap"}[m]
            return ("apply2", name, op.a, op.b)
        if isinstance(op, Controlled):
            return ("ctrl", tuple(op.controls), tuple(complex(z) for z in op.gate.m), op.target)
        if isinstance(op, Measure):
            return ("measure", op.qubit, op.into)
        return ("if", op.bit, conv(op.then))

    return (c.num_qubits(), c.num_classical(), [conv(o) for o in c.ops()])


def oracle_parse(src):
    try:
        nq, ncl, ops = Q.parse(src)
    except Q.QasmError as e:
        return ("error", e.line, e.col, e.message)
    return (nq, ncl, [_canon(o) for o in ops])


def _canon(op):
    if op[0] == "apply1":
        return ("apply1", tuple(complex(z) for z in op[1]), op[2])
    if op[0] == "ctrl":
        return ("ctrl", tuple(op[1]), tuple(complex(z) for z in op[2]), op[3])
    if op[0] == "if":
        return ("if", op[1], _canon(op[2]))
    return op


def same(a, b):
    """Bit-for-bit equality (a NaN angle would compare unequal to itself)."""
    return repr(a) == repr(b)


BELL = """OPENQASM 3.0;
include "stdgates.inc";
qubit[2] qr;
bit[2] cr;
h qr[0];
cx qr[0], qr[1];
cr[0] = measure qr[0];
measure qr[1] -> cr[1];
"""

CORPUS = [
    BELL,
    "OPENQASM 3;\nqubit[1] q;\nrx(pi/2) q[0];\nry(-pi/4) q[0];\nrz(2*pi) q[0];\np(tau/8) q[0];\n",
    "qubit[3] a;\nctrl @ x a[0], a[1];\nctrl(2) @ rz(0.25) a[0], a[1], a[2];\n",
    "OPENQASM 3.0;\ninclude \"stdgates.inc\";\ngate foo(t) x { rx(t) x; { h x; } }\nqubit[1] q;\nh q[0];\n",
    "qubit[1] q;\nbit[1] c;\nc[0] = measure q[0];\nif (c[0] == 1) x q[0];\n",
    "// leading comment\nqubit[1] q; /* trailing */\n/* two\n lines */\nh q[0];\n",
    "qubit[2] q;\nreset q[0];\nbarrier q[0], q[1];\nswap q[0], q[1];\ncz q[1], q[0];\nCX q[0], q[1];\ncnot q[1], q[0];\n",
    "qubit[2] q;\nid q[0]; s q[1]; t q[0]; y q[1]; z q[0]; phase(-0.5) q[1];\n",
    "qubit[1] q;\nrx(-(1.5e-3 + 2) * 3 / 4 - -1) q[0];\n",
    "qubit[4] q;\nqubit[2] r;\nbit[1] c;\nbit[3] d;\nh q[0];\n;;\n",
    "qubit[1] q;\nrx(1e) q[0];\nry(1.) q[0];\nrz(007) q[0];\np(1E+2) q[0];\n",
    "qubit[2] q;\nctrl(2) @ x q[0], q[1];\n",
    "qubit[2] q;\nh q[0], q[1];\n",
    "qubit[2] q;\ncx(0.1) q[0], q[1];\n",
    "qubit[1] q;\nfoo q[0];\n",
    "qubit[2] q;\nbar q[0], q[1];\n",
    "qubit[1] q;\nbit[1] c;\nif (c[0] == 0) x q[0];\n",
    "qubit[1] q;\nbit[1] c;\nif (c[0] == 1) ;\n",
    "qubit[1] q;\nbit[1] c;\nif (c[0] == 1) if (c[0] == 1) x q[0];\n",
    "qubit[1] q;\nmeasure q[0];\n",
    "qubit[1] q;\nbit[1] c;\nmeasure q[0] c[0];\n",
    "qubit[1] q;\nc[0] = h q[0];\n",
    "qubit[1] q;\nc[0] h q[0];\n",
    "qubit q;\n",
    "qubit[1] 5;\n",
    "qubit[1] q\nh q[0];\n",
    "OPENQASM 3.0\nqubit[1] q;\n",
    "include;\nqubit[1] q;\n",
    "qubit[1] q;\ngate g q { h q;\n",
    "qubit[1] q;\ngate g q ;\nh q[0];\n",
    "qubit[1] q;\nrx(pi/0) q[0];\n",
    "qubit[1] q;\nrx(pi/(1-1)) q[0];\n",
    "qubit[1] q;\nrx(--1) q[0];\n",
    "qubit[1] q;\nrx(1,) q[0];\n",
    "qubit[1] q;\nrx(1 q[0];\n",
    "qubit[1] q;\nh q[x];\n",
    "qubit[1] q;\nh q[0.5];\n",
    "qubit[3] q;\nctrl x q[0], q[1];\n",
    "qubit[3] q;\nctrl(1 @ x q[0], q[1];\n",
    "qubit[3] q;\nctrl @ measure q[0], q[1];\n",
    "qubit[3] q;\nctrl(3) @ x q[0], q[1], q[2];\n",
    "qubit[3] q;\nctrl @ foo q[0], q[1];\n",
    "qubit[1] q;\n} h q[0]; 42; pi;\n",
    "qubit[1] q;\nh q[0]; # x q[0];\n",
    "qubit[1] q;\nh\tq[0];\r\nx q[0];\x0b\x0c\n",
    "qubit[1] q;\nh q[0];  x q[0];\n",
    "qubit[1] q;\n/*/ h q[0]; */ x q[0];\n",
    "qubit[1] q;\n/* unterminated comment h q[0];\n",
    "qubit[1] q;\nh q[0]; // no newline at end",
    "qubit[18446744073709551616] q;\n",
    "qubit[1] q;\nrx(18446744073709551616) q[0];\n",
    "qubit[1] q;\nrx(1e400) q[0];\nry(1e-400) q[0];\n",
    "",
    "   \n\n",
    "OPENQASM 3.0;\n",
]


# ---- the oracle against the reference's own assertions ---------------------------

def test_oracle_pins_reference_assertions():
    nq, ncl, ops = Q.parse(BELL)                       # qasm_corpus.rs bell
    assert (nq, ncl, len(ops)) == (2, 2, 4)
    assert len(Q.parse(CORPUS[1])[2]) == 4             # rotations with pi expressions
    for src in ("qubit[1] q;\nbit[1] c;\nmeasure q[0] -> c[0];\n",
                "qubit[1] q;\nbit[1] c;\nc[0] = measure q[0];\n"):
        assert len(Q.parse(src)[2]) == 1               # both measure forms
    ops = Q.parse(CORPUS[2])[2]                        # ctrl modifier, multi-control
    assert len(ops) == 2 and ops[0][0] == "ctrl" and len(ops[1][1]) == 2
    assert len(Q.parse(CORPUS[3])[2]) == 1             # gate definitions skipped
    assert len(Q.parse(CORPUS[4])[2]) == 2             # classical control if
    assert len(Q.parse(CORPUS[5])[2]) == 1             # line and block comments
    assert len(Q.parse("qubit[1] q;\nh q[0];\n")[2]) == 1  # version optional
    nq, _, ops = Q.parse(BELL)                         # any register names
    assert nq == 2
    src = Q.emit((3, 0, []))                           # emitter header
    assert src.startswith("OPENQASM 3.0;\n")
    assert 'include "stdgates.inc";' in src and "qubit[3] q;" in src
    assert not any(line.startswith("bit[") for line in src.splitlines())
    x = Q.G_FIXED["x"]
    assert "ctrl @ x q[0], q[1];" in Q.emit((2, 0, [("ctrl", (0,), x, 1)]))
    assert "cx q[0], q[1];" in Q.emit((2, 0, [("apply2", Q.CNOT16, 0, 1)]))
    assert str(Q.QasmError(5, 10, "unexpected token")) == \
        "OpenQASM 3 error at 5:10: unexpected token"  # error.rs:145-153
    with pytest.raises(Q.QasmError):                   # nested if cannot be emitted
        Q.emit((1, 1, [("if", 0, ("if", 0, ("apply1", x, 0)))]))


def test_oracle_named_gates_round_trip():
    """mod.rs roundtrip_apply1_named_gates: every named gate is recognised
    and re-parsed to within 1e-12."""
    gates = [Q.G_FIXED["x"], Q.G_FIXED["y"], Q.G_FIXED["z"], Q.g_h(), Q.G_FIXED["s"], Q.g_t(),
             Q.G_FIXED["id"], Q.g_rx(0.7), Q.g_ry(-1.3), Q.g_rz(2.1), Q.g_phase(0.9)]
    for g in gates:
        src = Q.emit((1, 0, [("apply1", g, 0)]))
        (_, _, [op]) = Q.parse(src)
        assert all(abs(a - b) < 1e-12 for a, b in zip(op[1], g)), src


# ---- the engine against the oracle ----------------------------------------------

@pytest.mark.parametrize("i", range(len(CORPUS)))
def test_parse_matches_oracle_corpus(engine, i):
    src = CORPUS[i]
    assert same(lib_parse(src), oracle_parse(src)), src


FRAGMENTS = ["OPENQASM 3.0;", 'include "stdgates.inc";', "qubit[3] q;", "bit[2] c;", "h q[0];",
             "rx(pi/2) q[1];", "cx q[0], q[1];", "ctrl @ x q[0], q[1];",
             "ctrl(2) @ ry(0.3) q[0], q[1], q[2];", "c[0] = measure q[0];",
             "measure q[1] -> c[1];", "if (c[0] == 1) x q[2];", "gate g a { h a; }",
             "reset q[0];", "barrier q;", "// c\n", "/* b */", "p(-tau/4) q[0];",
             "swap q[1], q[2];", "rz(1.5e-2*3) q[2];", "y q[1];", "\n", " "]
NOISE = list("[](){};,=-><@*/+ \n\t0123456789.eqxhcr_\"") + ["pi", "==", "->", "ctrl", "if",
                                                             "measure", "qubit", "bit", "gate"]


def test_parse_matches_oracle_fuzz(engine):
    rng = random.Random(20241203)
    for case in range(3000):
        parts = [rng.choice(FRAGMENTS) for _ in range(rng.randint(1, 12))]
        src = "".join(p + (" " if rng.random() < 0.5 else "\n") for p in parts)
        for _ in range(rng.randint(0, 3)):  # mutations: insert, delete, replace
            pos = rng.randint(0, len(src))
            op = rng.random()
            if op < 0.4:
                src = src[:pos] + rng.choice(NOISE) + src[pos:]
            elif op < 0.7:
                src = src[:pos] + src[pos + rng.randint(1, 4):]
            else:
                src = src[:pos] + rng.choice(NOISE) + src[pos + 1:]
        assert same(lib_parse(src), oracle_parse(src)), (case, src)


def named_circuit(rng: Rng):
    """properties.rs:458-499 arb_named_circuit, drawn from the reference's Rng:
    2..5 qubits, 1..11 named 1-qubit ops, then CNOT, CZ and a controlled X."""
    n = 2 + int(rng.next_f64() * 4)
    c = Circuit(n)
    for _ in range(1 + int(rng.next_f64() * 11)):
        q = int(rng.next_f64() * n)
        which = int(rng.next_f64() * 11)
        angle = (rng.next_f64() * 2.0 - 1.0) * 2.0 * math.pi
        [lambda: c.h(q), lambda: c.x(q), lambda: c.y(q), lambda: c.z(q), lambda: c.s(q),
         lambda: c.t(q), lambda: c.rx(q, angle), lambda: c.ry(q, angle), lambda: c.rz(q, angle),
         lambda: c.phase(q, angle), lambda: c.gate1(Gate1.id(), q)][which]()
    c.cnot(0, 1).cz(0, 1)
    c.controlled([0], Gate1.x(), 1)
    return c


def to_oracle(c: Circuit):
    def conv(op):
        if isinstance(op, Apply1):
            return ("apply1", tuple(complex(z) for z in op.gate.m), op.target)
        if isinstance(op, Apply2):
            return ("apply2", tuple(complex(z) for z in op.gate.m), op.a, op.b)
        if isinstance(op, Controlled):
            return ("ctrl", tuple(op.controls), tuple(complex(z) for z in op.gate.m), op.target)
        if isinstance(op, Measure):
            return ("measure", op.qubit, op.into)
        return ("if", op.bit, conv(op.then))
    return (c.num_qubits(), c.num_classical(), [conv(o) for o in c.ops()])


def test_emit_matches_oracle_and_round_trips(engine):
    rng = Rng.seed_from_u64(517)
    for case in range(256):
        c = named_circuit(rng)
        if case % 3 == 0:
            c2 = Circuit.with_classical(c.num_qubits(), 2)
            c2.compose(c)
            c2.measure(0, 1).x_if(1, 1).controlled([0, 1], Gate1.rz(0.3), 1 + (c.num_qubits() > 2))
            c = c2
        text = c.to_qasm()
        assert text == Q.emit(to_oracle(c)), case
        back = Circuit.from_qasm(text)
        assert back.num_qubits() == c.num_qubits() and len(back) == len(c)
        for a, b in zip(c.ops(), back.ops()):
            ga = getattr(getattr(a, "then", a), "gate", None)
            gb = getattr(getattr(b, "then", b), "gate", None)
            if ga is not None:
                assert np.max(np.abs(ga.m - gb.m)) < 1e-12, (case, text)


def test_emit_errors_match_reference(engine):
    c = Circuit(2)
    c.gate1(Gate1(0.6, 0.8, 0.8, -0.6), 0)               # no stdgates name
    with pytest.raises(QasmError) as e:
        c.to_qasm()
    assert (e.value.line, e.value.col) == (0, 0) and "no OpenQASM 3 name" in e.value.message
    c = Circuit(2)
    c.gate2(Gate2.controlled(Gate1.h()), 0, 1)           # 2-qubit matrix without a name
    with pytest.raises(QasmError):
        c.to_qasm()
    c = Circuit.with_classical(1, 1)
    c.if_classic(0, IfClassic(0, Apply1(Gate1.x(), 0)))  # nested IfClassic
    with pytest.raises(QasmError) as e:
        c.to_qasm()
    assert "nested IfClassic" in e.value.message


def test_algorithm_circuits_emit_and_parse(engine):
    """mod.rs roundtrip_bell / ghz / qft: the generators' circuits emit and
    parse back to the same op count."""
    for c in (algorithms.bell(), algorithms.ghz(4), algorithms.qft(4)):
        back = Circuit.from_qasm(c.to_qasm())
        assert len(back) == len(c) and back.num_qubits() == c.num_qubits()
