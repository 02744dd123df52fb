"""OpenQASM 3 oracle: a plain-Python restatement of the reference's reader
and writer (hz2/everett src/qasm/parse.rs, emit.rs, gates.rs).

Test infrastructure only: the parity tests compare the engine's C++ parser
and emitter (``ev_qasm_parse`` / ``ev_qasm_emit``) against this module on the
same sources.  Every step follows the cited reference lines, including where
an error is reported (the position of the token after the one that failed,
as the reference's ``Parser::err`` peeks it).

Where the reference panics instead of returning an error (a multi-byte
character that is not whitespace, an unterminated string literal), this
restatement and the engine both treat the rest of that character / the rest
of the input as consumed; no parity case exercises those inputs.

Circuits are tuples: ``(num_qubits, num_classical, ops)`` with ops
  ("apply1", m4, target)            m4 = 4 complex entries, row-major
  ("apply2", name, a, b)            name in {"cx", "cz", "swap"}
  ("ctrl", controls, m4, target)
  ("measure", qubit, bit)
  ("if", bit, op)
"""
from __future__ import annotations

import math

PI = 3.141592653589793          # std::f64::consts::PI
TAU = 6.283185307179586         # std::f64::consts::TAU
FRAC_PI_4 = 0.7853981633974483  # std::f64::consts::FRAC_PI_4
FRAC_1_SQRT_2 = 0.7071067811865476


class QasmError(Exception):
    """Error::Qasm { line, col, message } (src/error.rs:45-52)."""

    def __init__(self, line: int, col: int, message: str):
        super().__init__(f"OpenQASM 3 error at {line}:{col}: {message}")
        self.line, self.col, self.message = line, col, message


# ---- gates (src/gate.rs:53-136, src/qasm/gates.rs) ---------------------------

def _sin(x):  # libm's sin / cos give NaN for an infinite argument
    return math.sin(x) if math.isfinite(x) else math.nan


def _cos(x):
    return math.cos(x) if math.isfinite(x) else math.nan


def _expi(t):
    return complex(_cos(t), _sin(t))


def g_h():
    s = FRAC_1_SQRT_2
    return (complex(s, 0.0), complex(s, 0.0), complex(s, 0.0), complex(-s, 0.0))


G_FIXED = {
    "id": (1 + 0j, 0j, 0j, 1 + 0j),
    "x": (0j, 1 + 0j, 1 + 0j, 0j),
    "y": (0j, complex(0.0, -1.0), complex(0.0, 1.0), 0j),
    "z": (1 + 0j, 0j, 0j, complex(-1.0, 0.0)),
    "s": (1 + 0j, 0j, 0j, 1j),
}


def g_t():
    return (1 + 0j, 0j, 0j, _expi(FRAC_PI_4))


def g_rx(t):
    h = t / 2.0
    s, c = _sin(h), _cos(h)
    return (complex(c, 0.0), complex(0.0, -s), complex(0.0, -s), complex(c, 0.0))


def g_ry(t):
    h = t / 2.0
    s, c = _sin(h), _cos(h)
    return (complex(c, 0.0), complex(-s, 0.0), complex(s, 0.0), complex(c, 0.0))


def g_rz(t):
    return (_expi(-t / 2.0), 0j, 0j, _expi(t / 2.0))


def g_phase(lam):
    return (1 + 0j, 0j, 0j, _expi(lam))


def lookup_1q(name, args):
    """gates.rs:113-133 (name, arity) -> matrix."""
    n = len(args)
    if n == 0:
        if name == "h":
            return g_h()
        if name == "t":
            return g_t()
        if name in G_FIXED:
            return G_FIXED[name]
    if n == 1:
        if name == "rx":
            return g_rx(args[0])
        if name == "ry":
            return g_ry(args[0])
        if name == "rz":
            return g_rz(args[0])
        if name in ("p", "phase"):
            return g_phase(args[0])
    raise QasmError(0, 0, f"unknown single-qubit gate '{name}'")


def lookup_2q(name):
    """gates.rs:136-148."""
    if name in ("cx", "cnot", "CX"):
        return "cx"
    if name in ("cz", "swap"):
        return name
    raise QasmError(0, 0, f"unknown two-qubit gate '{name}'")


# ---- lexer (parse.rs:9-224) ------------------------------------------------------

_WS = {0x09, 0x0A, 0x0B, 0x0C, 0x0D, 0x20, 0x85, 0xA0, 0x1680, 0x2028, 0x2029, 0x202F, 0x205F,
       0x3000} | set(range(0x2000, 0x200B))
KEYWORDS = {"OPENQASM": "KwOpenQasm", "include": "KwInclude", "qubit": "KwQubit", "bit": "KwBit",
            "measure": "KwMeasure", "if": "KwIf", "gate": "KwGate", "ctrl": "KwCtrl", "pi": "KwPi",
            "tau": "KwTau"}
SINGLE = {";": "Semi", "(": "LParen", ")": "RParen", "[": "LBrack", "]": "RBrack", "{": "LBrace",
          "}": "RBrace", ",": "Comma", "=": "Eq", "/": "Slash", "*": "Star", "+": "Plus",
          "-": "Minus", "@": "At"}


class Lexer:
    def __init__(self, src: str):
        self.s, self.pos, self.line, self.col = src, 0, 1, 1

    def advance(self, n):  # n characters
        for ch in self.s[self.pos:self.pos + n]:
            if ch == "\n":
                self.line += 1
                self.col = 1
            else:
                self.col += 1
        self.pos += n

    def skip(self):
        while True:
            k = 0
            while self.pos + k < len(self.s) and ord(self.s[self.pos + k]) in _WS:
                k += 1
            if k:
                self.advance(k)
                continue
            rem = self.s[self.pos:]
            if rem.startswith("//"):
                i = rem.find("\n")
                self.advance(len(rem) if i < 0 else i + 1)
                continue
            if rem.startswith("/*"):
                i = rem.find("*/")
                self.advance(len(rem) if i < 0 else i + 2)
                continue
            return

    @staticmethod
    def scan_number(rem):
        i = 0
        while i < len(rem) and rem[i].isdigit() and rem[i].isascii():
            i += 1
        if i < len(rem) and rem[i] == ".":
            i += 1
            while i < len(rem) and rem[i].isascii() and rem[i].isdigit():
                i += 1
        if i < len(rem) and rem[i] in "eE":
            i += 1
            if i < len(rem) and rem[i] in "+-":
                i += 1
            while i < len(rem) and rem[i].isascii() and rem[i].isdigit():
                i += 1
        return rem[:i]

    def next(self):
        """(kind, value, line, col)."""
        self.skip()
        line, col = self.line, self.col
        rem = self.s[self.pos:]
        if not rem:
            return ("Eof", None, line, col)
        ch = rem[0]
        if ch == '"':
            end = rem.find('"', 1)
            if end < 0:  # the reference panics here; consume the rest
                self.advance(len(rem))
                return ("Str", rem[1:], line, col)
            self.advance(end + 1)
            return ("Str", rem[1:end], line, col)
        if rem.startswith("=="):
            self.advance(2)
            return ("EqEq", None, line, col)
        if rem.startswith("->"):
            self.advance(2)
            return ("Arrow", None, line, col)
        if ch in SINGLE:
            self.advance(1)
            return (SINGLE[ch], None, line, col)
        if ch.isascii() and ch.isdigit():
            s = self.scan_number(rem)
            self.advance(len(s))
            if "." in s or "e" in s or "E" in s:
                return ("Float", _parse_f64(s), line, col)
            v = int(s)
            if v < (1 << 64):
                return ("Int", v, line, col)
            return ("Float", _parse_f64(s), line, col)
        if ch.isascii() and (ch.isalpha() or ch == "_"):
            i = 1
            while i < len(rem) and rem[i].isascii() and (rem[i].isalnum() or rem[i] == "_"):
                i += 1
            word = rem[:i]
            self.advance(i)
            if word in KEYWORDS:
                return (KEYWORDS[word], None, line, col)
            return ("Ident", word, line, col)
        self.advance(1)
        return ("Ident", "?", line, col)


def _parse_f64(s):
    """Rust's str::parse::<f64>, or 0.0 when it fails (parse.rs:166-170)."""
    import re
    if re.fullmatch(r"[0-9]+(\.[0-9]*)?([eE][+-]?[0-9]+)?", s) is None:
        return 0.0
    return float(s)


# ---- parser (parse.rs:229-816) ---------------------------------------------------

class Parser:
    def __init__(self, src):
        self.lex = Lexer(src)
        self.peeked = None

    def peek(self):
        if self.peeked is None:
            self.peeked = self.lex.next()
        return self.peeked

    def consume(self):
        if self.peeked is not None:
            t, self.peeked = self.peeked, None
            return t
        return self.lex.next()

    def err(self, msg):
        _, _, line, col = self.peek()
        return QasmError(line, col, msg)

    def expect_semi(self):
        if self.peek()[0] == "Semi":
            self.consume()
        else:
            raise self.err("expected ';'")

    def expect(self, kind, msg):
        if self.peek()[0] == kind:
            self.consume()
        else:
            raise self.err(msg)

    def parse_int(self):
        t = self.consume()
        if t[0] != "Int":
            raise self.err("expected integer")
        return t[1]

    def index(self):
        self.expect("LBrack", "expected '['")
        i = self.parse_int()
        self.expect("RBrack", "expected ']'")
        return i

    def reg_index(self, what):
        if self.peek()[0] != "Ident":
            raise self.err(f"expected {what} register name")
        self.consume()
        return self.index()

    def skip_block(self):
        if self.consume()[0] != "LBrace":
            raise self.err("expected '{' for gate body")
        depth = 1
        while True:
            k = self.consume()[0]
            if k == "LBrace":
                depth += 1
            elif k == "RBrace":
                depth -= 1
                if depth == 0:
                    return
            elif k == "Eof":
                raise self.err("unexpected EOF in gate body")

    def program(self):
        nq = ncl = 0
        ops = []
        if self.peek()[0] == "KwOpenQasm":
            self.consume()
            if self.peek()[0] in ("Int", "Float"):
                self.consume()
            self.expect_semi()
        if self.peek()[0] == "KwInclude":
            self.consume()
            self.consume()
            self.expect_semi()
        while True:
            k = self.peek()[0]
            if k == "Eof":
                break
            if k in ("KwQubit", "KwBit"):
                self.consume()
                self.expect("LBrack", "expected '['")
                n = self.parse_int()
                self.expect("RBrack", "expected ']'")
                if self.consume()[0] != "Ident":
                    raise self.err("expected qubit register name" if k == "KwQubit"
                                   else "expected classical register name")
                self.expect_semi()
                if k == "KwQubit":
                    nq = n
                else:
                    ncl = n
            elif k == "KwGate":
                self.consume()
                while self.peek()[0] not in ("LBrace", "Eof"):
                    self.consume()
                self.skip_block()
            else:
                op = self.statement()
                if op is not None:
                    ops.append(op)
        return (nq, ncl, ops)

    def statement(self):
        k, v, _, _ = self.peek()
        if k == "Semi":
            self.consume()
            return None
        if k == "KwMeasure":
            self.consume()
            q = self.reg_index("qubit")
            k2 = self.peek()[0]
            if k2 == "Arrow":
                self.consume()
                b = self.reg_index("classical")
                self.expect_semi()
                return ("measure", q, b)
            if k2 == "Semi":
                self.consume()
                raise QasmError(0, 0, "bare 'measure' without destination is not supported")
            raise self.err("expected '->' or ';' after measure operand")
        if k == "KwIf":
            return self.parse_if()
        if k == "KwCtrl":
            return self.ctrl_call()
        if k == "Ident":
            name = v
            if name in ("reset", "barrier"):
                while self.consume()[0] not in ("Semi", "Eof"):
                    pass
                return None
            self.consume()
            k2 = self.peek()[0]
            if k2 == "LBrack":
                self.consume()
                idx = self.parse_int()
                self.expect("RBrack", "expected ']'")
                if self.peek()[0] != "Eq":
                    raise self.err("unexpected token after register index")
                self.consume()
                if self.peek()[0] != "KwMeasure":
                    raise self.err("expected 'measure' after '='")
                self.consume()
                q = self.reg_index("qubit")
                self.expect_semi()
                return ("measure", q, idx)
            if k2 in ("LParen", "Ident", "Semi", "Comma"):
                return self.call_after_name(name)
            raise self.err("unexpected token in statement")
        self.consume()
        return None

    def parse_if(self):
        self.consume()
        if self.consume()[0] != "LParen":
            raise self.err("expected '(' after 'if'")
        if self.consume()[0] != "Ident":
            raise self.err("expected classical register in if condition")
        self.expect("LBrack", "expected '['")
        bit = self.parse_int()
        self.expect("RBrack", "expected ']'")
        if self.consume()[0] != "EqEq":
            raise self.err("expected '==' in if condition")
        t = self.consume()
        if not (t[0] == "Int" and t[1] == 1):
            raise QasmError(0, 0, "only 'if (c[i] == 1)' is supported")
        if self.consume()[0] != "RParen":
            raise self.err("expected ')' to close if condition")
        inner = self.statement()
        if inner is None:
            raise self.err("expected statement in if body")
        return ("if", bit, inner)

    def _gate_err(self, e):
        _, _, line, col = self.peek()
        return QasmError(line, col, e.message)

    def ctrl_call(self):
        self.consume()
        n = 1
        if self.peek()[0] == "LParen":
            self.consume()
            n = self.parse_int()
            if self.consume()[0] != "RParen":
                raise self.err("expected ')'")
        if self.consume()[0] != "At":
            raise self.err("expected '@' after ctrl")
        t = self.consume()
        if t[0] != "Ident":
            raise self.err("expected gate name after 'ctrl @'")
        args = self.arg_list()
        opnds = self.operand_list()
        self.expect_semi()
        if len(opnds) < n + 1:
            raise self.err("not enough operands for ctrl gate")
        try:
            m = lookup_1q(t[1], args)
        except QasmError as e:
            raise self._gate_err(e)
        return ("ctrl", tuple(opnds[:n]), m, opnds[n])

    def call_after_name(self, name):
        args = self.arg_list()
        opnds = self.operand_list()
        self.expect_semi()
        if len(opnds) == 1:
            try:
                return ("apply1", lookup_1q(name, args), opnds[0])
            except QasmError as e:
                raise self._gate_err(e)
        if len(opnds) == 2 and not args:
            try:
                return ("apply2", lookup_2q(name), opnds[0], opnds[1])
            except QasmError as e:
                raise self._gate_err(e)
        raise self.err("unexpected gate arity")

    def arg_list(self):
        if self.peek()[0] != "LParen":
            return []
        self.consume()
        args = []
        while True:
            k = self.peek()[0]
            if k == "RParen":
                self.consume()
                return args
            if k == "Comma":
                self.consume()
            else:
                args.append(self.expr())

    def operand_list(self):
        out = []
        while True:
            k = self.peek()[0]
            if k == "Ident":
                self.consume()
                out.append(self.index())
            elif k == "Comma":
                self.consume()
            else:
                return out

    def expr(self):
        lhs = self.mul()
        while True:
            k = self.peek()[0]
            if k == "Plus":
                self.consume()
                lhs = lhs + self.mul()
            elif k == "Minus":
                self.consume()
                lhs = lhs - self.mul()
            else:
                return lhs

    def mul(self):
        lhs = self.unary()
        while True:
            k = self.peek()[0]
            if k == "Star":
                self.consume()
                lhs = lhs * self.unary()
            elif k == "Slash":
                self.consume()
                rhs = self.unary()
                if rhs == 0.0:
                    raise self.err("division by zero in angle expression")
                lhs = lhs / rhs
            else:
                return lhs

    def unary(self):
        k = self.peek()[0]
        if k == "Minus":
            self.consume()
            return -self.primary()
        if k == "Plus":
            self.consume()
        return self.primary()

    def primary(self):
        k, v, _, _ = self.consume()
        if k == "Float":
            return v
        if k == "Int":
            return float(v)
        if k == "KwPi":
            return PI
        if k == "KwTau":
            return TAU
        if k == "LParen":
            val = self.expr()
            if self.consume()[0] != "RParen":
                raise self.err("expected ')'")
            return val
        raise self.err("expected numeric expression")


def parse(src: str):
    """parse.rs:813-816."""
    return Parser(src).program()


# ---- emitter (emit.rs:17-81, gates.rs:28-111) ------------------------------------

def _close(a, b):
    return all(abs(x - y) < 1e-12 for x, y in zip(a, b))


def gate_info_1q(m):
    m = tuple(complex(z) for z in m)
    if m == G_FIXED["x"]:
        return "x", ""
    if m == G_FIXED["y"]:
        return "y", ""
    if m == G_FIXED["z"]:
        return "z", ""
    if m == g_h():
        return "h", ""
    if m == G_FIXED["s"]:
        return "s", ""
    if m == g_t():
        return "t", ""
    if m == G_FIXED["id"]:
        return "id", ""
    if (m[0].imag == 0.0 and m[1].real == 0.0 and m[2].real == 0.0 and m[3].imag == 0.0
            and abs(m[0].real - m[3].real) < 1e-15):
        theta = 2.0 * math.atan2(-m[2].imag, m[0].real)
        if _close(m, g_rx(theta)):
            return "rx", "(%.17f)" % theta
    if (m[0].imag == 0.0 and m[1].imag == 0.0 and m[2].imag == 0.0 and m[3].imag == 0.0
            and abs(m[0].real - m[3].real) < 1e-15 and abs(m[1].real + m[2].real) < 1e-15):
        theta = 2.0 * math.atan2(m[2].real, m[0].real)
        if _close(m, g_ry(theta)):
            return "ry", "(%.17f)" % theta
    if m[1] == 0 and m[2] == 0:
        theta = -2.0 * math.atan2(m[0].imag, m[0].real)
        if _close(m, g_rz(theta)):
            return "rz", "(%.17f)" % theta
        lam = math.atan2(m[3].imag, m[3].real)
        if _close(m, g_phase(lam)):
            return "p", "(%.17f)" % lam
    raise QasmError(0, 0, "gate has no OpenQASM 3 name; use a named gate constructor")


def emit(circuit):
    """circuit = (num_qubits, num_classical, ops) in the module's op form,
    with apply2 carrying a 16-entry matrix instead of a name."""
    nq, ncl, ops = circuit
    out = ["OPENQASM 3.0;\n", 'include "stdgates.inc";\n']
    if nq > 0:
        out.append(f"qubit[{nq}] q;\n")
    if ncl > 0:
        out.append(f"bit[{ncl}] c;\n")
    out.append("\n")
    for op in ops:
        out.append(_emit_op(op, 0))
        out.append("\n")
    return "".join(out)


CNOT16 = tuple(complex(v) for v in (1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0))
CZ16 = tuple(complex(v) for v in (1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, -1))
SWAP16 = tuple(complex(v) for v in (1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 1))


def _emit_op(op, depth):
    kind = op[0]
    if kind == "apply1":
        name, args = gate_info_1q(op[1])
        return f"{name}{args} q[{op[2]}];"
    if kind == "apply2":
        m = tuple(complex(z) for z in op[1])
        name = {CNOT16: "cx", CZ16: "cz", SWAP16: "swap"}.get(m)
        if name is None:
            raise QasmError(0, 0, "gate has no OpenQASM 3 name; use a named gate constructor")
        return f"{name} q[{op[2]}], q[{op[3]}];"
    if kind == "ctrl":
        name, args = gate_info_1q(op[2])
        controls = op[1]
        head = "ctrl @ " if len(controls) == 1 else f"ctrl({len(controls)}) @ "
        qs = "".join(f"q[{c}], " for c in controls)
        return f"{head}{name}{args} {qs}q[{op[3]}];"
    if kind == "measure":
        return f"c[{op[2]}] = measure q[{op[1]}];"
    if kind == "if":
        if depth > 0:
            raise QasmError(0, 0, "nested IfClassic is not supported in OpenQASM 3 emit")
        return f"if (c[{op[1]}] == 1) " + _emit_op(op[2], depth + 1)
    raise ValueError(kind)
