"""Seeded synthetic workloads of the benchmark configurations.

All randomness comes from the reference's Rng (xoshiro256++ via SplitMix64)
with documented seeds; angles are 2*pi*next_f64().

  random_layers   depth layers of Rz(a) Ry(b) Rz(c) on every qubit (in that
                  gate order, qubit by qubit, a/b/c drawn in that order), then a
                  CNOT brick: (2i, 2i+1) on even layers, (2i+1, 2i+2) on odd.
  qft_on_basis    X on the set bits of a basis index j, then qft(n).
  haar_layers     a Haar-random 1-qubit unitary on every qubit (QR of a complex
                  Gaussian 2x2 by Gram-Schmidt, columns phase-fixed by
                  diag(R)/|diag(R)|), then a CZ brick with the same pattern.
  tfim_step_circuit
                  steps of RZZ(2 J_i dt) on every bond then RX(2 h_i dt) on
                  every qubit (open chain).
  ghz_midmeasure  GHZ(n), measure qubit 0 into c0, X on qubit n-1 if c0.
"""
from __future__ import annotations

import math

import numpy as np

from .algorithms import ghz, qft
from .circuit import Circuit
from .gate import Gate1, Gate2
from .rng import Rng


def random_layers(n: int, depth: int, seed: int = 1) -> Circuit:
    rng = Rng.seed_from_u64(seed)
    c = Circuit(n)
    for layer in range(depth):
        for q in range(n):
            a = math.tau * rng.next_f64()
            b = math.tau * rng.next_f64()
            cc = math.tau * rng.next_f64()
            c.rz(q, a).ry(q, b).rz(q, cc)
        start = 0 if layer % 2 == 0 else 1
        for i in range(start, n - 1, 2):
            c.cnot(i, i + 1)
    return c


def qft_on_basis(n: int, j: int) -> Circuit:
    c = Circuit(n)
    for bit in range(n):
        if (j >> bit) & 1:
            c.x(bit)
    c.compose(qft(n))
    return c


def qft_closed_form(n: int, j: int) -> np.ndarray:
    """QFT|j> = 2^{-n/2} sum_k e^{2 pi i jk / 2^n} |k> with jk reduced mod 2^n
    in integers before the trig."""
    dim = 1 << n
    k = np.arange(dim, dtype=np.uint64)
    ph = (np.uint64(j) * k) & np.uint64(dim - 1)
    ang = math.tau * ph.astype(np.float64) / float(dim)
    return (np.cos(ang) + 1j * np.sin(ang)) / math.sqrt(dim)


def _normal_pair(rng: Rng) -> tuple[float, float]:
    # Box-Muller on (1 - u1) in (0, 1] so the log is finite.
    u1 = 1.0 - rng.next_f64()
    u2 = rng.next_f64()
    r = math.sqrt(-2.0 * math.log(u1))
    return r * math.cos(math.tau * u2), r * math.sin(math.tau * u2)


def haar_1q(rng: Rng) -> Gate1:
    z = []
    for _ in range(4):
        g1, g2 = _normal_pair(rng)
        z.append(complex(g1, g2) / math.sqrt(2.0))
    a = np.array([[z[0], z[1]], [z[2], z[3]]], dtype=np.complex128)
    # Gram-Schmidt QR on the columns
    q0 = a[:, 0] / np.linalg.norm(a[:, 0])
    r00 = np.linalg.norm(a[:, 0])
    r01 = np.vdot(q0, a[:, 1])
    v = a[:, 1] - r01 * q0
    r11 = np.linalg.norm(v)
    q1 = v / r11
    # phase fix: Q * diag(R)/|diag(R)| (R's diagonal is real positive here)
    d0 = r00 / abs(r00)
    d1 = r11 / abs(r11)
    q = np.stack([q0 * d0, q1 * d1], axis=1)
    return Gate1(q[0, 0], q[0, 1], q[1, 0], q[1, 1])


def haar_layers(n: int, depth: int, seed: int = 3) -> Circuit:
    rng = Rng.seed_from_u64(seed)
    c = Circuit(n)
    for layer in range(depth):
        for q in range(n):
            c.gate1(haar_1q(rng), q)
        start = 0 if layer % 2 == 0 else 1
        for i in range(start, n - 1, 2):
            c.cz(i, i + 1)
    return c


def tfim_step_circuit(n: int, J, h, dt: float, steps: int) -> Circuit:
    c = Circuit(n)
    for _ in range(steps):
        for i in range(n - 1):
            c.gate2(Gate2.rzz(2.0 * J[i] * dt), i, i + 1)
        for i in range(n):
            c.rx(i, 2.0 * h[i] * dt)
    return c


def tfim_instance(rng: Rng, nmin: int = 8, nmax: int = 20, smin: int = 10, smax: int = 50,
                  dt: float = 0.05) -> Circuit:
    """One circuit of the batched TFIM workload: n ~ U{nmin..nmax},
    J_i, h_i ~ U[0.5, 1.5], steps ~ U{smin..smax}."""
    n = nmin + int(rng.next_u64() % (nmax - nmin + 1))
    steps = smin + int(rng.next_u64() % (smax - smin + 1))
    J = [0.5 + rng.next_f64() for _ in range(n - 1)]
    h = [0.5 + rng.next_f64() for _ in range(n)]
    return tfim_step_circuit(n, J, h, dt, steps)


def ghz_midmeasure(n: int) -> Circuit:
    c = Circuit.with_classical(n, 1)
    c.compose(ghz(n))
    c.measure(0, 0)
    c.x_if(0, n - 1)
    return c


def op_bytes(op, n: int, amp_bytes: int = 16) -> int:
    """Algorithmic HBM bytes of one op run on its own: 2 * N_t * B, with N_t
    the amplitudes the op can change (dense/diagonal 1q: N; phase 1q: N/2;
    c-controlled 1q: N/2^c, controlled phase N/2^(c+1); CNOT/SWAP: N/2;
    CZ: N/4; other 2q: N).  A measurement reads N and then reads and writes
    N (counted as 1.5 * 2 * N * B)."""
    from .circuit import Apply1, Apply2, Controlled, IfClassic, Measure
    dim = 1 << n
    if isinstance(op, Apply1):
        m = op.gate.m
        if m[1] == 0 and m[2] == 0 and m[0] == 1:
            return 0 if m[3] == 1 else 2 * (dim // 2) * amp_bytes
        return 2 * dim * amp_bytes
    if isinstance(op, Controlled):
        c = len(set(op.controls))
        m = op.gate.m
        if m[1] == 0 and m[2] == 0 and m[0] == 1:
            return 2 * (dim >> (c + 1)) * amp_bytes
        return 2 * (dim >> c) * amp_bytes
    if isinstance(op, Apply2):
        if op.gate == Gate2.cnot() or op.gate == Gate2.swap():
            return 2 * (dim // 2) * amp_bytes
        if op.gate == Gate2.cz():
            return 2 * (dim // 4) * amp_bytes
        return 2 * dim * amp_bytes
    if isinstance(op, Measure):
        return 3 * dim * amp_bytes
    if isinstance(op, IfClassic):
        return op_bytes(op.then, n, amp_bytes)
    return 0


def gate_bytes(circuit: Circuit, amp_bytes: int = 16) -> int:
    """Algorithmic HBM bytes of running a circuit gate by gate (sum of
    op_bytes)."""
    n = circuit.num_qubits()
    return sum(op_bytes(op, n, amp_bytes) for op in circuit.ops())


def _kind1(m) -> str:
    """The engine's 1-qubit classification (exact 0/1 tests, as classify1)."""
    off0 = m[1] == 0 and m[2] == 0
    if off0:
        if m[0] == 1 and m[3] == 1:
            return "ident"
        return "phase" if m[0] == 1 else "diag"
    if m[0] == 0 and m[3] == 0:
        return "anti"
    if all(complex(z).imag == 0 for z in m):
        return "real"
    return "dense"


# FP64 instructions per amplitude the op touches, from the kernels' source:
# a complex product in the reference's FMA form is 4 (2 mul + 2 fma), a
# complex add 2, a real-times-complex product 2.
_FP64_1Q = {"dense": 10, "real": 6, "diag": 4, "phase": 4, "anti": 4, "ident": 0}


def fp64_instructions(circuit: Circuit) -> float:
    """FP64 instructions a complex128 run of the circuit issues, summed over
    its gates (measurements excluded): the roofline of the exact path."""
    from .circuit import Apply1, Apply2, Controlled, IfClassic
    n = circuit.num_qubits()
    dim = float(1 << n)
    total = 0.0
    for op in circuit.ops():
        while isinstance(op, IfClassic):
            op = op.then
        if isinstance(op, Apply1):
            k = _kind1(op.gate.m)
            total += _FP64_1Q[k] * (dim / 2 if k == "phase" else dim)
        elif isinstance(op, Controlled):
            k = _kind1(op.gate.m)
            frac = dim / (1 << len(set(op.controls)))
            total += _FP64_1Q[k] * (frac / 2 if k == "phase" else frac)
        elif isinstance(op, Apply2):
            m = op.gate.m.reshape(4, 4)
            off = m - np.diag(np.diag(m))
            perm = bool(np.all((m == 0) | (m == 1) | (m == -1)))
            if perm:
                continue
            total += (4 if not np.any(off) else 22) * dim
    return total


class RawCircuit:
    """A gate-only circuit held directly as C ABI op records (for large
    generated workloads where building Python op objects would dominate)."""

    def __init__(self, n: int, ops: np.ndarray):
        from . import _native as N
        self._n = n
        self._ops = np.ascontiguousarray(ops, dtype=N.OP_DTYPE)
        self._ctrl = np.zeros(1, dtype=np.uint64)

    def num_qubits(self) -> int:
        return self._n

    def num_classical(self) -> int:
        return 0

    def __len__(self) -> int:
        return len(self._ops)

    def to_ev(self):
        return self._ops, self._ctrl, 0

    def ev_struct(self):
        from . import _native as N
        c = N.EvCircuit()
        c.num_qubits = self._n
        c.num_classical = 0
        c.ops = self._ops.ctypes.data if len(self._ops) else None
        c.nops = len(self._ops)
        c.ctrl_pool = self._ctrl.ctypes.data
        c.pool_len = 0
        return c

    def to_circuit(self) -> Circuit:
        """The same ops as a builder Circuit (for the oracle and small cases)."""
        from .gate import Gate1, Gate2
        c = Circuit(self._n)
        for r in self._ops:
            m = r["m"].view(np.complex128)
            if r["kind"] == 1:
                c.gate1(Gate1(*m[:4]), int(r["q0"]))
            else:
                c.gate2(Gate2(m), int(r["q0"]), int(r["q1"]))
        return c


def tfim_raw(rng: Rng, nmin: int = 8, nmax: int = 20, smin: int = 10, smax: int = 50,
             dt: float = 0.05) -> RawCircuit:
    """tfim_instance with the same draws, emitted as op records: steps of
    RZZ(2 J_i dt) on every bond, then RX(2 h_i dt) on every qubit."""
    from . import _native as N
    n = nmin + int(rng.next_u64() % (nmax - nmin + 1))
    steps = smin + int(rng.next_u64() % (smax - smin + 1))
    J = [0.5 + rng.next_f64() for _ in range(n - 1)]
    h = [0.5 + rng.next_f64() for _ in range(n)]
    step = np.zeros(2 * n - 1, dtype=N.OP_DTYPE)
    for i in range(n - 1):
        step[i]["kind"] = N.OP_APPLY2
        step[i]["q0"], step[i]["q1"] = i, i + 1
        step[i]["m"][:] = Gate2.rzz(2.0 * J[i] * dt).as_f64()
    for i in range(n):
        r = step[n - 1 + i]
        r["kind"] = N.OP_APPLY1
        r["q0"] = i
        r["m"][:8] = Gate1.rx(2.0 * h[i] * dt).as_f64()
    return RawCircuit(n, np.tile(step, steps))


def random_layers_raw(n: int, depth: int, seed: int = 1) -> RawCircuit:
    """random_layers with the same draws and matrices, as op records."""
    from . import _native as N
    rng = Rng.seed_from_u64(seed)
    recs = []
    for layer in range(depth):
        for q in range(n):
            for ctor in (Gate1.rz, Gate1.ry, Gate1.rz):
                r = np.zeros((), dtype=N.OP_DTYPE)
                r["kind"] = N.OP_APPLY1
                r["q0"] = q
                r["m"][:8] = ctor(math.tau * rng.next_f64()).as_f64()
                recs.append(r)
        for i in range(0 if layer % 2 == 0 else 1, n - 1, 2):
            r = np.zeros((), dtype=N.OP_DTYPE)
            r["kind"] = N.OP_APPLY2
            r["q0"], r["q1"] = i, i + 1
            r["m"][:] = Gate2.cnot().as_f64()
            recs.append(r)
    return RawCircuit(n, np.array(recs, dtype=N.OP_DTYPE))


def serve_request(rng: Rng, nmin: int = 10, nmax: int = 26):
    """One request of the serving mix: n ~ U{nmin..nmax}; 40% random layers
    at depth 2n, 20% QFT of a random basis state, 20% GHZ with a mid-circuit
    measurement of qubit 0 and an X on the last qubit if it read 1, 20%
    TFIM Trotter (steps 10..50).  Returns (kind, circuit)."""
    n = nmin + int(rng.next_u64() % (nmax - nmin + 1))
    u = rng.next_f64()
    if u < 0.4:
        return "random", random_layers_raw(n, 2 * n, seed=rng.next_u64())
    if u < 0.6:
        return "qft", qft_on_basis(n, int(rng.next_u64() % (1 << n)))
    if u < 0.8:
        return "ghz_measure", ghz_midmeasure(n)
    J = [0.5 + rng.next_f64() for _ in range(n - 1)]
    h = [0.5 + rng.next_f64() for _ in range(n)]
    steps = 10 + int(rng.next_u64() % 41)
    return "tfim", _tfim_raw_from(n, J, h, 0.05, steps)


def _tfim_raw_from(n, J, h, dt, steps) -> RawCircuit:
    from . import _native as N
    step = np.zeros(2 * n - 1, dtype=N.OP_DTYPE)
    for i in range(n - 1):
        step[i]["kind"] = N.OP_APPLY2
        step[i]["q0"], step[i]["q1"] = i, i + 1
        step[i]["m"][:] = Gate2.rzz(2.0 * J[i] * dt).as_f64()
    for i in range(n):
        r = step[n - 1 + i]
        r["kind"] = N.OP_APPLY1
        r["q0"] = i
        r["m"][:8] = Gate1.rx(2.0 * h[i] * dt).as_f64()
    return RawCircuit(n, np.tile(step, steps))
