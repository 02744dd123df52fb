"""Circuit generators of the reference (src/algorithms/*.rs) that build the
workloads of this engine: QFT (qft.rs:54-118), Trotterised TFIM
(hamiltonian.rs:91-118), Bell/GHZ preparation (prep.rs:51-59),
teleportation (teleport.rs:45-85), superdense coding (superdense.rs:35-50)
and phase estimation (phase_estimation.rs:55-121)."""
from __future__ import annotations

import math

from .circuit import Circuit
from .gate import Gate1


def _apply_qft_no_swap(c: Circuit, n: int) -> None:
    for j in range(n - 1, -1, -1):
        c.h(j)
        for k in range(j - 1, -1, -1):
            m = j - k + 1
            c.controlled([k], Gate1.phase(math.tau / float(1 << m)), j)


def _apply_iqft_no_swap(c: Circuit, n: int) -> None:
    for j in range(n):
        for k in range(j):
            m = j - k + 1
            c.controlled([k], Gate1.phase(-math.tau / float(1 << m)), j)
        c.h(j)


def qft(n: int) -> Circuit:
    c = Circuit(n)
    _apply_qft_no_swap(c, n)
    for i in range(n // 2):
        c.swap(i, n - 1 - i)
    return c


def iqft(n: int) -> Circuit:
    c = Circuit(n)
    for i in range(n // 2):
        c.swap(i, n - 1 - i)
    _apply_iqft_no_swap(c, n)
    return c


def trotter_single_z(t: float, steps: int) -> Circuit:
    c = Circuit(1)
    dt = t / float(steps)
    for _ in range(steps):
        c.rz(0, 2.0 * dt)
    return c


def trotter_tfim(n: int, jzz: float, hx: float, t: float, steps: int) -> Circuit:
    assert n >= 1
    c = Circuit(n)
    dt = t / float(steps)
    for _ in range(steps):
        rx_angle = -2.0 * hx * dt
        for i in range(n):
            c.rx(i, rx_angle)
        zz_angle = -2.0 * jzz * dt
        for i in range(n - 1):
            c.cnot(i, i + 1)
            c.rz(i + 1, zz_angle)
            c.cnot(i, i + 1)
    return c


def bell() -> Circuit:
    c = Circuit(2)
    c.h(0).cnot(0, 1)
    return c


def ghz(n: int) -> Circuit:
    assert n >= 2, "GHZ state requires at least 2 qubits"
    c = Circuit(n)
    c.h(0)
    for k in range(n - 1):
        c.cnot(k, k + 1)
    return c


def teleport_circuit() -> Circuit:
    c = Circuit.with_classical(3, 2)
    c.h(1).cnot(1, 2)
    c.cnot(0, 1).h(0)
    c.measure(0, 0).measure(1, 1)
    c.x_if(1, 2).z_if(0, 2)
    return c


def teleport_state(alpha: complex, beta: complex) -> Circuit:
    prep = Gate1(alpha, -beta.conjugate(), beta, alpha.conjugate())
    c = Circuit.with_classical(3, 2)
    c.gate1(prep, 0)
    c.compose(teleport_circuit())
    return c


def superdense_circuit(bit0: bool, bit1: bool) -> Circuit:
    """Encode two bits on one half of a Bell pair and decode them into
    classical bits 0 and 1 (superdense.rs:35-50)."""
    c = Circuit.with_classical(2, 2)
    c.h(0).cnot(0, 1)
    if bit1:
        c.x(0)
    if bit0:
        c.z(0)
    c.cnot(0, 1).h(0)
    c.measure(0, 0).measure(1, 1)
    return c


def phase_estimation(counting_qubits: int, phi: float) -> Circuit:
    """m counting qubits 0..m-1 and the eigenstate qubit m of phase(2*pi*phi)
    (phase_estimation.rs:55-87): X on the target, H on the counting register,
    controlled phase(2*pi*phi*2^j) from counting qubit j, then iqft(m)."""
    m = counting_qubits
    c = Circuit(m + 1)
    c.x(m)
    for j in range(m):
        c.h(j)
    for j in range(m):
        c.controlled([j], Gate1.phase(math.tau * phi * float(1 << j)), m)
    c.compose(iqft(m))
    return c


def most_probable_phase(state, counting_qubits: int) -> float:
    """The most probable counting-register value over 2^m
    (phase_estimation.rs:97-121). The marginal over the other qubits is a
    device reduction summed in the reference's basis order; among equal
    maxima the last index wins, as Rust's Iterator::max_by returns it."""
    m = counting_qubits
    if m > state.num_qubits():
        raise ValueError("most_probable_phase: more counting qubits than the state has")
    marg = state.marginal_low(m)
    best = 0
    for i in range(1, marg.shape[0]):
        if not marg[best] > marg[i]:
            best = i
    return best / float(1 << m)
