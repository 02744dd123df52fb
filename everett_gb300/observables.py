"""Pauli-string observables, mirroring everett's PauliString
(src/backend/stabilizer.rs:26-137), evaluated on device-resident states.

``PauliString.expectation(state)`` is ``<psi|P|psi>``; ``expectations``
evaluates many strings at once, sharing one pass over the state among
strings with the same X part (ev_pauli_expectation).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


class PauliString:
    """A Pauli operator on n qubits with a +1/-1 sign: per qubit an (x, z)
    bit pair, I = (0, 0), X = (1, 0), Z = (0, 1), Y = (1, 1)."""

    __slots__ = ("x", "z", "neg")

    def __init__(self, x, z, neg: bool = False):
        if len(x) != len(z):
            raise ValueError("x and z must have one bit per qubit")
        self.x = np.asarray(x, dtype=bool).copy()
        self.z = np.asarray(z, dtype=bool).copy()
        self.neg = bool(neg)

    @classmethod
    def parse(cls, text: str) -> "PauliString":
        """From the Display form, e.g. "+XZIY" or "-ZZ" (qubit 0 first)."""
        neg = text.startswith("-")
        body = text[1:] if text[:1] in "+-" else text
        x = [c in "XY" for c in body]
        z = [c in "ZY" for c in body]
        if any(c not in "IXYZ" for c in body):
            raise ValueError(f"not a Pauli string: {text!r}")
        return cls(x, z, neg)

    def num_qubits(self) -> int:
        return len(self.x)

    def is_negative(self) -> bool:
        return self.neg

    def pauli(self, q: int) -> str:
        return "IZXY"[2 * int(self.x[q]) + int(self.z[q])]

    def masks(self) -> tuple:
        xm = sum(1 << int(q) for q in np.flatnonzero(self.x))
        zm = sum(1 << int(q) for q in np.flatnonzero(self.z))
        return xm, zm

    def __str__(self):
        codes = np.array(list("IZXY"))[2 * self.x.astype(int) + self.z.astype(int)]
        return ("-" if self.neg else "+") + "".join(codes.tolist())

    def __repr__(self):
        return f"PauliString({str(self)!r})"

    def __eq__(self, other):
        return (isinstance(other, PauliString) and np.array_equal(self.x, other.x)
                and np.array_equal(self.z, other.z) and self.neg == other.neg)

    def expectation(self, state) -> float:
        if state.num_qubits() != self.num_qubits():
            raise ValueError("qubit count mismatch")
        return expectations(state, [self])[0]


def expectations(state, paulis) -> np.ndarray:
    """<psi|P_t|psi> for every P_t (PauliString or its text form)."""
    ps = [p if isinstance(p, PauliString) else PauliString.parse(p) for p in paulis]
    n = state.num_qubits()
    for p in ps:
        if p.num_qubits() != n:
            raise ValueError("qubit count mismatch")
    xm = np.array([p.masks()[0] for p in ps] or [0], dtype=np.uint64)
    zm = np.array([p.masks()[1] for p in ps] or [0], dtype=np.uint64)
    neg = np.array([p.neg for p in ps] or [0], dtype=np.uint8)
    out = np.zeros(max(1, len(ps)))
    N.check(N.lib().ev_pauli_expectation(state.handle, xm.ctypes.data, zm.ctypes.data,
                                         neg.ctypes.data, len(ps), out.ctypes.data))
    return out[:len(ps)]
