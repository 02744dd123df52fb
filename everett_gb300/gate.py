"""Gate matrices, mirroring everett's Gate1 / Gate2 (src/gate.rs:21-291).

Matrices are built on the host with libm sin/cos exactly as the reference
builds them (Python's math module calls the same C library); the engine only
ever receives matrices.
"""
from __future__ import annotations

import math

import numpy as np

FRAC_1_SQRT_2 = 0.7071067811865476  # std::f64::consts::FRAC_1_SQRT_2


def _expi(theta: float) -> complex:
    return complex(math.cos(theta), math.sin(theta))


class Gate1:
    """A 2x2 complex matrix, row-major [m00, m01, m10, m11] (gate.rs:21-25)."""

    __slots__ = ("m",)

    def __init__(self, m00, m01, m10, m11):
        self.m = np.array([m00, m01, m10, m11], dtype=np.complex128)

    def __eq__(self, other):
        return isinstance(other, Gate1) and bool(np.all(self.m == other.m))

    def __repr__(self):
        return f"Gate1({self.m.tolist()})"

    @classmethod
    def id(cls):
        return cls(1, 0, 0, 1)

    @classmethod
    def x(cls):
        return cls(0, 1, 1, 0)

    @classmethod
    def y(cls):
        return cls(0, complex(0.0, -1.0), complex(0.0, 1.0), 0)

    @classmethod
    def z(cls):
        return cls(1, 0, 0, -1)

    @classmethod
    def h(cls):
        s = FRAC_1_SQRT_2
        return cls(s, s, s, -s)

    @classmethod
    def s(cls):
        return cls(1, 0, 0, 1j)

    @classmethod
    def t(cls):
        return cls(1, 0, 0, _expi(math.pi / 4))

    @classmethod
    def rx(cls, theta: float):  # gate.rs:106-110
        s, co = math.sin(theta / 2.0), math.cos(theta / 2.0)
        return cls(complex(co, 0.0), complex(0.0, -s), complex(0.0, -s), complex(co, 0.0))

    @classmethod
    def ry(cls, theta: float):  # gate.rs:114-118
        s, co = math.sin(theta / 2.0), math.cos(theta / 2.0)
        return cls(complex(co, 0.0), complex(-s, 0.0), complex(s, 0.0), complex(co, 0.0))

    @classmethod
    def rz(cls, theta: float):  # gate.rs:122-130
        return cls(_expi(-theta / 2.0), 0, 0, _expi(theta / 2.0))

    @classmethod
    def phase(cls, lam: float):  # gate.rs:134-136
        return cls(1, 0, 0, _expi(lam))

    @classmethod
    def from_matrix(cls, mat) -> "Gate1":
        a = np.asarray(mat, dtype=np.complex128).reshape(4)
        return cls(*a)

    def adjoint(self) -> "Gate1":
        m = self.m
        return Gate1(m[0].conjugate(), m[2].conjugate(), m[1].conjugate(), m[3].conjugate())

    def as_f64(self) -> np.ndarray:
        """8 interleaved doubles, the C ABI's layout."""
        return self.m.view(np.float64).copy()


class Gate2:
    """A 4x4 complex matrix in the basis |q_a q_b>, a the more significant
    operand (gate.rs:27-35)."""

    __slots__ = ("m",)

    def __init__(self, m):
        self.m = np.asarray(m, dtype=np.complex128).reshape(16).copy()

    def __eq__(self, other):
        return isinstance(other, Gate2) and bool(np.all(self.m == other.m))

    def __repr__(self):
        return f"Gate2({self.m.reshape(4, 4).tolist()})"

    @classmethod
    def cnot(cls):
        return cls([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])

    @classmethod
    def cz(cls):
        return cls(np.diag([1, 1, 1, -1]))

    @classmethod
    def swap(cls):
        return cls([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]])

    @classmethod
    def controlled(cls, u: Gate1):  # gate.rs:240-247
        m = np.zeros((4, 4), dtype=np.complex128)
        m[0, 0] = m[1, 1] = 1
        m[2:, 2:] = u.m.reshape(2, 2)
        return cls(m)

    @classmethod
    def rzz(cls, theta: float):
        """exp(-i theta/2 Z(x)Z): diag(e^{-it/2}, e^{it/2}, e^{it/2}, e^{-it/2})."""
        a, b = _expi(-theta / 2.0), _expi(theta / 2.0)
        return cls(np.diag([a, b, b, a]))

    def adjoint(self) -> "Gate2":
        return Gate2(self.m.reshape(4, 4).conj().T)

    def as_f64(self) -> np.ndarray:
        return self.m.view(np.float64).copy()
