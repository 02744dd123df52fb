"""Density matrices and noise, mirroring everett's DensityMatrix
(src/density.rs), NoiseModel / Channel (src/noise.rs) and
DensityMatrixBackend (src/backend/density_matrix.rs), with the matrix
resident in GB300 HBM.

Kraus operators are built on the host with the reference's formulas
(IEEE square roots); the engine applies rho -> U rho U^dagger and
rho -> sum_k K_k rho K_k^dagger with the reference's operation order.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .circuit import Circuit

MAX_KRAUS = 16


class EvChannel(C.Structure):
    _fields_ = [("nops", C.c_uint32), ("reserved", C.c_uint32),
                ("k", (C.c_double * 8) * MAX_KRAUS)]


class EvNoiseModel(C.Structure):
    _fields_ = [("after_1q", EvChannel), ("after_2q", EvChannel), ("readout_error", C.c_double)]


class KrausOp:
    """A 2x2 Kraus operator, row-major (density.rs KrausOp)."""

    __slots__ = ("m",)

    def __init__(self, m):
        self.m = np.asarray(m, dtype=np.complex128).reshape(4).copy()


def _k(a, b, c, d):
    return KrausOp([a, b, c, d])


class Channel:
    """noise.rs Channel: Depolarizing, AmplitudeDamping, PhaseDamping,
    BitFlip, Dephasing, or Custom Kraus operators."""

    def __init__(self, kind: str, param=None):
        self.kind, self.param = kind, param

    @classmethod
    def depolarizing(cls, p):
        return cls("depolarizing", float(p))

    @classmethod
    def amplitude_damping(cls, gamma):
        return cls("amplitude_damping", float(gamma))

    @classmethod
    def phase_damping(cls, lam):
        return cls("phase_damping", float(lam))

    @classmethod
    def bit_flip(cls, p):
        return cls("bit_flip", float(p))

    @classmethod
    def dephasing(cls, p):
        return cls("dephasing", float(p))

    @classmethod
    def custom(cls, ops):
        return cls("custom", [o if isinstance(o, KrausOp) else KrausOp(o) for o in ops])

    def kraus_ops(self) -> list:
        """Channel::kraus_ops (noise.rs)."""
        p = self.param
        if self.kind == "depolarizing":
            a, b = math.sqrt(1.0 - p), math.sqrt(p / 3.0)
            return [_k(a, 0, 0, a), _k(0, b, b, 0), _k(0, complex(0.0, -b), complex(0.0, b), 0),
                    _k(b, 0, 0, -b)]
        if self.kind == "amplitude_damping":
            return [_k(1.0, 0, 0, math.sqrt(1.0 - p)), _k(0, math.sqrt(p), 0, 0)]
        if self.kind == "phase_damping":
            return [_k(1.0, 0, 0, math.sqrt(1.0 - p)), _k(0, 0, 0, math.sqrt(p))]
        if self.kind == "bit_flip":
            a, b = math.sqrt(1.0 - p), math.sqrt(p)
            return [_k(a, 0, 0, a), _k(0, b, b, 0)]
        if self.kind == "dephasing":
            a, b = math.sqrt(1.0 - p), math.sqrt(p)
            return [_k(a, 0, 0, a), _k(b, 0, 0, -b)]
        return list(p)


class NoiseModel:
    """noise.rs NoiseModel: a channel after 1-qubit gates, one after
    2-qubit gates, and a readout-flip probability."""

    def __init__(self, after_1q: Channel | None = None, after_2q: Channel | None = None,
                 readout_error: float = 0.0):
        self.after_1q, self.after_2q, self.readout_error = after_1q, after_2q, float(readout_error)

    @staticmethod
    def _check(v, name):
        if not 0.0 <= v <= 1.0:
            raise ValueError(f"{name} {v} not in [0, 1]")

    @classmethod
    def ideal(cls):
        return cls()

    @classmethod
    def uniform_depolarizing(cls, p):
        cls._check(p, "depolarizing probability")
        return cls(Channel.depolarizing(p), Channel.depolarizing(p))

    @classmethod
    def amplitude_damping(cls, gamma):
        cls._check(gamma, "gamma")
        return cls(Channel.amplitude_damping(gamma), Channel.amplitude_damping(gamma))

    @classmethod
    def phase_damping(cls, lam):
        cls._check(lam, "lambda")
        return cls(Channel.phase_damping(lam), None)

    @classmethod
    def bit_flip(cls, p):
        cls._check(p, "bit-flip probability")
        return cls(Channel.bit_flip(p), None)

    @classmethod
    def dephasing(cls, p):
        cls._check(p, "dephasing probability")
        return cls(Channel.dephasing(p), None)

    def ev_struct(self) -> EvNoiseModel:
        nm = EvNoiseModel()
        for field, ch in (("after_1q", self.after_1q), ("after_2q", self.after_2q)):
            dst = getattr(nm, field)
            ops = ch.kraus_ops() if ch is not None else []
            if len(ops) > MAX_KRAUS:
                raise ValueError(f"at most {MAX_KRAUS} Kraus operators per channel")
            dst.nops = len(ops)
            for i, op in enumerate(ops):
                for e in range(4):
                    dst.k[i][2 * e] = op.m[e].real
                    dst.k[i][2 * e + 1] = op.m[e].imag
        nm.readout_error = self.readout_error
        return nm


class DensityMatrix:
    """A device-resident 2^n x 2^n density matrix (density.rs:32-295)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def zero(cls, n: int) -> "DensityMatrix":
        h = C.c_void_p()
        N.check(N.lib().ev_dm_create(n, C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_statevector(cls, amps) -> "DensityMatrix":
        a = np.ascontiguousarray(amps, dtype=np.complex128)
        h = C.c_void_p()
        N.check(N.lib().ev_dm_from_amplitudes(a.ctypes.data, a.shape[0], C.byref(h)))
        return cls(h.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().ev_dm_destroy(h)
            except Exception:
                pass
            self._h = None

    def num_qubits(self) -> int:
        out = C.c_uint64()
        N.check(N.lib().ev_dm_num_qubits(self._h, C.byref(out)))
        return out.value

    def dim(self) -> int:
        return 1 << self.num_qubits()

    def data(self) -> np.ndarray:
        """The matrix, (dim, dim) complex128, row-major (data(), density.rs:97-102)."""
        d = self.dim()
        out = np.empty((d, d), dtype=np.complex128)
        N.check(N.lib().ev_dm_download(self._h, out.ctypes.data, d * d))
        return out

    def get(self, i: int, j: int) -> complex:
        out = (C.c_double * 2)()
        N.check(N.lib().ev_dm_get(self._h, i, j, out))
        return complex(out[0], out[1])

    def trace(self) -> float:
        out = C.c_double()
        N.check(N.lib().ev_dm_trace(self._h, C.byref(out)))
        return out.value

    def purity(self) -> float:
        out = C.c_double()
        N.check(N.lib().ev_dm_purity(self._h, C.byref(out)))
        return out.value

    def probability(self, basis: int) -> float:
        out = C.c_double()
        N.check(N.lib().ev_dm_probability(self._h, basis, C.byref(out)))
        return out.value

    def expectation_pauli(self, qubit: int, observable: str) -> float:
        out = C.c_double()
        N.check(N.lib().ev_dm_expectation_pauli(self._h, qubit, observable.encode()[:1],
                                                C.byref(out)))
        return out.value

    def partial_trace_1q(self, qubit: int) -> list:
        out = (C.c_double * 8)()
        N.check(N.lib().ev_dm_partial_trace_1q(self._h, qubit, out))
        return [complex(out[2 * e], out[2 * e + 1]) for e in range(4)]


class DensityMatrixExecution:
    """The final density matrix and classical register (density_matrix.rs:27-49)."""

    def __init__(self, rho: DensityMatrix, classical: list):
        self._rho, self._classical = rho, classical

    def density_matrix(self) -> DensityMatrix:
        return self._rho

    def classical(self) -> list:
        return self._classical

    def into_density_matrix(self) -> DensityMatrix:
        return self._rho


class DensityMatrixBackend:
    """DensityMatrixBackend::run / run_with_noise / run_with_noise_seeded
    (density_matrix.rs:52-79) on the GPU."""

    @classmethod
    def run(cls, circuit: Circuit) -> DensityMatrixExecution:
        return cls.run_with_noise_seeded(circuit, NoiseModel.ideal(), 0)

    @classmethod
    def run_with_noise(cls, circuit: Circuit, noise: NoiseModel) -> DensityMatrixExecution:
        return cls.run_with_noise_seeded(circuit, noise, 0)

    @classmethod
    def run_with_noise_seeded(cls, circuit: Circuit, noise: NoiseModel,
                              seed: int) -> DensityMatrixExecution:
        c = circuit.ev_struct()
        nm = noise.ev_struct()
        h = C.c_void_p()
        ncl = circuit.num_classical()
        classical = np.zeros(max(1, ncl), dtype=np.uint8)
        N.check(N.lib().ev_dm_run(C.byref(c), C.byref(nm), seed, C.byref(h),
                                  classical.ctypes.data))
        return DensityMatrixExecution(DensityMatrix(h.value), [bool(b) for b in classical[:ncl]])
