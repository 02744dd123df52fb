"""The stabilizer backend, mirroring everett's StabilizerBackend
(src/backend/stabilizer.rs): Clifford circuits on an Aaronson-Gottesman
tableau held bit-packed in GB300 HBM.  Gates are recognised up to global
phase; any other gate makes the run raise NonClifford."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .circuit import Circuit
from .observables import PauliString


class StabilizerExecution:
    """The final stabilizer generators and classical register
    (stabilizer.rs:179-197)."""

    def __init__(self, generators: list, classical: list):
        self._generators, self._classical = generators, classical

    def generators(self) -> list:
        return self._generators

    def classical(self) -> list:
        return self._classical


class StabilizerBackend:
    @classmethod
    def run(cls, circuit: Circuit) -> StabilizerExecution:
        return cls.run_seeded(circuit, 0)

    @classmethod
    def run_seeded(cls, circuit: Circuit, seed: int) -> StabilizerExecution:
        c = circuit.ev_struct()
        h = C.c_void_p()
        ncl = circuit.num_classical()
        classical = np.zeros(max(1, ncl), dtype=np.uint8)
        N.check(N.lib().ev_stab_run(C.byref(c), seed, C.byref(h), classical.ctypes.data))
        try:
            n = circuit.num_qubits()
            x = np.zeros((max(1, n), max(1, n)), dtype=np.uint8)
            z = np.zeros_like(x)
            neg = np.zeros(max(1, n), dtype=np.uint8)
            N.check(N.lib().ev_stab_generators(h, x.ctypes.data, z.ctypes.data, neg.ctypes.data))
        finally:
            N.lib().ev_stab_destroy(h)
        gens = [PauliString(x[i, :n], z[i, :n], bool(neg[i])) for i in range(n)]
        return StabilizerExecution(gens, [bool(b) for b in classical[:ncl]])
