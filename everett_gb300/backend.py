"""CudaStateVectorBackend: the drop-in for everett's StateVectorBackend
(src/backend/statevector.rs:25-106), with the state resident in GB300 HBM.

``run`` / ``run_seeded`` validate the circuit, start from |0...0>, seed the
measurement stream with the reference's Rng and walk the ops on the device;
the returned :class:`Execution` holds a device-resident :class:`State` and
the classical register.  The per-op methods mirror the ``Backend`` trait
(src/backend/mod.rs:25-39) for callers that drive gates themselves.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .circuit import Circuit
from .gate import Gate1, Gate2
from .rng import Rng

_DTYPES = {"complex128": N.C128, "c128": N.C128, "complex64": N.C64, "c64": N.C64,
           N.C128: N.C128, N.C64: N.C64}
_MODES = {"exact": N.MODE_EXACT, "tiled": N.MODE_TILED, "fused": N.MODE_FUSED,
          N.MODE_EXACT: N.MODE_EXACT, N.MODE_TILED: N.MODE_TILED, N.MODE_FUSED: N.MODE_FUSED}
_VARIANTS = {"tf32x3": N.FUSED_TF32X3, "bf16x3": N.FUSED_BF16X3, "fp32": N.FUSED_FP32,
             "ozaki": N.FUSED_OZAKI, "ozaki6": N.FUSED_OZAKI6,
             N.FUSED_TF32X3: N.FUSED_TF32X3, N.FUSED_BF16X3: N.FUSED_BF16X3,
             N.FUSED_FP32: N.FUSED_FP32, N.FUSED_OZAKI: N.FUSED_OZAKI,
             N.FUSED_OZAKI6: N.FUSED_OZAKI6}


class State:
    """A device-resident statevector (src/state.rs:24-185)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def zero(cls, n: int, dtype="complex128") -> "State":
        h = C.c_void_p()
        N.check(N.lib().ev_state_create(n, _DTYPES[dtype], C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_amplitudes(cls, amps, dtype="complex128") -> "State":
        a = np.ascontiguousarray(amps, dtype=np.complex128)
        length = a.shape[0]
        if length == 0 or length & (length - 1):
            from .error import DimensionMismatch
            raise DimensionMismatch(
                f"amplitude buffer has length {length}, expected "
                f"{1 << max(0, (length - 1).bit_length())}")
        s = cls.zero(length.bit_length() - 1, dtype)
        N.check(N.lib().ev_state_upload(s._h, a.ctypes.data, length))
        return s

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().ev_state_destroy(h)
            except Exception:
                pass
            self._h = None

    def close(self) -> None:
        self.__del__()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def num_qubits(self) -> int:
        out = C.c_uint64()
        N.check(N.lib().ev_state_num_qubits(self._h, C.byref(out)))
        return out.value

    def dtype(self) -> str:
        out = C.c_int32()
        N.check(N.lib().ev_state_dtype(self._h, C.byref(out)))
        return "complex128" if out.value == N.C128 else "complex64"

    def dim(self) -> int:
        return 1 << self.num_qubits()

    def amplitudes(self) -> np.ndarray:
        out = np.empty(self.dim(), dtype=np.complex128)
        N.check(N.lib().ev_state_download(self._h, out.ctypes.data, out.shape[0]))
        return out

    def upload(self, amps) -> None:
        a = np.ascontiguousarray(amps, dtype=np.complex128)
        N.check(N.lib().ev_state_upload(self._h, a.ctypes.data, a.shape[0]))

    def set_zero(self) -> None:
        N.check(N.lib().ev_state_set_zero(self._h))

    def norm_sqr(self) -> float:
        out = C.c_double()
        N.check(N.lib().ev_norm_sqr(self._h, C.byref(out)))
        return out.value

    def normalize(self) -> None:
        N.check(N.lib().ev_normalize(self._h))

    def probability(self, basis: int) -> float:
        out = C.c_double()
        N.check(N.lib().ev_probability(self._h, basis, C.byref(out)))
        return out.value

    def amplitude(self, basis: int) -> complex:
        out = (C.c_double * 2)()
        N.check(N.lib().ev_amplitude(self._h, basis, out))
        return complex(out[0], out[1])

    def overlap(self, other: "State") -> complex:
        out = (C.c_double * 2)()
        N.check(N.lib().ev_overlap(self._h, other._h, out))
        return complex(out[0], out[1])

    def max_abs_diff(self, other: "State") -> float:
        """max_j |self_j - other_j| (either amplitude type), on the device."""
        out = C.c_double()
        N.check(N.lib().ev_max_abs_diff(self._h, other._h, C.byref(out)))
        return out.value

    def fidelity(self, other: "State") -> float:
        out = C.c_double()
        N.check(N.lib().ev_fidelity(self._h, other._h, C.byref(out)))
        return out.value

    def marginal_low(self, m: int) -> np.ndarray:
        """Probabilities of the low m qubits summed over the others
        (most_probable_phase's marginal, phase_estimation.rs:97-110), reduced
        on the device; 2^m doubles come back."""
        out = np.empty(1 << m, dtype=np.float64)
        N.check(N.lib().ev_marginal_low(self._h, m, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def bloch_vector(self, qubit: int) -> list:
        out = (C.c_double * 3)()
        N.check(N.lib().ev_bloch_vector(self._h, qubit, out))
        return [out[0], out[1], out[2]]

    def pauli_expectation(self, paulis) -> np.ndarray:
        """<psi|P|psi> for each Pauli string (PauliString or text like "+XZI")."""
        from .observables import expectations
        return expectations(self, paulis)

    def sample(self, shots: int, seed: int = 0) -> np.ndarray:
        """Full-register shots (bit q of each value = qubit q)."""
        out = np.empty(shots, dtype=np.uint64)
        N.check(N.lib().ev_sample(self._h, seed, shots, out.ctypes.data))
        return out

    def synchronize(self) -> None:
        N.check(N.lib().ev_state_synchronize(self._h))

    # gate kernels (kernel.rs:76, :192, :299)
    def apply_1q(self, k: int, gate: Gate1) -> None:
        m = gate.as_f64()
        N.check(N.lib().ev_apply_1q(self._h, k, m.ctypes.data))

    def apply_2q(self, a: int, b: int, gate: Gate2) -> None:
        m = gate.as_f64()
        N.check(N.lib().ev_apply_2q(self._h, a, b, m.ctypes.data))

    def apply_controlled_1q(self, controls, target: int, gate: Gate1) -> None:
        m = gate.as_f64()
        cs = np.array(list(controls) or [0], dtype=np.uint64)
        N.check(N.lib().ev_apply_controlled_1q(self._h, cs.ctypes.data, len(controls), target,
                                               m.ctypes.data))

    def measure_qubit(self, k: int, u: float) -> bool:
        out = C.c_int32()
        N.check(N.lib().ev_measure_qubit(self._h, k, u, C.byref(out)))
        return bool(out.value)


class Execution:
    """The final state and classical register (statevector.rs:40-54)."""

    def __init__(self, state: State, classical: list):
        self._state = state
        self._classical = classical

    def state(self) -> State:
        return self._state

    def classical(self) -> list:
        return self._classical

    def into_state(self) -> State:
        return self._state


class PreparedRun:
    """A circuit planned once for a state and recorded as one CUDA graph.

    ``launch(seed)`` replays the whole run (reset, gates, device-side
    measurement and classical control) with a single graph launch and gives
    the classical register; the state then holds the run's final amplitudes,
    exactly as after ``CudaStateVectorBackend.run_into`` with the same seed.
    """

    def __init__(self, state: State, circuit: Circuit, mode="tiled", tile_bits=0,
                 variant=None):
        c = circuit.ev_struct()
        opts = _options(state.dtype(), mode, tile_bits, variant)
        h = C.c_void_p()
        N.check(N.lib().ev_prepare(state.handle, C.byref(c), C.byref(opts), C.byref(h)))
        self._h = h
        self._state = state  # the state must outlive the prepared run
        self._ncl = circuit.num_classical()
        self._classical = np.zeros(max(1, self._ncl), dtype=np.uint8)

    def launch(self, seed: int = 0) -> list:
        N.check(N.lib().ev_prepared_launch(self._h, seed, self._classical.ctypes.data))
        return [bool(b) for b in self._classical[:self._ncl]]

    def kernels(self) -> int:
        out = C.c_uint64()
        N.check(N.lib().ev_prepared_kernels(self._h, C.byref(out)))
        return out.value

    def state(self) -> State:
        return self._state

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().ev_prepared_destroy(h)
            except Exception:
                pass
            self._h = None

    def __del__(self):
        self.close()


def _options(dtype, mode, tile_bits, variant=None) -> N.EvRunOptions:
    o = N.EvRunOptions()
    o.dtype = _DTYPES[dtype]
    o.mode = _MODES[mode]
    o.tile_bits = int(tile_bits)
    if variant is None:  # the fused arithmetic of the state's type
        variant = "ozaki" if o.dtype == N.C128 else "tf32x3"
    o.variant = _VARIANTS[variant]
    return o


class CudaStateVectorBackend:
    """Simulates a circuit on one GB300 by evolving a device-resident State.

    The class methods mirror ``StateVectorBackend::run`` / ``run_seeded``; an
    instance mirrors the ``Backend`` trait (apply_1q, apply_2q,
    apply_controlled, measure) with its own seeded Rng.
    """

    def __init__(self, num_qubits: int, seed: int = 0, dtype="complex128"):
        self._state = State.zero(num_qubits, dtype)
        self._rng = Rng.seed_from_u64(seed)

    @classmethod
    def run(cls, circuit: Circuit, dtype="complex128", mode="tiled", tile_bits=0,
            variant=None) -> Execution:
        """mode: "exact" (one kernel per op), "tiled" (runs of ops per
        shared-memory pass) or "fused" (dense k-qubit unitaries, k =
        tile_bits; complex64 arithmetic = variant "tf32x3" (default) |
        "bf16x3" | "fp32", complex128 = "ozaki" or "ozaki6" (six digits,
        faster, ~7e-14 of a row's largest value per pass): 5-qubit unitaries on the
        tensor cores by 8-bit digit slicing)."""
        return cls.run_seeded(circuit, 0, dtype=dtype, mode=mode, tile_bits=tile_bits,
                              variant=variant)

    @classmethod
    def run_seeded(cls, circuit: Circuit, seed: int, dtype="complex128", mode="tiled",
                   tile_bits=0, variant=None) -> Execution:
        c = circuit.ev_struct()
        opts = _options(dtype, mode, tile_bits, variant)
        h = C.c_void_p()
        ncl = circuit.num_classical()
        classical = np.zeros(max(1, ncl), dtype=np.uint8)
        N.check(N.lib().ev_run_seeded(C.byref(c), seed, C.byref(opts), C.byref(h),
                                      classical.ctypes.data))
        return Execution(State(h.value), [bool(b) for b in classical[:ncl]])

    @staticmethod
    def run_into(state: State, circuit: Circuit, seed: int = 0, mode="tiled",
                 tile_bits=0, variant=None) -> list:
        """Runs a circuit on an existing state (reset to |0...0> first)."""
        c = circuit.ev_struct()
        opts = _options(state.dtype(), mode, tile_bits, variant)
        ncl = circuit.num_classical()
        classical = np.zeros(max(1, ncl), dtype=np.uint8)
        N.check(N.lib().ev_state_run(state.handle, C.byref(c), seed, C.byref(opts),
                                     classical.ctypes.data))
        return [bool(b) for b in classical[:ncl]]

    @staticmethod
    def drive(state: State, circuit: Circuit, seed: int = 0, mode="tiled",
              tile_bits=0, variant=None) -> list:
        """Applies a circuit's ops to the state as it stands (drive,
        backend/mod.rs:43-72); returns the classical register."""
        c = circuit.ev_struct()
        opts = _options(state.dtype(), mode, tile_bits, variant)
        ncl = circuit.num_classical()
        classical = np.zeros(max(1, ncl), dtype=np.uint8)
        N.check(N.lib().ev_state_drive(state.handle, C.byref(c), seed, C.byref(opts),
                                       classical.ctypes.data))
        return [bool(b) for b in classical[:ncl]]

    @staticmethod
    def prepare(state: State, circuit: Circuit, mode="tiled", tile_bits=0,
                variant=None) -> PreparedRun:
        """Plans a circuit for a state once and records it as a CUDA graph;
        each ``launch(seed)`` of the result equals ``run_into`` with that
        seed."""
        return PreparedRun(state, circuit, mode, tile_bits, variant)

    # Backend trait (src/backend/mod.rs:25-39)
    def state(self) -> State:
        return self._state

    def apply_1q(self, gate: Gate1, target: int) -> None:
        self._state.apply_1q(target, gate)

    def apply_2q(self, gate: Gate2, a: int, b: int) -> None:
        self._state.apply_2q(a, b, gate)

    def apply_controlled(self, controls, gate: Gate1, target: int) -> None:
        self._state.apply_controlled_1q(controls, target, gate)

    def measure(self, qubit: int) -> bool:
        return self._state.measure_qubit(qubit, self._rng.next_f64())
