"""everett_gb300: a GB300-native statevector engine that is a drop-in for
everett's CPU StateVectorBackend (hz2/everett, src/backend/statevector.rs).

The compute path is hand-written CUDA for sm_103a behind the C ABI in
include/everett_cuda.h; this package is the host-side mirror of the
reference's public surface (Circuit, Gate1/Gate2, Op, State, Execution, Rng).
"""
from . import algorithms, batch, density, observables, serve, stabilizer, workloads
from ._native import device_count
from .backend import CudaStateVectorBackend, Execution, PreparedRun, State
from .circuit import Apply1, Apply2, Circuit, Controlled, IfClassic, Measure
from .error import (ClassicalBitOutOfRange, DimensionMismatch, DuplicateQubit, EverettError,
                    NonClifford, QasmError, QubitOutOfRange)
from .gate import Gate1, Gate2
from .observables import PauliString
from .rng import Rng

__all__ = [
    "algorithms", "batch", "density", "observables", "serve", "stabilizer", "workloads",
    "PauliString", "NonClifford", "device_count", "CudaStateVectorBackend", "Execution", "PreparedRun",
    "State",
    "Apply1", "Apply2", "Circuit", "Controlled", "IfClassic", "Measure", "ClassicalBitOutOfRange",
    "DimensionMismatch", "DuplicateQubit", "EverettError", "QasmError", "QubitOutOfRange", "Gate1", "Gate2",
    "Rng",
]
