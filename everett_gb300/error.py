"""Errors of the engine, mirroring everett::Error (src/error.rs:10-53).

The first four classes correspond one-to-one to the reference's variants that
the statevector path can raise; the rest are device conditions the CPU crate
has no counterpart for.
"""
from __future__ import annotations

from . import _native as N


class EverettError(Exception):
    """Base class; ``code`` is the C ABI's EV_ERR_* value."""

    code = -1


class QubitOutOfRange(EverettError):
    code = N.ERR_QUBIT_OUT_OF_RANGE


class ClassicalBitOutOfRange(EverettError):
    code = N.ERR_CLASSICAL_BIT_OUT_OF_RANGE


class DuplicateQubit(EverettError):
    code = N.ERR_DUPLICATE_QUBIT


class DimensionMismatch(EverettError):
    code = N.ERR_DIMENSION_MISMATCH


class NonClifford(EverettError):
    """Error::NonClifford (src/error.rs:38-43): the stabilizer backend met a
    gate outside the Clifford group."""

    code = N.ERR_NON_CLIFFORD


class QasmError(EverettError):
    """Error::Qasm { line, col, message } (src/error.rs:45-52); str() reads
    "OpenQASM 3 error at L:C: message" as the reference's Display does."""

    code = N.ERR_QASM

    def __init__(self, text: str = "", line: int = 0, col: int = 0, message: str = ""):
        super().__init__(text)
        self.line, self.col, self.message = line, col, message
        if text and not message:
            head = "OpenQASM 3 error at "
            if text.startswith(head):
                pos, _, rest = text[len(head):].partition(": ")
                l, _, c = pos.partition(":")
                if l.isdigit() and c.isdigit():
                    self.line, self.col, self.message = int(l), int(c), rest


class InvalidArgument(EverettError):
    code = N.ERR_INVALID_ARGUMENT


class DeviceOutOfMemory(EverettError):
    code = N.ERR_OOM


class CudaError(EverettError):
    code = N.ERR_CUDA


class DeviceTimeout(EverettError):
    code = N.ERR_TIMEOUT


class AdmissionRefused(EverettError):
    code = N.ERR_ADMISSION


class Cancelled(EverettError):
    code = N.ERR_CANCELLED


_BY_CODE = {cls.code: cls for cls in (
    QubitOutOfRange, ClassicalBitOutOfRange, DuplicateQubit, DimensionMismatch, NonClifford,
    QasmError,
    InvalidArgument,
    DeviceOutOfMemory, CudaError, DeviceTimeout, AdmissionRefused, Cancelled)}


def error_for_code(code: int, message: str) -> EverettError:
    cls = _BY_CODE.get(code, EverettError)
    err = cls(message or f"error code {code}")
    err.code = code
    return err
