"""ctypes binding of the engine's C ABI (include/everett_cuda.h).

The shared library is built in-tree by :mod:`everett_gb300.build`.  There is
no fallback: if the library is missing or cannot be loaded, every entry point
raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libeverett_gb300.so"

# ev_op, 288 bytes (include/everett_cuda.h)
OP_DTYPE = np.dtype(
    [("kind", "<u4"), ("nctrl", "<u4"), ("ctrl_off", "<u8"), ("q0", "<u8"), ("q1", "<u8"),
     ("m", "<f8", (32,))],
    align=True,
)
assert OP_DTYPE.itemsize == 288

OP_APPLY1, OP_APPLY2, OP_CONTROLLED, OP_MEASURE, OP_IF = 1, 2, 3, 4, 5
C128, C64 = 0, 1
MODE_EXACT, MODE_TILED, MODE_FUSED = 0, 1, 2
FUSED_TF32X3, FUSED_BF16X3, FUSED_FP32, FUSED_OZAKI, FUSED_OZAKI6 = 0, 1, 2, 3, 4

OK = 0
ERR_QUBIT_OUT_OF_RANGE = 1
ERR_CLASSICAL_BIT_OUT_OF_RANGE = 2
ERR_DUPLICATE_QUBIT = 3
ERR_DIMENSION_MISMATCH = 4
ERR_NON_CLIFFORD = 5
ERR_QASM = 6
ERR_INVALID_ARGUMENT = 16
ERR_OOM = 17
ERR_CUDA = 18
ERR_TIMEOUT = 19
ERR_ADMISSION = 20
ERR_CANCELLED = 21


class EvCircuit(C.Structure):
    _fields_ = [("num_qubits", C.c_uint64), ("num_classical", C.c_uint64), ("ops", C.c_void_p),
                ("nops", C.c_uint64), ("ctrl_pool", C.c_void_p), ("pool_len", C.c_uint64)]


class EvRunOptions(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("mode", C.c_int32), ("tile_bits", C.c_int32),
                ("variant", C.c_int32)]


_P = C.c_void_p
_U64 = C.c_uint64
_I32 = C.c_int32
_DP = C.POINTER(C.c_double)

# name -> (argtypes)
_SIGS = {
    "ev_last_error": [],
    "ev_version": [],
    "ev_device_count": [C.POINTER(C.c_int)],
    "ev_state_create": [_U64, _I32, C.POINTER(_P)],
    "ev_state_destroy": [_P],
    "ev_state_num_qubits": [_P, C.POINTER(_U64)],
    "ev_state_dtype": [_P, C.POINTER(_I32)],
    "ev_state_set_zero": [_P],
    "ev_state_upload": [_P, _P, _U64],
    "ev_state_download": [_P, _P, _U64],
    "ev_state_synchronize": [_P],
    "ev_apply_1q": [_P, _U64, _P],
    "ev_apply_2q": [_P, _U64, _U64, _P],
    "ev_apply_controlled_1q": [_P, _P, _U64, _U64, _P],
    "ev_measure_qubit": [_P, _U64, C.c_double, C.POINTER(_I32)],
    "ev_measure_qubit_noalloc": [_P, _U64, _U64, C.c_double, _P, C.POINTER(_I32)],
    "ev_norm_sqr": [_P, _DP],
    "ev_normalize": [_P],
    "ev_probability": [_P, _U64, _DP],
    "ev_amplitude": [_P, _U64, _P],
    "ev_overlap": [_P, _P, _P],
    "ev_fidelity": [_P, _P, _DP],
    "ev_bloch_vector": [_P, _U64, _P],
    "ev_validate": [C.POINTER(EvCircuit)],
    "ev_run_seeded": [C.POINTER(EvCircuit), _U64, C.POINTER(EvRunOptions), C.POINTER(_P), _P],
    "ev_state_run": [_P, C.POINTER(EvCircuit), _U64, C.POINTER(EvRunOptions), _P],
    "ev_state_drive": [_P, C.POINTER(EvCircuit), _U64, C.POINTER(EvRunOptions), _P],
    "ev_sample": [_P, _U64, _U64, _P],
    "ev_state_record_event": [_P, _I32],
    "ev_state_elapsed_ms": [_P, _I32, _I32, C.POINTER(C.c_float)],
    "ev_state_launch_count": [_P, C.POINTER(_U64)],
    "ev_state_profile": [_P, _I32],
    "ev_state_profile_read": [_P, _P, _I32, C.POINTER(_I32)],
    "ev_batch_run": [_P, _U64, _P, _P],
    "ev_stab_run": [C.POINTER(EvCircuit), _U64, C.POINTER(_P), _P],
    "ev_stab_num_qubits": [_P, C.POINTER(_U64)],
    "ev_stab_generators": [_P, _P, _P, _P],
    "ev_stab_destroy": [_P],
    "ev_dm_create": [_U64, C.POINTER(_P)],
    "ev_dm_destroy": [_P],
    "ev_dm_num_qubits": [_P, C.POINTER(_U64)],
    "ev_dm_from_amplitudes": [_P, _U64, C.POINTER(_P)],
    "ev_dm_download": [_P, _P, _U64],
    "ev_dm_get": [_P, _U64, _U64, _P],
    "ev_dm_trace": [_P, _DP],
    "ev_dm_purity": [_P, _DP],
    "ev_dm_probability": [_P, _U64, _DP],
    "ev_dm_expectation_pauli": [_P, _U64, C.c_char, _DP],
    "ev_dm_partial_trace_1q": [_P, _U64, _P],
    "ev_dm_run": [C.POINTER(EvCircuit), _P, _U64, C.POINTER(_P), _P],
    "ev_pauli_expectation": [_P, _P, _P, _P, _U64, _P],
    "ev_qasm_parse": [C.c_char_p, _U64, C.POINTER(_P), C.POINTER(_U64), C.POINTER(_U64)],
    "ev_program_circuit": [_P, C.POINTER(EvCircuit)],
    "ev_program_free": [_P],
    "ev_qasm_emit": [C.POINTER(EvCircuit), _P, _U64, C.POINTER(_U64)],
    "ev_server_submit_qasm": [_P, C.c_char_p, _U64, _U64, _U64, _P, C.POINTER(_U64)],
    "ev_prepare": [_P, _P, _P, C.POINTER(_P)],
    "ev_prepared_launch": [_P, _U64, _P],
    "ev_prepared_kernels": [_P, C.POINTER(_U64)],
    "ev_prepared_destroy": [_P],
    "ev_server_create": [_P, C.POINTER(_P)],
    "ev_server_submit": [_P, C.POINTER(EvCircuit), _U64, _U64, _P, C.POINTER(_U64)],
    "ev_server_cancel": [_P, _U64],
    "ev_server_poll": [_P, _P, _I32, C.POINTER(_I32), _I32],
    "ev_server_resume": [_P],
    "ev_server_stats_get": [_P, _P],
    "ev_server_destroy": [_P],
    "ev_probe_fp64": [_DP],
    "ev_marginal_low": [_P, _U64, _DP],
    "ev_softfp_check": [_U64, _U64, C.POINTER(_U64)],
    "ev_softfp_add_check": [_U64, _U64, C.POINTER(_U64)],
    "ev_probe_softadd": [_DP],
    "ev_ff_check": [_U64, _U64, C.POINTER(_U64)],
    "ev_ozaki_gemm_host": [_DP, _U64, _DP, _DP],
    "ev_ozaki_gemm_host_digits": [_DP, _U64, _DP, _DP, _I32],
    "ev_max_abs_diff": [_P, _P, _DP],
    "ev_host_alloc": [_U64, C.POINTER(_P)],
    "ev_host_free": [_P],
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """Loads the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH.name} is not built; run everett_gb300.build.build() first")
            handle = C.CDLL(str(LIB_PATH))
            for name, args in _SIGS.items():
                fn = getattr(handle, name)
                fn.argtypes = args
                fn.restype = C.c_char_p if name in ("ev_last_error", "ev_version") else C.c_int
            _lib = handle
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def last_error() -> str:
    return lib().ev_last_error().decode()


def check(rc: int) -> None:
    """Raises the Python mirror of everett::Error for a non-zero code."""
    if rc == OK:
        return
    from .error import error_for_code
    raise error_for_code(rc, last_error())


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def device_count() -> int:
    n = C.c_int(0)
    check(lib().ev_device_count(C.byref(n)))
    return n.value
