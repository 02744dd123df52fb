"""Python handle on the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/libev_oracle.so (scalar, matching the reference's
single-threaded loops) or libev_oracle_omp.so (the same source with its
independent loops split over host threads; bit-identical results).  Only the
tests, the smoke check and the benchmark's CPU-baseline leg use this module;
the engine never does.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_libs: dict = {}


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def lib(parallel: bool = False) -> C.CDLL:
    name = "libev_oracle_omp.so" if parallel else "libev_oracle.so"
    if name in _libs:
        return _libs[name]
    path = HERE / name
    if not path.exists():
        build()
    h = C.CDLL(str(path))
    P, U = C.c_void_p, C.c_uint64
    sig = {
        "oracle_gate_h": ([P], None),
        "oracle_gate_rx": ([C.c_double, P], None),
        "oracle_gate_ry": ([C.c_double, P], None),
        "oracle_gate_rz": ([C.c_double, P], None),
        "oracle_gate_phase": ([C.c_double, P], None),
        "oracle_apply_1q": ([P, U, U, P], None),
        "oracle_apply_2q": ([P, U, U, U, P], None),
        "oracle_apply_2q_dense": ([P, U, U, U, P], None),
        "oracle_apply_controlled_1q": ([P, U, P, U, U, P], None),
        "oracle_measure_qubit": ([P, U, U, C.c_double], C.c_int),
        "oracle_norm_sqr": ([P, U], C.c_double),
        "oracle_normalize": ([P, U], None),
        "oracle_overlap": ([P, P, U, P], None),
        "oracle_bloch_vector": ([P, U, U, P], None),
        "oracle_marginal_low": ([P, U, U, P], None),
        "oracle_pauli_expectation": ([P, U, U, U, C.c_int], C.c_double),
        "oracle_dm_run": ([P, P, U, P, P], C.c_int),
        "oracle_dm_from_amplitudes": ([P, U, P], None),
        "oracle_dm_observables": ([P, U, U, P], None),
        "oracle_stab_run": ([P, U, P, P, P, P], C.c_int),
        "oracle_rng_u64": ([U, U, P], None),
        "oracle_rng_f64": ([U, U, P], None),
        "oracle_rng_raw": ([P, U, P], None),
        "oracle_rng_seed_words": ([U, P], None),
        "oracle_validate": ([P], C.c_int),
        "oracle_run_seeded": ([P, U, P, P], C.c_int),
        "oracle_apply_ops": ([P, U, U, P], None),
        "oracle_sample_literal": ([P, U, U, U, P], None),
        "oracle_sample_tree": ([P, U, U, U, P], None),
    }
    for fn, (args, res) in sig.items():
        f = getattr(h, fn)
        f.argtypes = args
        f.restype = res
    _libs[name] = h
    return h


def _m(gate) -> np.ndarray:
    return np.ascontiguousarray(gate.as_f64())


def apply_1q(amps: np.ndarray, k: int, gate) -> None:
    m = _m(gate)
    lib().oracle_apply_1q(amps.ctypes.data, amps.shape[0], k, m.ctypes.data)


def apply_2q(amps: np.ndarray, a: int, b: int, gate) -> None:
    m = _m(gate)
    lib().oracle_apply_2q(amps.ctypes.data, amps.shape[0], a, b, m.ctypes.data)


def apply_2q_dense(amps: np.ndarray, a: int, b: int, gate) -> None:
    m = _m(gate)
    lib().oracle_apply_2q_dense(amps.ctypes.data, amps.shape[0], a, b, m.ctypes.data)


def apply_controlled_1q(amps: np.ndarray, controls, target: int, gate) -> None:
    m = _m(gate)
    cs = np.array(list(controls) or [0], dtype=np.uint64)
    lib().oracle_apply_controlled_1q(amps.ctypes.data, amps.shape[0], cs.ctypes.data,
                                     len(controls), target, m.ctypes.data)


def measure_qubit(amps: np.ndarray, k: int, u: float) -> bool:
    return bool(lib().oracle_measure_qubit(amps.ctypes.data, amps.shape[0], k, u))


def norm_sqr(amps: np.ndarray) -> float:
    return lib().oracle_norm_sqr(amps.ctypes.data, amps.shape[0])


def normalize(amps: np.ndarray) -> None:
    lib().oracle_normalize(amps.ctypes.data, amps.shape[0])


def overlap(a: np.ndarray, b: np.ndarray) -> complex:
    out = np.zeros(2)
    lib().oracle_overlap(a.ctypes.data, b.ctypes.data, a.shape[0], out.ctypes.data)
    return complex(out[0], out[1])


def bloch_vector(amps: np.ndarray, q: int) -> list:
    out = np.zeros(3)
    lib().oracle_bloch_vector(amps.ctypes.data, amps.shape[0], q, out.ctypes.data)
    return out.tolist()


def marginal_low(amps: np.ndarray, m: int) -> np.ndarray:
    out = np.zeros(1 << m)
    lib().oracle_marginal_low(amps.ctypes.data, amps.shape[0], m, out.ctypes.data)
    return out


def most_probable_phase(amps: np.ndarray, m: int) -> float:
    """phase_estimation.rs:97-121: the LAST index among equal maxima (Rust's
    Iterator::max_by keeps the later of two equal elements)."""
    marg = marginal_low(amps, m)
    best = 0
    for i in range(1, marg.shape[0]):
        if not marg[i] < marg[best]:
            best = i
    return best / float(1 << m)


def pauli_expectation(amps: np.ndarray, x_mask: int, z_mask: int, negative: bool = False) -> float:
    n = amps.shape[0].bit_length() - 1
    return lib().oracle_pauli_expectation(amps.ctypes.data, n, x_mask, z_mask, int(negative))


def dm_run(circuit, noise=None, seed: int = 0):
    """DensityMatrixBackend::run_with_noise_seeded: (rho [dim x dim], classical)."""
    import ctypes as C_
    c = circuit.ev_struct()
    n = circuit.num_qubits()
    dim = 1 << n
    rho = np.zeros((dim, dim), dtype=np.complex128)
    cl = np.zeros(max(1, circuit.num_classical()), dtype=np.uint8)
    nz = C_.byref(noise) if noise is not None else None
    rc = lib().oracle_dm_run(C_.addressof(c), nz, seed, rho.ctypes.data, cl.ctypes.data)
    if rc:
        raise ValueError(f"oracle validation error {rc}")
    return rho, [bool(b) for b in cl[:circuit.num_classical()]]


def dm_from_amplitudes(amps: np.ndarray) -> np.ndarray:
    dim = amps.shape[0]
    rho = np.zeros((dim, dim), dtype=np.complex128)
    lib().oracle_dm_from_amplitudes(np.ascontiguousarray(amps).ctypes.data, dim, rho.ctypes.data)
    return rho


def dm_observables(rho: np.ndarray, qubit: int) -> dict:
    """trace, purity, <I>, <X>, <Y>, <Z> on qubit, and its reduced 2x2 matrix."""
    n = rho.shape[0].bit_length() - 1
    out = np.zeros(14)
    lib().oracle_dm_observables(np.ascontiguousarray(rho).ctypes.data, n, qubit, out.ctypes.data)
    red = out[6:14].view(np.complex128)
    return {"trace": out[0], "purity": out[1], "I": out[2], "X": out[3], "Y": out[4],
            "Z": out[5], "reduced": red.copy()}


def stab_run(circuit, seed: int = 0):
    """StabilizerBackend::run_seeded: (x [n x n], z [n x n], neg [n], classical),
    or the error code (EV_ERR_NON_CLIFFORD = 5) as an int."""
    import ctypes as C_
    c = circuit.ev_struct()
    n = circuit.num_qubits()
    x = np.zeros((max(1, n), max(1, n)), dtype=np.uint8)
    z = np.zeros_like(x)
    neg = np.zeros(max(1, n), dtype=np.uint8)
    cl = np.zeros(max(1, circuit.num_classical()), dtype=np.uint8)
    rc = lib().oracle_stab_run(C_.addressof(c), seed, x.ctypes.data, z.ctypes.data,
                               neg.ctypes.data, cl.ctypes.data)
    if rc:
        return rc
    return x[:n, :n], z[:n, :n], neg[:n], [bool(b) for b in cl[:circuit.num_classical()]]


def rng_u64(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=np.uint64)
    lib().oracle_rng_u64(seed, count, out.ctypes.data)
    return out


def rng_f64(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=np.float64)
    lib().oracle_rng_f64(seed, count, out.ctypes.data)
    return out


def rng_raw(state, count: int) -> np.ndarray:
    """xoshiro256++ outputs from a raw 4-word state (no seeding)."""
    st = np.array(state, dtype=np.uint64)
    out = np.zeros(count, dtype=np.uint64)
    lib().oracle_rng_raw(st.ctypes.data, count, out.ctypes.data)
    return out


def rng_seed_words(seed: int) -> np.ndarray:
    """The 4 state words Rng::seed_from_u64(seed) derives with SplitMix64."""
    out = np.zeros(4, dtype=np.uint64)
    lib().oracle_rng_seed_words(seed, out.ctypes.data)
    return out


def validate(circuit) -> int:
    c = circuit.ev_struct()
    return lib().oracle_validate(C.byref(c))


def run_seeded(circuit, seed: int = 0, parallel: bool = False):
    """(amplitudes, classical bits, code) of StateVectorBackend::run_seeded."""
    c = circuit.ev_struct()
    amps = np.zeros(1 << circuit.num_qubits(), dtype=np.complex128)
    cl = np.zeros(max(1, circuit.num_classical()), dtype=np.uint8)
    rc = lib(parallel).oracle_run_seeded(C.byref(c), seed, amps.ctypes.data, cl.ctypes.data)
    return amps, [bool(b) for b in cl[: circuit.num_classical()]], rc


def apply_ops(circuit, amps: np.ndarray, first: int, last: int, parallel: bool = False) -> None:
    c = circuit.ev_struct()
    lib(parallel).oracle_apply_ops(C.byref(c), first, last, amps.ctypes.data)


def sample_literal(amps: np.ndarray, seed: int, shots: int) -> np.ndarray:
    n = amps.shape[0].bit_length() - 1
    out = np.zeros(shots, dtype=np.uint64)
    lib().oracle_sample_literal(amps.ctypes.data, n, seed, shots, out.ctypes.data)
    return out


def sample_tree(amps: np.ndarray, seed: int, shots: int) -> np.ndarray:
    n = amps.shape[0].bit_length() - 1
    out = np.zeros(shots, dtype=np.uint64)
    lib().oracle_sample_tree(amps.ctypes.data, n, seed, shots, out.ctypes.data)
    return out


def sample_state(n: int) -> np.ndarray:
    """The reference's deterministic test fixture (kernel.rs:631-635):
    amp_j = (0.1 + 0.03 j) + (-0.2 + 0.017 j) i."""
    j = np.arange(1 << n, dtype=np.float64)
    return (0.1 + j * 0.03) + 1j * (-0.2 + j * 0.017)
