"""Batched runs: many independent circuits in one persistent launch.

Each circuit runs from |0...0> and reports <Z_0> and full-register shots
drawn like ``State.sample`` with its own seed.  Circuits that fit one CTA
(at most tile_bits qubits) may also measure and apply classically controlled
ops, with the uniforms of their run seed, as ``CudaStateVectorBackend.run_seeded``
does; their classical registers come back with the results.  The tile
size and threads per CTA come from the caller or from the autotuner, which
caches its choice per (amplitude type, qubit-count mix, 2-qubit share).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .circuit import Circuit


class EvBatchCircuit(C.Structure):
    _fields_ = [("circuit", N.EvCircuit), ("seed", C.c_uint64), ("shots", C.c_uint64),
                ("shots_out", C.c_void_p), ("expz_out", C.c_void_p), ("amps_out", C.c_void_p),
                ("run_seed", C.c_uint64), ("classical_out", C.c_void_p)]


class EvBatchOptions(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("tile_bits", C.c_int32), ("threads", C.c_int32),
                ("autotune", C.c_int32), ("test_stall", C.c_int32), ("reserved", C.c_int32)]


class EvBatchStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("host_ms", C.c_double), ("items", C.c_uint64),
                ("launches", C.c_uint64), ("tile_bits", C.c_int32), ("threads", C.c_int32),
                ("from_cache", C.c_int32), ("reserved", C.c_int32)]


@dataclass
class BatchResult:
    expz: float
    shots: np.ndarray
    amplitudes: np.ndarray | None = None
    classical: list | None = None


def run_batch(circuits, seeds=None, shots=1000, dtype="complex64", tile_bits=0, threads=0,
              autotune=False, return_states=False, test_stall=False, run_seeds=None):
    """Runs ``circuits`` in one batch; returns (results, stats dict).
    ``seeds`` seed the shot streams, ``run_seeds`` (default 0, as ``run``)
    the mid-circuit measurements."""
    count = len(circuits)
    seeds = list(range(count)) if seeds is None else list(seeds)
    run_seeds = [0] * count if run_seeds is None else list(run_seeds)
    shots = [shots] * count if isinstance(shots, int) else list(shots)
    items = (EvBatchCircuit * max(1, count))()
    keep = []
    results = []
    for i, c in enumerate(circuits):
        it = items[i]
        it.circuit = c.ev_struct()
        keep.append(c.to_ev())
        it.seed = seeds[i]
        it.shots = shots[i]
        sh = np.zeros(max(1, shots[i]), dtype=np.uint64)
        ez = np.zeros(1, dtype=np.float64)
        am = np.zeros(2 << c.num_qubits(), dtype=np.float64) if return_states else None
        it.shots_out = sh.ctypes.data
        it.expz_out = ez.ctypes.data
        it.amps_out = am.ctypes.data if am is not None else None
        it.run_seed = run_seeds[i]
        cl = np.zeros(max(1, c.num_classical()), dtype=np.uint8)
        it.classical_out = cl.ctypes.data
        results.append((sh, ez, am, cl))
    opts = EvBatchOptions(N.C128 if dtype in ("complex128", "c128") else N.C64, int(tile_bits),
                          int(threads), 1 if autotune else 0, 1 if test_stall else 0, 0)
    st = EvBatchStats()
    N.check(N.lib().ev_batch_run(items, count, C.byref(opts), C.byref(st)))
    out = [BatchResult(float(ez[0]), sh[:shots[i]],
                       am.view(np.complex128) if am is not None else None,
                       [bool(b) for b in cl[:circuits[i].num_classical()]])
           for i, (sh, ez, am, cl) in enumerate(results)]
    stats = {"device_ms": st.device_ms, "host_ms": st.host_ms, "items": st.items,
             "launches": st.launches, "tile_bits": st.tile_bits, "threads": st.threads,
             "from_cache": bool(st.from_cache)}
    return out, stats
