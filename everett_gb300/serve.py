"""Continuous-batching request loop (native, include/everett_cuda.h
ev_server_*) and a Poisson load driver.

Requests are admitted in arrival order while the state memory of admitted
requests stays within the HBM budget; admitted requests run concurrently on
separate streams and small gate-only requests admitted together share one
batched launch.  Mid-circuit measurement and classical control stay on the
device.  A request's result does not depend on what else is in flight.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


class EvServerOptions(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("workers", C.c_int32), ("mode", C.c_int32),
                ("variant", C.c_int32), ("hbm_budget", C.c_uint64), ("batch_small", C.c_int32),
                ("batch_qubits", C.c_int32), ("start_paused", C.c_int32), ("reserved", C.c_int32)]


class EvServerResult(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("num_classical", C.c_int32),
                ("shots", C.c_uint64), ("queue_ms", C.c_double), ("latency_ms", C.c_double),
                ("classical", C.c_uint8 * 64)]


class EvServerStats(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in (
        "submitted", "admitted", "completed", "failed", "refused", "cancelled", "running",
        "pending", "batched_launches", "batched_requests", "reserved_bytes", "budget_bytes")]


@dataclass
class Result:
    id: int
    status: int
    shots: np.ndarray
    classical: list
    queue_ms: float
    latency_ms: float


_MODES = {"exact": N.MODE_EXACT, "tiled": N.MODE_TILED, "fused": N.MODE_FUSED}
_VARIANTS = {"tf32x3": N.FUSED_TF32X3, "bf16x3": N.FUSED_BF16X3, "fp32": N.FUSED_FP32,
             "ozaki": N.FUSED_OZAKI, "ozaki6": N.FUSED_OZAKI6}


class Server:
    def __init__(self, dtype="complex64", workers=8, mode="fused", variant=None,
                 hbm_budget=0, batch_small=True, batch_qubits=0, start_paused=False):
        o = EvServerOptions()
        o.dtype = N.C128 if dtype in ("complex128", "c128") else N.C64
        o.workers = workers
        o.mode = _MODES[mode]
        if variant is None:  # the fused arithmetic of the amplitude type
            variant = "ozaki" if o.dtype == N.C128 else "bf16x3"
        o.variant = _VARIANTS[variant]
        o.hbm_budget = int(hbm_budget)
        o.batch_small = 1 if batch_small else 0
        o.batch_qubits = int(batch_qubits)
        o.start_paused = 1 if start_paused else 0
        self._h = C.c_void_p()
        N.check(N.lib().ev_server_create(C.byref(o), C.byref(self._h)))
        self._buffers = {}
        self._lock = threading.Lock()

    def submit(self, circuit, seed: int = 0, shots: int = 1000) -> int:
        buf = np.zeros(max(1, shots), dtype=np.uint64)
        c = circuit.ev_struct()
        rid = C.c_uint64()
        keep = circuit.to_ev()
        with self._lock:
            N.check(N.lib().ev_server_submit(self._h, C.byref(c), seed, shots, buf.ctypes.data,
                                             C.byref(rid)))
            self._buffers[rid.value] = (buf, shots, keep)
        return rid.value

    def submit_qasm(self, src: str, seed: int = 0, shots: int = 1000) -> int:
        """Submits OpenQASM 3 text; a parse error raises QasmError here."""
        buf = np.zeros(max(1, shots), dtype=np.uint64)
        data = src.encode("utf-8")
        rid = C.c_uint64()
        with self._lock:
            N.check(N.lib().ev_server_submit_qasm(self._h, data, len(data), seed, shots,
                                                  buf.ctypes.data, C.byref(rid)))
            self._buffers[rid.value] = (buf, shots, None)
        return rid.value

    def cancel(self, rid: int) -> None:
        N.check(N.lib().ev_server_cancel(self._h, rid))

    def resume(self) -> None:
        N.check(N.lib().ev_server_resume(self._h))

    def poll(self, max_results: int = 256, wait_ms: int = 0) -> list:
        arr = (EvServerResult * max_results)()
        cnt = C.c_int32()
        N.check(N.lib().ev_server_poll(self._h, arr, max_results, C.byref(cnt), wait_ms))
        out = []
        for i in range(cnt.value):
            r = arr[i]
            with self._lock:
                buf, shots, _ = self._buffers.pop(r.id)
            out.append(Result(r.id, r.status, buf[:shots] if r.status == 0 else buf[:0],
                              [bool(r.classical[j]) for j in range(min(64, r.num_classical))],
                              r.queue_ms, r.latency_ms))
        return out

    def stats(self) -> dict:
        s = EvServerStats()
        N.check(N.lib().ev_server_stats_get(self._h, C.byref(s)))
        return {name: getattr(s, name) for name, _ in EvServerStats._fields_}

    def close(self) -> None:
        if self._h:
            N.lib().ev_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run_all(self, requests, timeout_s: float = 600.0) -> dict:
        """Submits (circuit, seed, shots) requests at once; returns id -> Result."""
        ids = [self.submit(c, seed, shots) for c, seed, shots in requests]
        results = {}
        deadline = time.monotonic() + timeout_s
        while len(results) < len(ids) and time.monotonic() < deadline:
            for r in self.poll(wait_ms=50):
                results[r.id] = r
        return {i: results.get(i) for i in ids}


def poisson_run(server: Server, requests, rate: float, seed: int = 0, timeout_s: float = 600.0):
    """Submits requests at Poisson arrival times (rate per second); returns
    (results in submit order, wall seconds from first arrival to last
    completion)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(requests))
    results = {}
    ids = []
    t0 = time.perf_counter()
    next_t = t0
    for (c, s, shots), gap in zip(requests, gaps):
        next_t += gap
        while True:
            now = time.perf_counter()
            if now >= next_t:
                break
            for r in server.poll(wait_ms=0):
                results[r.id] = r
            time.sleep(min(0.001, next_t - now))
        ids.append(server.submit(c, s, shots))
    deadline = time.monotonic() + timeout_s
    while len(results) < len(ids) and time.monotonic() < deadline:
        for r in server.poll(wait_ms=20):
            results[r.id] = r
    wall = time.perf_counter() - t0
    return [results.get(i) for i in ids], wall


def latency_summary(results, wall: float) -> dict:
    lat = np.array([r.latency_ms for r in results if r is not None and r.status == 0])
    ok = len(lat)
    return {"completed": ok, "failed": sum(1 for r in results if r is None or r.status != 0),
            "circuits_per_s": ok / wall if wall > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if ok else None,
            "p99_ms": float(np.percentile(lat, 99)) if ok else None,
            "mean_ms": float(lat.mean()) if ok else None}
