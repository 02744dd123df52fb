#!/usr/bin/env python3
"""Benchmark: gate-pass throughput of the statevector engine on one GB300.

Workload: the seeded random-layer circuit at 30 qubits, depth 20 (1800
single-qubit rotations Rz-Ry-Rz on every qubit per layer, 290 CNOTs in
alternating bricks) on the plain complex128 path, state resident in HBM.
A step is one full run of the circuit from |0...0>.

value   = sum over ops of the algorithmic bytes 2 * N_t * 16 (the bytes a
          gate-by-gate run must move) / device time of the step, in GB/s
e2e     = the same bytes / host wall time of a step through the C ABI:
          op records copied in from pinned host memory, run, and the full
          final state copied back to pinned host memory
roofline: the shared-memory tile pass (the dominant kernel), its algorithmic
          bytes per launch (one read and one write of the 2^n amplitudes)
          over its live event-timed launch duration, against the measured HBM
          copy bandwidth
cpu_baseline: the CPU oracle (the reference's scalar loops restated in C++,
          one core) on a bounded prefix of the same circuit family at 24
          qubits, same unit
--impl reference: the same oracle with its independent loops split over
          every host core, each step a bounded prefix at 26 qubits.

With torchrun (N>1) every rank runs an independent replica on its own GPU
(the path does not shard); value is the sum over ranks' work over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30q gate GB/s (% HBM peak); batched circuits/s + p99 at fidelity>=1-1e-6 vs FP64"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=20)
    ap.add_argument("--mode", default="tiled", choices=["tiled", "exact"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


class Dist:
    """Barrier and max-over-ranks for replica runs (gloo on the host)."""

    def __init__(self):
        self.rank = int(os.environ.get("RANK", 0))
        self.world = int(os.environ.get("WORLD_SIZE", 1))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """DRAM bytes per launch from a committed ncu summary, if one exists."""
    p = ROOT / "profiles" / f"{kernel}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_size:"):
            return float(line.split(":", 1)[1])
    return None


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v == "Active"})
        loaded = [r[0] for r in rows if r[0] > 0.5 * r[1]] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def cpu_oracle_rate(n: int, depth: int, seconds: float, parallel: bool):
    """GB/s of the CPU oracle over a prefix of the random-layer circuit."""
    import numpy as np

    import oracle as O
    from everett_gb300 import workloads
    c = workloads.random_layers(n, depth, seed=1)
    amps = np.zeros(1 << n, dtype=np.complex128)
    amps[0] = 1
    ops = c.ops()
    done = 0
    nbytes = 0
    t0 = time.perf_counter()
    # per-op calls through the run loop of the oracle (ops [done, done+1))
    while done < len(ops) and time.perf_counter() - t0 < seconds:
        O.apply_ops(c, amps, done, done + 1, parallel=parallel)
        nbytes += workloads.op_bytes(ops[done], n, 16)
        done += 1
    dt = time.perf_counter() - t0
    return nbytes / dt / 1e9, done, dt


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    cores = os.cpu_count() or 1
    n = min(args.qubits, 26)
    steps = []
    for i in range(args.warmup + args.steps):
        rate, ops_done, dt = cpu_oracle_rate(n, args.depth, 6.0, parallel=True)
        if i >= args.warmup:
            steps.append((rate, ops_done, dt))
    rate = statistics.median(s[0] for s in steps)
    ms = statistics.median(s[2] for s in steps) * 1000
    line = {
        "impl": "reference", "metric": METRIC, "value": round(rate, 3), "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random-layer circuit)",
        "config": {"workload": f"random-layer circuit, {n} qubits (bounded prefix per step), "
                               f"depth {args.depth}, complex128",
                   "parallelism": "replicas only", "l2": "CPU run"},
        "cpu_baseline": {"value": round(rate, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"{steps[0][1]} ops of the {n}-qubit circuit per step, "
                                   f"oracle restatement of the reference's scalar loops, "
                                   f"OpenMP over independent pairs"},
        "e2e": {"value": round(rate, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, dist: Dist):
    import ctypes as C

    import numpy as np

    from everett_gb300 import CudaStateVectorBackend, State, _native, build, workloads
    build.build()
    L = _native.lib()
    n, depth = args.qubits, args.depth
    circuit = workloads.random_layers(n, depth, seed=1)
    bytes_per_step = workloads.gate_bytes(circuit, 16)
    state = State.zero(n, "complex128")
    h = state.handle

    def step():
        CudaStateVectorBackend.run_into(state, circuit, 0, mode=args.mode)

    for _ in range(args.warmup):
        step()
    state.synchronize()
    dist.barrier()
    lc0 = C.c_uint64()
    L.ev_state_launch_count(h, C.byref(lc0))
    _native.check(L.ev_state_profile(h, 1))
    gpu_index = int(os.environ.get("LOCAL_RANK", 0))
    with Clocks(gpu_index if dist.world == 1 else 0) as clk:
        _native.check(L.ev_state_record_event(h, 0))
        for _ in range(args.steps):
            step()
        _native.check(L.ev_state_record_event(h, 1))
        ms = C.c_float()
        _native.check(L.ev_state_elapsed_ms(h, 0, 1, C.byref(ms)))
    total_ms = ms.value
    lc1 = C.c_uint64()
    L.ev_state_launch_count(h, C.byref(lc1))
    prof = read_profile(L, h)
    _native.check(L.ev_state_profile(h, 0))
    dist.barrier()
    worst_ms = dist.max(total_ms)
    value = dist.world * bytes_per_step * args.steps / (worst_ms / 1000) / 1e9

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        ops, ctrl, npool = circuit.to_ev()
        pinned_ops = C.c_void_p()
        _native.check(L.ev_host_alloc(ops.nbytes, C.byref(pinned_ops)))
        out = C.c_void_p()
        out_bytes = (1 << n) * 16
        _native.check(L.ev_host_alloc(out_bytes, C.byref(out)))
        C.memmove(pinned_ops, ops.ctypes.data, ops.nbytes)
        circ = _native.EvCircuit(n, 0, pinned_ops.value, len(ops), ctrl.ctypes.data, npool)
        opts = _native.EvRunOptions(_native.C128, 1 if args.mode == "tiled" else 0, 0, 0)
        cl = np.zeros(1, dtype=np.uint8)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            _native.check(L.ev_state_run(h, C.byref(circ), 0, C.byref(opts), cl.ctypes.data))
            _native.check(L.ev_state_download(h, out, 1 << n))
        e2e_s = time.perf_counter() - t0
        e2e_s = dist.max(e2e_s)
        L.ev_host_free(pinned_ops)
        L.ev_host_free(out)
        e2e = {"value": round(dist.world * bytes_per_step * args.steps / e2e_s / 1e9, 2),
               "unit": "GB/s", "h2d_bytes_per_step": int(ops.nbytes),
               "d2h_bytes_per_step": int(out_bytes)}

    peak, peak_kind = measured_peaks()
    tile = prof.get("tile_pass")
    roofline = None
    if tile and tile["launches"]:
        per_launch_bytes = 2.0 * (1 << n) * 16
        avg_ms = tile["ms"] / tile["launches"]
        achieved = per_launch_bytes / (avg_ms / 1000) / 1e9
        roofline = {"kernel": "k_tile<double2> (shared-memory tile pass, complex128)",
                    "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                    "unit": "GB/s", "frac": round(achieved / peak, 4),
                    "peak_source": f"{peak_kind} hbm_gbs",
                    "traffic": ncu_traffic("k_tile_c128"),
                    "launches": tile["launches"], "avg_launch_ms": round(avg_ms, 3),
                    "algorithmic_bytes_per_launch": per_launch_bytes}

    cpu = None
    if dist.rank == 0:
        rate, ops_done, dt = cpu_oracle_rate(min(n, 24), depth, args.cpu_seconds, parallel=False)
        cpu = {"value": round(rate, 3), "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": f"first {ops_done} ops of the random-layer circuit at {min(n, 24)} "
                         f"qubits, {dt:.1f} s, scalar oracle (the reference's loops)"}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(worst_ms / args.steps, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-layer circuit)",
            "config": {"workload": f"random-layer circuit, {n} qubits, depth {depth}, "
                                   f"complex128, {args.mode} mode",
                       "ops": len(circuit), "algorithmic_bytes_per_step": bytes_per_step,
                       "parallelism": "replicas only" if dist.world > 1 else "1 GPU",
                       "l2": f"inputs larger than L2 ({(1 << n) * 16 / 2**30:.1f} GiB state), "
                             f"no flush"},
            "pct_hbm_peak": round(100 * value / peak, 1),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(lc1.value - lc0.value),
            "clocks": clk.summary(),
            "kernel_profile": prof,
        }
        print(json.dumps(line), flush=True)


def read_profile(L, h):
    import ctypes as C

    class Stat(C.Structure):
        _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("ms", C.c_double),
                    ("bytes", C.c_double)]
    arr = (Stat * 16)()
    cnt = C.c_int32()
    L.ev_state_profile_read(h, arr, 16, C.byref(cnt))
    out = {}
    for i in range(min(cnt.value, 16)):
        s = arr[i]
        out[s.name.decode()] = {"launches": int(s.launches), "ms": round(s.ms, 3),
                                "bytes": s.bytes}
    return out


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
