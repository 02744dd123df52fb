#!/usr/bin/env python3
"""Benchmark of the statevector engine on one GB300.

Headline (value): the seeded random-layer circuit at 30 qubits, depth 20
(Rz-Ry-Rz on every qubit per layer, CNOT bricks; 1800 rotations, 290
CNOTs) on the plain complex128 path (tiled mode: bit-identical to the
reference's arithmetic), state resident in HBM.  A step is one full run of
the circuit from |0...0>.

  value         sum over ops of the algorithmic bytes 2 * N_t * 16 (what a
                gate-by-gate run must move) / device time of a step, GB/s
  e2e           the same bytes / host wall time of a step through the C ABI:
                op records copied in from pinned host memory, the run, and
                the full final state copied back to pinned host memory
  roofline      the shared-memory tile pass (dominant kernel): one read and
                one write of the 2^n amplitudes per launch over its live
                event-timed launch duration, against the measured HBM copy
                bandwidth (the pass is bound by the FP64 pipe instead; the
                committed ncu summary gives its FP64 utilisation)
  cpu_baseline  the CPU oracle (the reference's scalar loops restated in
                C++) on one host core over the first ops of the same
                30-qubit circuit, same unit
  gate_bytes_pct_of_hbm_peak   value over the measured HBM copy bandwidth:
                the gate-by-gate bytes the tile passes stand for, not traffic
  hbm_traffic_pct_of_peak      the bytes HBM actually moves (the tile
                passes' ncu DRAM traffic per launch x launches) per second,
                over the same peak

Additional measured sections (same run, rank 0): the complex64 fused
tensor-core path on the same 30-qubit circuit (time, speed-up over
complex128, fidelity against the complex128 state), the 30-qubit QFT,
the 28-qubit Haar/CZ depth-40 circuit per fused arithmetic, the 4096-circuit
TFIM batch, and the serving mix under Poisson arrivals.

--impl reference times the same oracle with its independent loops split over
every host core on the same 30-qubit circuit, each step ~4 s of ops resuming
where the previous step stopped.

Under torchrun (N>1) every rank runs an independent replica on its own GPU
(the path does not shard); value is the ranks' summed work over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import contextlib
import ctypes as C
import json
import math
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
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=20)
    ap.add_argument("--mode", default="tiled", choices=["tiled", "exact"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--batch-count", type=int, default=4096,
                    help="circuits of the TFIM batch for --case batch (4096: the workload)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-clocks", action="store_true",
                    help="sample nvidia-smi clocks during the end-to-end steps too")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--kernel-reps", type=int, default=3,
                    help="timed calls per case for --case kernels (0: one untimed call each)")
    ap.add_argument("--fuse-bits", type=int, default=5,
                    help="qubits per fused unitary for --case fused (5 or 6)")
    ap.add_argument("--case", default="headline",
                    choices=["headline", "fused", "tiled64", "batch", "serve", "serve_small",
                             "prepared", "kernels", "density", "stabilizer"],
                    help="run one section alone (for profiling): the complex64 fused or tiled "
                         "path on the random-layer circuit, the TFIM batch, the serving mix, "
                         "prepared-graph replay, or each streaming kernel class alone")
    ap.add_argument("--variant", default="bf16x3",
                    choices=["bf16x3", "tf32x3", "fp32", "ozaki", "ozaki6"],
                    help="fused arithmetic for --case fused (ozaki, ozaki6: the complex128 ones)")
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


def bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["bf16_tflops"]), "measured bf16_tflops (burst)"
    return 1900.0, "fallback"


def ncu_figure(name: str, key: str):
    """A number from a committed ncu summary (profiles/<name>.txt)."""
    p = ROOT / "profiles" / f"{name}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(key + ":"):
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


class OracleWindow:
    """The CPU oracle (the reference's scalar loops restated in C++) walking
    the random-layer circuit op by op on a host state; each step resumes where
    the previous one stopped, from |0...0> again after the circuit's last op.
    Only op application is timed."""

    def __init__(self, n: int, depth: int, parallel: bool):
        import numpy as np

        from everett_gb300 import workloads
        self.n, self.parallel = n, parallel
        self.circuit = workloads.random_layers(n, depth, seed=1)
        self.ops = self.circuit.ops()
        self.amps = np.zeros(1 << n, dtype=np.complex128)
        self.amps.fill(0)  # touch every page before any op is timed
        self.amps[0] = 1
        self.pos = 0

    def step(self, seconds: float):
        """Applies ops for about `seconds`; returns (GB/s, ops, seconds)."""
        import oracle as O
        from everett_gb300 import workloads
        nbytes = done = 0
        busy = 0.0
        while busy < seconds:
            if self.pos == len(self.ops):
                self.amps[:] = 0
                self.amps[0] = 1
                self.pos = 0
            t0 = time.perf_counter()
            O.apply_ops(self.circuit, self.amps, self.pos, self.pos + 1, parallel=self.parallel)
            busy += time.perf_counter() - t0
            nbytes += workloads.op_bytes(self.ops[self.pos], self.n, 16)
            self.pos += 1
            done += 1
        return nbytes / busy / 1e9, done, busy


def workload_name(n: int, depth: int) -> str:
    return f"random-layer circuit, {n} qubits, depth {depth}, complex128"


def oracle_window(n: int, depth: int, parallel: bool):
    """An OracleWindow at n qubits, or at 26 when the host cannot hold the
    2^n-amplitude state (the fallback is named in the line)."""
    try:
        return OracleWindow(n, depth, parallel)
    except MemoryError:
        return OracleWindow(min(n, 26), depth, parallel)


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    cores = os.cpu_count() or 1
    win = oracle_window(args.qubits, args.depth, parallel=True)
    n = win.n
    seconds = 4.0
    timed = []
    for i in range(args.warmup + args.steps):
        res = win.step(seconds)
        if i >= args.warmup:
            timed.append(res)
    gbytes = sum(r[0] * r[2] for r in timed)
    busy = sum(r[2] for r in timed)
    rate = gbytes / busy
    ops = sum(r[1] for r in timed)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(rate, 3), "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * busy / len(timed), 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-layer circuit)",
        "config": {"workload": workload_name(n, args.depth), "parallelism": "replicas only",
                   "l2": "CPU run"},
        "cpu_baseline": {"value": round(rate, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"{ops} ops of the {n}-qubit circuit over {len(timed)} steps of "
                                   f"~{seconds:.0f} s, each resuming where the last stopped; "
                                   f"oracle restatement of the reference's scalar loops, OpenMP "
                                   f"over independent pairs"},
        "e2e": {"value": round(rate, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class Stat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("ms", C.c_double),
                ("bytes", C.c_double)]


def read_profile(L, h):
    arr = (Stat * 16)()
    cnt = C.c_int32()
    L.ev_state_profile_read(h, arr, 16, C.byref(cnt))
    out = {}
    for i in range(min(cnt.value, 16)):
        s = arr[i]
        out[s.name.decode()] = {"launches": int(s.launches), "ms": round(s.ms, 3),
                                "bytes": s.bytes}
    return out


def timed_runs(L, N, state, circuit, reps, **kw):
    """Device ms per run (events on the state's stream) and the per-kernel
    profile of the timed runs."""
    from everett_gb300 import CudaStateVectorBackend
    h = state.handle
    N.check(L.ev_state_profile(h, 1))
    N.check(L.ev_state_record_event(h, 0))
    for _ in range(reps):
        CudaStateVectorBackend.run_into(state, circuit, 0, **kw)
    N.check(L.ev_state_record_event(h, 1))
    ms = C.c_float()
    N.check(L.ev_state_elapsed_ms(h, 0, 1, C.byref(ms)))
    prof = read_profile(L, h)
    N.check(L.ev_state_profile(h, 0))
    return ms.value / reps, prof


def fidelity(a, b) -> float:
    ov = a.overlap(b)
    return abs(ov) ** 2 / (a.norm_sqr() * b.norm_sqr())


def roofline_of(prof, name, per_launch_bytes, peak, peak_kind, kernel, traffic):
    k = prof.get(name)
    if not k or not k["launches"]:
        return None
    avg_ms = k["ms"] / k["launches"]
    achieved = per_launch_bytes / (avg_ms / 1000) / 1e9
    return {"kernel": kernel, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
            "traffic": traffic, "launches": k["launches"], "avg_launch_ms": round(avg_ms, 3),
            "algorithmic_bytes_per_launch": per_launch_bytes}


def extras_c64(L, N, ref_state, circuit, c128_ms, bytes_per_step, peak, peak_kind):
    from everett_gb300 import State
    n = circuit.num_qubits()
    st = State.zero(n, "complex64")
    out = {}
    for variant in ("bf16x3", "tf32x3"):
        kw = dict(mode="fused", variant=variant, tile_bits=5)
        timed_runs(L, N, st, circuit, 1, **kw)
        ms, prof = timed_runs(L, N, st, circuit, 3, **kw)
        roof = roofline_of(prof, "fused_unitary", 2.0 * (1 << n) * 8, peak, peak_kind,
                           f"k_fused_tc<5,{variant}> (fused 5-qubit unitary, tcgen05)",
                           ncu_figure(f"k_fused_tc_{variant}", "traffic_bytes_per_launch_full_size"))
        if roof:
            # 3 split products of a 64 x 64 real GEMM per row of 32 amplitudes:
            # 3 * 2 * 64 * 64 / 32 = 768 flops per amplitude (TF32 runs at half
            # the BF16 rate, so its fraction is against half the BF16 peak)
            flops = 768.0 * (1 << n)
            tf = flops / (roof["avg_launch_ms"] / 1e3) / 1e12
            bf = bf16_peak()
            pk = bf[0] if variant == "bf16x3" else bf[0] / 2
            roof["tensor"] = {"achieved_tflops": round(tf, 1), "peak_tflops": round(pk, 1),
                              "frac": round(tf / pk, 4), "peak_source": bf[1] +
                              ("" if variant == "bf16x3" else ", halved for TF32"),
                              "flops_per_launch": flops}
        out[variant] = {
            "ms_per_run": round(ms, 2), "speedup_vs_complex128": round(c128_ms / ms, 1),
            "gate_GBps_complex128_equivalent": round(bytes_per_step / (ms / 1e3) / 1e9, 1),
            "fidelity_vs_complex128": fidelity(ref_state, st),
            "max_abs_err_vs_complex128": ref_state.max_abs_diff(st),
            "amplitude_updates_per_s": float(f"{len(circuit) * (1 << n) / (ms / 1e3):.4g}"),
            "roofline": roof}
    del st
    return out


def extras_c128_fused(L, N, ref_state, circuit, c128_ms, bytes_per_step, peak, peak_kind,
                      variant="ozaki"):
    """The same circuit through the complex128 fused path: 5-qubit unitaries
    on the FP16 tensor cores with 8-bit digit slicing (seven digits, or six
    with variant "ozaki6"), against the bit-exact tiled complex128 result."""
    from everett_gb300 import State
    n = circuit.num_qubits()
    nd = 6 if variant == "ozaki6" else 7
    st = State.zero(n, "complex128")
    kw = dict(mode="fused", variant=variant)
    timed_runs(L, N, st, circuit, 1, **kw)
    ms, prof = timed_runs(L, N, st, circuit, 2, **kw)
    ov = ref_state.overlap(st)
    roof = roofline_of(prof, "fused_unitary", 2.0 * (1 << n) * 16, peak, peak_kind,
                       "k_fused_oz (fused 5-qubit unitary, complex128 by digit slicing, tcgen05)",
                       ncu_figure("k_fused_oz_c128", "traffic_bytes_per_launch_full_size"))
    if roof:
        # digit-pair MMAs per launch: 2^n / 4096 steps x 2 halves x
        # nd(nd+1)/2 pairs x 4 K-steps of 2 x 128 x 32 x 16 flops -- 7168
        # flops per amplitude with seven digits, 5376 with six
        flops = 128.0 * nd * (nd + 1) * (1 << n)
        tf = flops / (roof["avg_launch_ms"] / 1e3) / 1e12
        bf = bf16_peak()
        roof["tensor"] = {"achieved_tflops": round(tf, 1), "peak_tflops": bf[0],
                          "frac": round(tf / bf[0], 4), "peak_source": bf[1],
                          "flops_per_launch": flops}
    out = {"workload": f"random-layer circuit, {n} qubits, depth 20, complex128 fused "
                       f"({variant}: {nd} 8-bit FP16 digits per f64, exact f32 digit-pair sums, "
                       f"int64 recombination)",
           "ms_per_run": round(ms, 2), "speedup_vs_complex128_tiled": round(c128_ms / ms, 2),
           "gate_GBps": round(bytes_per_step / (ms / 1e3) / 1e9, 1),
           "max_abs_err_vs_complex128_bit_exact": ref_state.max_abs_diff(st),
           "fidelity_vs_complex128_bit_exact": abs(ov) ** 2,
           "amplitude_updates_per_s": float(f"{len(circuit) * (1 << n) / (ms / 1e3):.4g}"),
           "passes": prof.get("fused_unitary", {}).get("launches", 0) // 2,
           "roofline": roof}
    del st
    return out


def extras_cfg0(L, N):
    """The 20-qubit depth-20 random-layer circuit with 10000 full-register
    shots: the GPU paths (circuit and shots timed on the device) beside the
    scalar oracle of the reference's loops on one host core (a CPU baseline
    leg: the whole circuit and the same shots)."""
    import numpy as np

    import oracle as O
    from everett_gb300 import State, workloads
    n, depth, shots = 20, 20, 10000
    c = workloads.random_layers(n, depth, seed=1)
    t0 = time.perf_counter()
    want, _, _ = O.run_seeded(c, 0)
    cpu_shots = O.sample_tree(want, 7, shots)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    out = {"workload": f"random-layer circuit, {n} qubits, depth {depth} ({len(c)} ops), "
                       f"complex128, then {shots} full-register shots",
           "cpu_oracle_1_core_ms": round(cpu_ms, 1)}
    for name, kw in (("tiled", dict(mode="tiled")),
                     ("fused_ozaki", dict(mode="fused", variant="ozaki"))):
        st = State.zero(n, "complex128")
        from everett_gb300 import CudaStateVectorBackend
        CudaStateVectorBackend.run_into(st, c, 0, **kw)
        st.sample(shots, seed=7)
        h = st.handle
        reps = 5
        N.check(L.ev_state_record_event(h, 0))
        for _ in range(reps):
            CudaStateVectorBackend.run_into(st, c, 0, **kw)
            got_shots = st.sample(shots, seed=7)
        N.check(L.ev_state_record_event(h, 1))
        ms = C.c_float()
        N.check(L.ev_state_elapsed_ms(h, 0, 1, C.byref(ms)))
        err = float(np.max(np.abs(st.amplitudes() - want)))
        out[name] = {"ms_per_run_with_shots": round(ms.value / reps, 3),
                     "speedup_vs_cpu_oracle_1_core": round(cpu_ms / (ms.value / reps), 1),
                     "max_abs_err_vs_oracle": err,
                     "shots_equal_oracle": bool(np.array_equal(got_shots, cpu_shots))}
        del st
    return out


def extras_qft(L, N, n, peak):
    import numpy as np

    from everett_gb300 import State, workloads
    j = 0x2A5A5A5A & ((1 << n) - 1)
    c = workloads.qft_on_basis(n, j)
    st = State.zero(n, "complex128")
    timed_runs(L, N, st, c, 1, mode="tiled")
    ms, prof = timed_runs(L, N, st, c, 2, mode="tiled")
    rng = np.random.default_rng(1)
    idx = rng.integers(0, 1 << n, size=2048)
    err = 0.0
    for k in idx:
        k = int(k)
        ph = (j * k) & ((1 << n) - 1)
        ang = math.tau * ph / float(1 << n)
        want = complex(math.cos(ang), math.sin(ang)) / math.sqrt(1 << n)
        err = max(err, abs(st.amplitude(k) - want))
    gb = workloads.gate_bytes(c, 16)
    return {"workload": f"QFT of basis state {j} on {n} qubits, complex128 tiled",
            "ops": len(c), "ms_per_run": round(ms, 2),
            "gate_GBps": round(gb / (ms / 1e3) / 1e9, 1),
            "max_abs_err_vs_closed_form_2048_sampled": err,
            "passes": prof.get("tile_pass", {}).get("launches", 0) // 2}


def extras_haar(L, N):
    from everett_gb300 import State, workloads
    n, depth = 28, 40
    c = workloads.haar_layers(n, depth, seed=3)
    ref = State.zero(n, "complex128")
    ms128, _ = timed_runs(L, N, ref, c, 1, mode="tiled")
    st = State.zero(n, "complex64")
    out = {"workload": "Haar 1q on every qubit + CZ bricks, 28 qubits, depth 40 (1120 + 540 ops)",
           "complex128_tiled_ms": round(ms128, 1), "fusion_qubits": 5}
    for variant in ("bf16x3", "tf32x3", "fp32"):
        kw = dict(mode="fused", variant=variant, tile_bits=5)
        timed_runs(L, N, st, c, 1, **kw)
        ms, prof = timed_runs(L, N, st, c, 2, **kw)
        out[variant] = {"ms_per_run": round(ms, 1), "speedup_vs_complex128": round(ms128 / ms, 1),
                        "fidelity_vs_complex128": fidelity(ref, st),
                        "max_abs_err_vs_complex128": ref.max_abs_diff(st),
                        "blocks": prof.get("fused_unitary", {}).get("launches", 0) // 2}
    return out


def extras_batch(count: int = 4096):
    """cfg3: 4096 TFIM circuits (8-20 qubits, 10-50 steps, complex64, <Z_0>
    and 1000 shots each) in one persistent launch; the same circuits as 8
    consecutive batches of 512 for per-circuit latency; against one
    prepared CUDA-graph launch per circuit (planning and capture done
    beforehand, outside the timing) plus its <Z_0> and shots."""
    import numpy as np

    from everett_gb300 import CudaStateVectorBackend, Rng, State, batch, workloads
    rng = Rng.seed_from_u64(2024)
    cs = [workloads.tfim_raw(rng) for _ in range(count)]
    batch.run_batch(cs[:64], shots=1000, tile_bits=13, threads=256)
    t0 = time.perf_counter()
    res, st = batch.run_batch(cs, shots=1000, tile_bits=13, threads=256)
    wall = time.perf_counter() - t0
    # per-circuit latency: a circuit's result is ready when its batch ends
    lat = []
    t0 = time.perf_counter()
    for j in range(0, len(cs), 512):
        part = cs[j:j + 512]
        batch.run_batch(part, shots=1000, tile_bits=13, threads=256)
        lat += [(time.perf_counter() - t0) * 1e3] * len(part)
    chunked_wall = time.perf_counter() - t0
    # one prepared graph launch per circuit
    sample = cs[::16]
    states, preps = {}, []
    for c in sample:
        n = c.num_qubits()
        if n not in states:
            states[n] = State.zero(n, "complex64")
        preps.append((states[n], CudaStateVectorBackend.prepare(states[n], c)))
    for s_, p_ in preps[:8]:
        p_.launch(0)
        s_.bloch_vector(0)
        s_.sample(1000, seed=1)
    one = []
    t0 = time.perf_counter()
    for s_, p_ in preps:
        t1 = time.perf_counter()
        p_.launch(0)
        s_.bloch_vector(0)
        s_.sample(1000, seed=1)
        one.append((time.perf_counter() - t1) * 1e3)
    base = len(sample) / (time.perf_counter() - t0)
    for _, p_ in preps:
        p_.close()
    # every record sweeps its circuit's whole state in shared memory (read and
    # write of 2^n complex64 amplitudes)
    smem_bytes = sum(len(c) * 16 * (1 << c.num_qubits()) for c in cs)
    smem_peak = 152 * 128 * 2.07e9 / 1e9  # GB/s: 128 B per clock per SM, nominal
    achieved = smem_bytes / (st["device_ms"] / 1e3) / 1e9
    return {"workload": f"{count} TFIM Trotter circuits, 8-20 qubits, 10-50 steps, complex64, "
                        "<Z_0> + 1000 shots each", "circuits_per_s": round(count / wall, 1),
            "wall_s": round(wall, 3), "device_ms": round(st["device_ms"], 1),
            "latency_one_batch": {"p50_ms": round(wall * 1e3, 1), "p99_ms": round(wall * 1e3, 1),
                                  "note": "every circuit's result arrives when the launch ends"},
            "latency_8_batches_of_512": {
                "circuits_per_s": round(len(cs) / chunked_wall, 1),
                "p50_ms": round(float(np.percentile(lat, 50)), 1),
                "p99_ms": round(float(np.percentile(lat, 99)), 1)},
            "one_graph_launch_per_circuit": {
                "circuits_per_s": round(base, 1),
                "p50_ms_service": round(float(np.percentile(one, 50)), 3),
                "p99_ms_service": round(float(np.percentile(one, 99)), 3),
                "sample": f"every 16th circuit ({len(sample)})"},
            "speedup": round(count / wall / base, 1), "queue_items": st["items"],
            "tile_bits": st["tile_bits"], "threads": st["threads"],
            "roofline": {"kernel": "k_batch<float2>", "bound": "shared memory",
                         "achieved": round(achieved, 1), "peak": round(smem_peak, 1),
                         "unit": "GB/s", "frac": round(achieved / smem_peak, 3),
                         "peak_source": "nominal (128 B per clock per SM at 2.07 GHz; no "
                                        "measured shared-memory peak)",
                         "algorithmic_bytes": float(f"{smem_bytes:.4g}"),
                         "note": "each gate record reads and writes its circuit's whole "
                                 "state in shared memory once"}}


def extras_serve():
    from everett_gb300 import Rng, serve, workloads
    rng = Rng.seed_from_u64(42)
    reqs = [workloads.serve_request(rng, 10, 26) for _ in range(160)]
    requests = [(c, i, 1000) for i, (_, c) in enumerate(reqs)]
    srv = serve.Server(dtype="complex64", workers=8, mode="fused")
    srv.run_all(requests[:16])
    srv.close()
    srv = serve.Server(dtype="complex64", workers=1, mode="fused", batch_small=False)
    res, wall = serve.poisson_run(srv, requests, rate=1e6)
    srv.close()
    serial = serve.latency_summary(res, wall)
    out = {"workload": "Poisson mix, 10-26 qubits: 40% random layers depth 2n, 20% QFT, "
                       "20% GHZ + mid-circuit measurement + classical control, 20% TFIM; "
                       "1000 shots each; complex64 fused BF16x3",
           "serial_one_request_at_a_time": serial,
           "device_floor": serve_device_floor(requests, "complex64", "bf16x3")}
    for rate in (50.0, 1e6):
        srv = serve.Server(dtype="complex64", workers=8, mode="fused")
        res, wall = serve.poisson_run(srv, requests, rate=rate, seed=int(rate) % 1000)
        srv.close()
        key = "saturated_all_at_once" if rate > 1e5 else f"poisson_{int(rate)}_per_s"
        out[key] = serve.latency_summary(res, wall)
    # the same mix in complex128: fused digit-sliced passes for 12+ qubits
    c128 = {"workload": "the same requests in complex128, fused (ozaki) for 12 qubits and up"}
    srv = serve.Server(dtype="complex128", workers=1, mode="fused", batch_small=False)
    res, wall = serve.poisson_run(srv, requests, rate=1e6)
    srv.close()
    c128["serial_one_request_at_a_time"] = serve.latency_summary(res, wall)
    for rate in (50.0, 1e6):
        srv = serve.Server(dtype="complex128", workers=8, mode="fused")
        res, wall = serve.poisson_run(srv, requests, rate=rate, seed=int(rate) % 1000)
        srv.close()
        key = "saturated_all_at_once" if rate > 1e5 else f"poisson_{int(rate)}_per_s"
        c128[key] = serve.latency_summary(res, wall)
    c128["device_floor"] = serve_device_floor(requests, "complex128", "ozaki")
    out["complex128"] = c128
    for part in (out, c128):
        fl = part["device_floor"]["circuits_per_s"]
        part["saturated_over_floor"] = round(part["saturated_all_at_once"]["circuits_per_s"] / fl, 3)
    return out


def serve_device_floor(requests, dtype: str, variant: str):
    """The mix's device-time floor: each request run alone on the device (the
    kernels of the run and of its shots, each timed with CUDA events on the
    state's stream, host gaps excluded; fused passes above 12 qubits, tiled at
    or below, as the server runs them), summed.
    The large requests each saturate HBM on their own, so the sum bounds what
    any overlap of them can reach; overlap can only gain on the small ones."""
    from everett_gb300 import CudaStateVectorBackend, State, _native as N
    L = N.lib()
    states = {}
    total_ms = 0.0
    for c, seed, shots in requests:
        n = c.num_qubits()
        if n not in states:
            states[n] = State.zero(n, dtype)
        st = states[n]
        kw = (dict(mode="fused", variant=variant) if n > 12 else dict(mode="tiled"))
        CudaStateVectorBackend.run_into(st, c, seed, **kw)  # warm
        h = st.handle
        N.check(L.ev_state_profile(h, 1))
        CudaStateVectorBackend.run_into(st, c, seed, **kw)
        st.sample(shots, seed=seed)
        prof = read_profile(L, h)
        N.check(L.ev_state_profile(h, 0))
        total_ms += sum(v["ms"] for v in prof.values())
    states.clear()
    return {"sum_device_ms": round(total_ms, 1),
            "circuits_per_s": round(len(requests) / (total_ms / 1e3), 1)}


def extras_serve_small():
    """Continuous batching of small circuits: 2000 TFIM requests of 8-13
    qubits (complex64, 1000 shots each) through the server, which runs the
    small gate-only requests admitted together as one persistent batched
    launch, against serving them one request at a time with one launch
    sequence per circuit (run + sample)."""
    import numpy as np

    from everett_gb300 import CudaStateVectorBackend, Rng, State, serve, workloads
    rng = Rng.seed_from_u64(99)
    cs = [workloads.tfim_raw(rng, nmin=8, nmax=13) for _ in range(2000)]
    requests = [(c, i, 1000) for i, c in enumerate(cs)]
    states = {}
    sample = cs[::8]
    for c in sample[:8]:
        n = c.num_qubits()
        states.setdefault(n, State.zero(n, "complex64"))
        CudaStateVectorBackend.run_into(states[n], c, 0, mode="tiled")
    t0 = time.perf_counter()
    lat = []
    for c in sample:
        n = c.num_qubits()
        if n not in states:
            states[n] = State.zero(n, "complex64")
        t1 = time.perf_counter()
        CudaStateVectorBackend.run_into(states[n], c, 0, mode="tiled")
        states[n].sample(1000, seed=1)
        lat.append((time.perf_counter() - t1) * 1e3)
    base = len(sample) / (time.perf_counter() - t0)
    out = {"workload": "2000 TFIM Trotter requests, 8-13 qubits, 10-50 steps, complex64, "
                       "1000 shots each",
           "one_request_at_a_time_one_launch_sequence_each": {
               "circuits_per_s": round(base, 1),
               "p50_ms_service": round(float(np.percentile(lat, 50)), 3),
               "p99_ms_service": round(float(np.percentile(lat, 99)), 3)}}
    srv = serve.Server(dtype="complex64", workers=4, mode="tiled")
    try:
        srv.run_all(requests[:64])
        for rate in (2000.0, 1e6):
            res, wall = serve.poisson_run(srv, requests, rate=rate, seed=int(rate) % 997)
            key = "saturated_all_at_once" if rate > 1e5 else f"poisson_{int(rate)}_per_s"
            summ = serve.latency_summary(res, wall)
            summ["speedup_vs_one_at_a_time"] = round(summ["circuits_per_s"] / base, 1)
            out[key] = summ
        st = srv.stats()
        out["batched_launches"] = st["batched_launches"]
        out["batched_requests"] = st["batched_requests"]
    finally:
        srv.close()
    return out


def extras_prepared():
    """Replaying one circuit as a recorded CUDA graph against planning and
    launching it at every run (ev_state_run), same circuit and seeds."""
    from everett_gb300 import CudaStateVectorBackend, State, workloads
    out = {}
    for n, dtype, mode, depth in ((12, "complex128", "exact", 20), (20, "complex64", "tiled", 20)):
        c = workloads.ghz_midmeasure(n).compose(workloads.random_layers(n, depth, 7))
        c.measure(1, 0)
        st = State.zero(n, dtype)
        prep = CudaStateVectorBackend.prepare(st, c, mode=mode)
        reps = 200
        for seed in range(5):
            prep.launch(seed)
            CudaStateVectorBackend.run_into(st, c, seed, mode=mode)
        t0 = time.perf_counter()
        for seed in range(reps):
            CudaStateVectorBackend.run_into(st, c, seed, mode=mode)
        plain = reps / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        for seed in range(reps):
            prep.launch(seed)
        graph = reps / (time.perf_counter() - t0)
        out[f"{n}q_{dtype}_{mode}"] = {
            "workload": f"GHZ + mid-circuit measurement + X_if, then random layers depth {depth}, "
                        f"{n} qubits, {dtype}, {mode} mode, {len(c)} ops",
            "kernels_per_run": prep.kernels(), "runs_per_s_run_into": round(plain, 1),
            "runs_per_s_prepared_graph": round(graph, 1), "speedup": round(graph / plain, 2)}
        prep.close()
    return out


def extras_kernels(n: int, peak: float, reps: int = 3):
    """Each streaming kernel class alone on an n-qubit state, timed with CUDA
    events on the state's stream, against the measured copy bandwidth.
    Bytes are the algorithmic bytes the engine's kernel moves (2 * N_t * B for
    a gate; measure: the half with bit k read, then the kept half read and all
    written; normalize: one read for the norm, then a read and a write;
    sampling: one read of the state plus a write and a read of the 2^n - 1
    doubles of the probability tree).

    complex128 arithmetic is FP64, which GB300 issues at a small fraction of
    its FP32 rate, so each complex128 case also carries its FP64 floor: the
    FP64-pipe instructions its kernel issues per state amplitude (dadd, dfma
    and the dmul left on that pipe, counted from the source: a complex
    product in the reference's FMA form is 2 FMAs there plus 2 products
    formed on the integer pipes, a complex add 2) times 2^n, over the
    measured FMA issue rate.  The state is dense (a depth-2 random-layer
    circuit), as a circuit leaves it."""
    import ctypes as C

    import numpy as np

    from everett_gb300 import Gate1, Gate2, Rng, State, _native as N, workloads
    L = N.lib()
    rate = C.c_double()
    N.check(L.ev_probe_fp64(C.byref(rate)))
    soft_add = C.c_double()
    N.check(L.ev_probe_softadd(C.byref(soft_add)))
    g_dense = workloads.haar_1q(Rng.seed_from_u64(5))
    rng = np.random.default_rng(3)
    g2 = Gate2(rng.normal(size=16) + 1j * rng.normal(size=16))
    out = {"fp64_fma_per_s_measured": float(f"{rate.value:.4g}"),
           "integer_pipe_add_per_s_measured": float(f"{soft_add.value:.4g}")}
    prng = np.random.default_rng(9)
    zdiag = ["+" + "".join("Z" if b else "I" for b in prng.integers(0, 2, n)) for _ in range(8)]
    # eight strings with one X part and one Y pattern (one pass), Z varying
    xpart, ypart = prng.integers(0, 2, n), prng.integers(0, 2, n)
    xshared = ["+" + "".join(("XY"[int(y)] if xb else "IZ"[int(b)])
                             for xb, y, b in zip(xpart, ypart, prng.integers(0, 2, n)))
               for _ in range(8)]
    # eight strings with X on qubits 0 and 2 (partners inside blocks of 8)
    xlow = ["+X" + "IZ"[int(prng.integers(0, 2))] + "X"
            + "".join("IZ"[int(b)] for b in prng.integers(0, 2, n - 3)) for _ in range(8)]
    from everett_gb300 import CudaStateVectorBackend
    dense = workloads.random_layers(n, 2, seed=11)
    for dtype, B in (("complex128", 16), ("complex64", 8)):
        # dense states, as a circuit leaves them: every amplitude nonzero and
        # complex (the complex128 gates form their products on the integer
        # pipes only for operands in a normal range; zeros take the FP64 pipe)
        st = State.zero(n, dtype)
        other = State.zero(n, dtype)
        CudaStateVectorBackend.run_into(st, dense, 0, mode="tiled")
        CudaStateVectorBackend.run_into(other, dense, 1, mode="tiled")
        h = st.handle
        Nn = 1 << n
        hi, lo = n - 1, 0
        # name, call, algorithmic bytes, FP64-pipe instructions per amplitude
        # (complex128, with the plain products on the integer pipes)
        cases = [
            ("1q_dense_high", lambda: st.apply_1q(hi, g_dense), 2 * Nn * B, 6),
            ("1q_dense_low", lambda: st.apply_1q(lo, g_dense), 2 * Nn * B, 6),
            ("1q_real_h", lambda: st.apply_1q(hi - 3, Gate1.h()), 2 * Nn * B, 2),
            ("1q_real_h_low", lambda: st.apply_1q(2, Gate1.h()), 2 * Nn * B, 2),
            ("1q_anti_x_low", lambda: st.apply_1q(1, Gate1.x()), 2 * Nn * B, 0),
            ("1q_diag_rz", lambda: st.apply_1q(hi - 1, Gate1.rz(0.3)), 2 * Nn * B, 2),
            ("1q_phase", lambda: st.apply_1q(hi - 2, Gate1.phase(0.3)), Nn * B, 1),
            # X: a permutation (entries 0 and 1), no FP64 instruction
            ("1q_anti_x", lambda: st.apply_1q(7, Gate1.x()), 2 * Nn * B, 0),
            ("cnot", lambda: st.apply_2q(hi, 3, Gate2.cnot()), Nn * B, 0),
            ("cz", lambda: st.apply_2q(hi, 3, Gate2.cz()), Nn * B // 2, 0),
            ("swap", lambda: st.apply_2q(hi, 3, Gate2.swap()), Nn * B, 0),
            # 16 FMA-form products (their 32 FMAs on the FP64 pipe, the 32
            # plain products on the integer pipes) and 24 adds per quad
            ("2q_dense", lambda: st.apply_2q(hi, 3, g2), 2 * Nn * B, 14),
            ("controlled_1q_1ctrl", lambda: st.apply_controlled_1q([hi], 5, g_dense), Nn * B, 3),
            ("measure_high", lambda: st.measure_qubit(hi, 0.25), 2 * Nn * B, 2),
            ("measure_low", lambda: st.measure_qubit(lo, 0.25), 2 * Nn * B, 2),
            ("norm_sqr", lambda: st.norm_sqr(), Nn * B, 2),
            ("normalize", lambda: st.normalize(), 3 * Nn * B, 4),
            ("overlap", lambda: st.overlap(other), 2 * Nn * B, 4),
            ("sample_1000_shots", lambda: st.sample(1000, seed=1), Nn * B + 8 * Nn, 3),
            # per aligned block of 8 indices: 8 values (2 each), a 3-level
            # Walsh-Hadamard transform (24 adds) and one add per term: 6 per
            # index, 2^n indices for Z-only terms and 2^(n-1) with a shared X
            ("pauli_8_diagonal_terms", lambda: st.pauli_expectation(zdiag), Nn * B, 6),
            ("pauli_8_terms_shared_x", lambda: st.pauli_expectation(xshared), Nn * B, 3),
            # X below qubit 3: the blocks cover all 2^n indices
            ("pauli_8_terms_low_x", lambda: st.pauli_expectation(xlow), Nn * B, 6),
        ]
        res = {}
        for name, fn, nbytes, fp64 in cases:
            fn()
            if reps == 0:  # one call per case (a profiling target)
                continue
            N.check(L.ev_state_record_event(h, 0))
            for _ in range(reps):
                fn()
            N.check(L.ev_state_record_event(h, 1))
            ms = C.c_float()
            N.check(L.ev_state_elapsed_ms(h, 0, 1, C.byref(ms)))
            per = ms.value / reps
            gbs = nbytes / (per / 1e3) / 1e9
            r = {"ms": round(per, 3), "GB_s": round(gbs, 1), "frac": round(gbs / peak, 3)}
            if dtype == "complex128" and fp64:
                floor = fp64 * Nn / rate.value * 1e3
                hbm = nbytes / (peak * 1e9) * 1e3
                r["fp64_floor_ms"] = round(floor, 3)
                r["bound"] = "fp64" if floor > hbm else "hbm"
                r["frac_of_bound"] = round(max(floor, hbm) / per, 3)
            res[name] = r
            if name.startswith("measure"):
                N.check(L.ev_normalize(h))  # undo the collapse's zeroed half for later cases
                st.apply_1q(hi, Gate1.h())
                st.apply_1q(lo, Gate1.h())
        out[dtype] = res
        del st, other
    out["note"] = (f"{n} qubits; frac against the measured copy bandwidth {peak:.0f} GB/s; "
                   "complex128 cases with FP64 arithmetic also against the measured FP64 FMA "
                   "rate (frac_of_bound = the larger floor over the time)")
    return out


def extras_density():
    """Noisy density-matrix runs (DensityMatrixBackend with uniform
    depolarizing noise) on the GPU, against the oracle on the same circuit
    structure at a size it finishes quickly; both as matrix-element updates
    per second (ops x 4^n / time)."""
    import ctypes as C

    from everett_gb300 import _native as N, workloads
    from everett_gb300.density import DensityMatrixBackend, NoiseModel
    import oracle as O
    nm = NoiseModel.uniform_depolarizing(0.001)
    out = {}
    for n in (12, 14):
        c = workloads.random_layers(n, 4, seed=n)
        DensityMatrixBackend.run_with_noise(c, nm)  # warm-up
        t0 = time.perf_counter()
        ex = DensityMatrixBackend.run_with_noise(c, nm)
        ms = (time.perf_counter() - t0) * 1e3
        rho = ex.density_matrix()
        out[f"{n}q"] = {"ms_per_run": round(ms, 2), "ops": len(c),
                        "element_updates_per_s": float(f"{len(c) * 4.0 ** n / (ms / 1e3):.4g}"),
                        "trace": rho.trace(), "purity": rho.purity()}
        del ex, rho
    n = 7
    c = workloads.random_layers(n, 4, seed=n)
    t0 = time.perf_counter()
    O.dm_run(c, nm.ev_struct())
    cpu_s = time.perf_counter() - t0
    out["oracle_cpu"] = {"qubits": n, "ms_per_run": round(cpu_s * 1e3, 2), "cores": 1,
                         "element_updates_per_s": float(f"{len(c) * 4.0 ** n / cpu_s:.4g}"),
                         "note": "the reference's loops restated (index groups, scratch "
                                 "matrices); 1 core"}
    out["workload"] = ("random-layer circuit depth 4 (Rz Ry Rz per qubit + CNOT bricks), "
                       "depolarizing p=0.001 after every gate, complex128")
    return out


def extras_stabilizer():
    """Random Clifford circuits with mid-circuit measurements on the GPU
    tableau, against the oracle (the reference's tableau loops) on the same
    circuit."""
    from everett_gb300 import Circuit, Rng
    from everett_gb300.stabilizer import StabilizerBackend
    import oracle as O

    def circuit(n, gates, meas, seed):
        rng = Rng.seed_from_u64(seed)
        c = Circuit.with_classical(n, n)
        every = max(1, gates // max(1, meas))
        for k in range(gates):
            a = int(rng.next_u64() % n)
            b = (a + 1 + int(rng.next_u64() % (n - 1))) % n
            [lambda: c.h(a), lambda: c.s(a), lambda: c.cnot(a, b), lambda: c.cz(a, b)][k % 4]()
            if k % every == every - 1:
                c.measure(a, a)
        return c

    out = {"workload": "random H / S / CNOT / CZ circuit with a measurement every gates/meas gates"}
    for n, gates, meas in ((1000, 20000, 200), (4000, 40000, 100)):
        c = circuit(n, gates, meas, n)
        c.to_ev()  # the op records are encoded once, outside the timed region
        StabilizerBackend.run_seeded(circuit(64, 200, 4, 1), 0)
        t0 = time.perf_counter()
        ex = StabilizerBackend.run_seeded(c, 7)
        ms = (time.perf_counter() - t0) * 1e3
        row = {"gpu_ms": round(ms, 1), "gates": gates, "measurements": meas}
        if n <= 1000:
            t0 = time.perf_counter()
            want = O.stab_run(c, 7)
            cpu_ms = (time.perf_counter() - t0) * 1e3
            row["oracle_cpu_ms_1_core"] = round(cpu_ms, 1)
            row["speedup"] = round(cpu_ms / ms, 1)
            row["classical_equal"] = ex.classical() == want[3]
        out[f"{n}q"] = row
    return out


def run_ours(args, dist: Dist):
    import numpy as np

    from everett_gb300 import CudaStateVectorBackend, State, _native as N, build, workloads
    build.build()
    L = N.lib()
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
    N.check(L.ev_state_profile(h, 1))
    gpu_index = int(os.environ.get("LOCAL_RANK", 0))
    with Clocks(gpu_index if dist.world == 1 else 0) as clk:
        N.check(L.ev_state_record_event(h, 0))
        for _ in range(args.steps):
            step()
        N.check(L.ev_state_record_event(h, 1))
        ms = C.c_float()
        N.check(L.ev_state_elapsed_ms(h, 0, 1, C.byref(ms)))
    total_ms = ms.value
    lc1 = C.c_uint64()
    L.ev_state_launch_count(h, C.byref(lc1))
    prof = read_profile(L, h)
    N.check(L.ev_state_profile(h, 0))
    dist.barrier()
    worst_ms = dist.max(total_ms)
    value = dist.world * bytes_per_step * args.steps / (worst_ms / 1000) / 1e9

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        ops, ctrl, npool = circuit.to_ev()
        pinned_ops = C.c_void_p()
        N.check(L.ev_host_alloc(ops.nbytes, C.byref(pinned_ops)))
        out = C.c_void_p()
        out_bytes = (1 << n) * 16
        N.check(L.ev_host_alloc(out_bytes, C.byref(out)))
        C.memmove(pinned_ops, ops.ctypes.data, ops.nbytes)
        circ = N.EvCircuit(n, 0, pinned_ops.value, len(ops), ctrl.ctypes.data, npool)
        opts = N.EvRunOptions(N.C128, 1 if args.mode == "tiled" else 0, 0, 0)
        cl = np.zeros(1, dtype=np.uint8)
        dist.barrier()
        run_s = dl_s = 0.0
        # no nvidia-smi sampler here: its queries slow the host link (a 16 GiB
        # read-back measured 27-41 GB/s with it running, 136-190 GB/s without)
        clk_e2e = Clocks(gpu_index if dist.world == 1 else 0) if args.e2e_clocks else None
        with (clk_e2e if clk_e2e is not None else contextlib.nullcontext()):
            t0 = time.perf_counter()
            for _ in range(args.steps):
                t1 = time.perf_counter()
                N.check(L.ev_state_run(h, C.byref(circ), 0, C.byref(opts), cl.ctypes.data))
                t2 = time.perf_counter()
                N.check(L.ev_state_download(h, out, 1 << n))
                run_s += t2 - t1
                dl_s += time.perf_counter() - t2
            e2e_s = dist.max(time.perf_counter() - t0)
        L.ev_host_free(pinned_ops)
        L.ev_host_free(out)
        e2e = {"value": round(dist.world * bytes_per_step * args.steps / e2e_s / 1e9, 2),
               "unit": "GB/s", "h2d_bytes_per_step": int(ops.nbytes),
               "d2h_bytes_per_step": int(out_bytes),
               "ms_per_step_run": round(1e3 * run_s / args.steps, 1),
               "ms_per_step_download": round(1e3 * dl_s / args.steps, 1)}
        if clk_e2e is not None:
            e2e["clocks"] = clk_e2e.summary()

    peak, peak_kind = measured_peaks()
    roofline = roofline_of(prof, "tile_pass", 2.0 * (1 << n) * 16, peak, peak_kind,
                           "k_tile<double2> (shared-memory tile pass, complex128)",
                           ncu_figure("k_tile_c128", "traffic_bytes_per_launch_full_size"))
    fp64 = None
    if roofline is not None:
        rate = C.c_double()
        N.check(L.ev_probe_fp64(C.byref(rate)))
        instr = workloads.fp64_instructions(circuit)
        tile_ms = prof.get("tile_pass", {}).get("ms", 0.0) / max(1, args.steps)
        if tile_ms > 0:
            achieved = instr / (tile_ms / 1e3)
            fp64 = {"instructions_per_step": float(f"{instr:.4g}"),
                    "achieved_per_s": float(f"{achieved:.4g}"),
                    "peak_per_s": float(f"{rate.value:.4g}"),
                    "peak_source": "measured (ev_probe_fp64: sustained FP64 FMA issue rate)",
                    "frac": round(achieved / rate.value, 3),
                    "note": ("the reference's FP64 operations counted from the source, per "
                             "second of tile pass; above 1 because the pass forms part of its "
                             "products on the integer pipes (bit-identical)")}
            roofline["fp64"] = fp64
    if roofline is not None:
        roofline["note"] = (
            "compute-bound: GB300 issues FP64 at 1/64 of the FP32 rate, so the pass splits its "
            "products between the FP64 pipe and an exact integer-pipe multiply; ncu in rotation "
            f"passes: alu pipe {ncu_figure('k_tile_c128', 'alu_pipe_pct')}%, fp64 pipe "
            f"{ncu_figure('k_tile_c128', 'fp64_pipe_pct')}%, fma-heavy pipe "
            f"{ncu_figure('k_tile_c128', 'fmaheavy_pipe_pct')}% busy")

    # what HBM actually moves: the tile passes' measured DRAM traffic per
    # launch (ncu) times the launches of a step, over the step's time
    hbm_traffic_pct = None
    if roofline is not None and roofline.get("traffic"):
        per_step = roofline["traffic"] * roofline["launches"] / args.steps
        hbm_traffic_pct = round(100 * per_step / (worst_ms / args.steps / 1e3) / 1e9 / peak, 2)

    cpu = None
    extras = {}
    if dist.rank == 0:
        win = oracle_window(n, depth, parallel=False)
        rate, ops_done, dt = win.step(args.cpu_seconds)
        cpu = {"value": round(rate, 3), "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": f"first {ops_done} ops of the random-layer circuit at {win.n} "
                         f"qubits, {dt:.1f} s, scalar oracle (the reference's loops)"}
        del win
        if not args.no_extras:
            c128_ms = worst_ms / args.steps
            for key, fn in (("complex128_fused_same_circuit",
                             lambda: extras_c128_fused(L, N, state, circuit, c128_ms,
                                                       bytes_per_step, peak, peak_kind)),
                            ("complex128_fused6_same_circuit",
                             lambda: extras_c128_fused(L, N, state, circuit, c128_ms,
                                                       bytes_per_step, peak, peak_kind,
                                                       variant="ozaki6")),
                            ("complex64_fused_same_circuit",
                             lambda: extras_c64(L, N, state, circuit, c128_ms, bytes_per_step,
                                                peak, peak_kind)),
                            ("cfg0_20q_shots", lambda: extras_cfg0(L, N)),
                            ("qft", lambda: extras_qft(L, N, n, peak)),
                            ("haar28_depth40", lambda: extras_haar(L, N)),
                            ("batch_tfim4096", extras_batch),
                            ("serve_mix", extras_serve),
                            ("serve_small_batched", extras_serve_small),
                            ("prepared_graph", extras_prepared),
                            ("density_noisy", extras_density),
                            ("stabilizer", extras_stabilizer)):
                try:
                    extras[key] = fn()
                except Exception as exc:  # report, do not hide
                    extras[key] = {"error": f"{type(exc).__name__}: {exc}"}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(worst_ms / args.steps, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-layer circuit)",
            "config": {"workload": workload_name(n, depth), "mode": args.mode,
                       "ops": len(circuit), "algorithmic_bytes_per_step": bytes_per_step,
                       "parallelism": "replicas only" if dist.world > 1 else "1 GPU",
                       "l2": f"inputs larger than L2 ({(1 << n) * 16 / 2**30:.1f} GiB state), "
                             f"no flush"},
            "gate_bytes_pct_of_hbm_peak": round(100 * value / peak, 1),
            "hbm_traffic_pct_of_peak": hbm_traffic_pct,
            "amplitude_updates_per_s": float(f"{len(circuit) * (1 << n) / (worst_ms / args.steps / 1e3):.4g}"),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(lc1.value - lc0.value),
            "clocks": clk.summary(),
            "kernel_profile": prof,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)


def run_case(args):
    """One section alone, printing its own JSON line (a profiling target)."""
    from everett_gb300 import State, _native as N, build, workloads
    build.build()
    if args.case == "kernels":
        peak, _ = measured_peaks()
        print(json.dumps({"case": "kernels", **extras_kernels(args.qubits, peak, args.kernel_reps)}))
        return
    if args.case in ("batch", "serve", "serve_small", "prepared", "density", "stabilizer"):
        fn = {"batch": lambda: extras_batch(args.batch_count), "serve": extras_serve, "serve_small": extras_serve_small,
              "prepared": extras_prepared, "density": extras_density,
              "stabilizer": extras_stabilizer}[args.case]
        print(json.dumps({"case": args.case, **fn()}))
        return
    L = N.lib()
    c = workloads.random_layers(args.qubits, args.depth, seed=1)
    dtype = ("complex128" if args.case == "fused" and args.variant in ("ozaki", "ozaki6")
             else "complex64")
    st = State.zero(args.qubits, dtype)
    kw = (dict(mode="fused", variant=args.variant, tile_bits=args.fuse_bits) if args.case == "fused"
          else dict(mode="tiled"))
    for _ in range(args.warmup):
        timed_runs(L, N, st, c, 1, **kw)
    ms, prof = timed_runs(L, N, st, c, args.steps, **kw)
    print(json.dumps({"case": args.case, "qubits": args.qubits, "depth": args.depth, "dtype": dtype, **kw,
                      "ms_per_run": round(ms, 3), "kernel_profile": prof}))


def main():
    args = parse_args()
    if args.case != "headline":
        run_case(args)
        return
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
