"""OpenQASM 3 circuits on the GPU: the reference's round-trip property
(properties.rs:501-517: emit, parse back, same state to fidelity 1 - 1e-10)
and serving requests given as QASM text (same result as the parsed circuit
submitted directly)."""
import numpy as np
import pytest

from everett_gb300 import Circuit, CudaStateVectorBackend, Rng, algorithms, serve
from everett_gb300.error import QasmError

from test_qasm import named_circuit

pytestmark = pytest.mark.gpu


def test_qasm_round_trip_preserves_state(gpu):
    rng = Rng.seed_from_u64(501)
    for case in range(128):
        c = named_circuit(rng)
        back = Circuit.from_qasm(c.to_qasm())
        s1 = CudaStateVectorBackend.run(c).state()
        s2 = CudaStateVectorBackend.run(back).state()
        assert s1.fidelity(s2) > 1.0 - 1e-10, case


def test_algorithms_round_trip_fidelity(gpu):  # mod.rs roundtrip_bell / ghz / qft
    for c in (algorithms.bell(), algorithms.ghz(4), algorithms.qft(4)):
        back = Circuit.from_qasm(c.to_qasm())
        s1 = CudaStateVectorBackend.run(c).state()
        s2 = CudaStateVectorBackend.run(back).state()
        assert s1.fidelity(s2) > 1.0 - 1e-10


def test_serving_qasm_text(gpu):
    srcs = []
    for n in (6, 9, 12):
        c = Circuit.with_classical(n, 1)
        c.compose(algorithms.qft(n))
        c.measure(0, 0).x_if(0, n - 1)
        srcs.append(c.to_qasm())
    srv = serve.Server(dtype="complex128", workers=4, mode="tiled")
    try:
        ids = [srv.submit_qasm(s, seed=7 + i, shots=200) for i, s in enumerate(srcs)]
        direct = [srv.submit(Circuit.from_qasm(s), seed=7 + i, shots=200)
                  for i, s in enumerate(srcs)]
        with pytest.raises(QasmError):
            srv.submit_qasm("qubit[2] q;\nfoo q[0];\n")
        got = {}
        while len(got) < 6:
            for r in srv.poll(wait_ms=200):
                got[r.id] = r
    finally:
        srv.close()
    for a, b in zip(ids, direct):
        assert got[a].status == 0 and got[b].status == 0
        assert np.array_equal(got[a].shots, got[b].shots)
        assert got[a].classical == got[b].classical
