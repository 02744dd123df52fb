"""GPU serving: each request's result is the same alone and in the mix.

Requests of every kind of the serving mix (random layers, QFT, GHZ with a
mid-circuit measurement and classical control, TFIM) are served once each
alone (one at a time) and once together with all the others in flight.
Shots and classical bits must be identical (the path a request takes and
every path's arithmetic are independent of the rest of the mix).  For
complex128 they must also equal the oracle's run (classical bits) and the
oracle's sampler on the oracle's final state (shots) -- in tiled mode because
its arithmetic is the reference's, in fused mode (5-qubit unitaries by digit
slicing, within ~1e-16 of it) because no uniform of these seeds falls that
close to a decision boundary."""
import numpy as np
import pytest

import oracle as O
from everett_gb300 import Rng, serve, workloads

pytestmark = pytest.mark.gpu


def mix(count, seed, nmin, nmax):
    rng = Rng.seed_from_u64(seed)
    return [workloads.serve_request(rng, nmin, nmax) for _ in range(count)]


@pytest.mark.parametrize("dtype,mode", [("complex128", "tiled"), ("complex128", "fused"),
                                        ("complex64", "fused"), ("complex64", "tiled")])
def test_serving_alone_equals_mixed(gpu, dtype, mode):
    reqs = mix(24, 7, 6, 16)
    alone = []
    srv = serve.Server(dtype=dtype, workers=1, mode=mode)
    try:
        for i, (_, c) in enumerate(reqs):
            out = srv.run_all([(c, 1000 + i, 300)])
            alone.append(next(iter(out.values())))
    finally:
        srv.close()
    srv = serve.Server(dtype=dtype, workers=8, mode=mode)
    try:
        mixed = list(srv.run_all([(c, 1000 + i, 300) for i, (_, c) in enumerate(reqs)]).values())
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == len(reqs) and st["reserved_bytes"] == 0
    for (kind, c), a, m in zip(reqs, alone, mixed):
        assert a.status == 0 and m.status == 0, kind
        assert np.array_equal(a.shots, m.shots), kind
        assert a.classical == m.classical, kind
    if dtype == "complex128":
        for i, ((kind, c), a) in enumerate(zip(reqs, alone)):
            circ = c.to_circuit() if hasattr(c, "to_circuit") else c
            want, bits, _ = O.run_seeded(circ, 1000 + i)
            assert a.classical == bits, kind
            assert np.array_equal(a.shots, O.sample_tree(want, 1000 + i, 300)), kind


def test_serving_admission_under_tight_budget(gpu):
    reqs = mix(16, 3, 10, 14)
    budget = 3 * (1 << 14) * 8
    srv = serve.Server(dtype="complex64", workers=8, hbm_budget=budget)
    try:
        out = srv.run_all([(c, i, 100) for i, (_, c) in enumerate(reqs)])
        st = srv.stats()
    finally:
        srv.close()
    assert all(r is not None and r.status == 0 for r in out.values())
    assert st["completed"] == 16 and st["reserved_bytes"] == 0 and st["budget_bytes"] == budget
