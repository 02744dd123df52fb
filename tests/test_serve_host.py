"""Serving-loop admission and cancellation, exercised on the host: requests
that can never fit the HBM budget are refused at submit, and a pending
request can be cancelled before it is admitted (the server starts paused so
nothing reaches a GPU before the checks)."""
import pytest

from everett_gb300 import Circuit, _native, serve


def test_admission_refusal_and_cancel(engine):
    srv = serve.Server(dtype="complex64", workers=2, hbm_budget=4096, start_paused=True)
    try:
        big = Circuit(12)  # 2^12 x 8 bytes = 32 KiB > 4 KiB budget
        big.h(0)
        small = Circuit(2)
        small.h(0).cnot(0, 1)
        rid_big = srv.submit(big, seed=1, shots=4)
        rid_a = srv.submit(small, seed=2, shots=4)
        rid_b = srv.submit(small, seed=3, shots=4)
        res = srv.poll(wait_ms=100)
        assert [(r.id, r.status) for r in res] == [(rid_big, _native.ERR_ADMISSION)]
        srv.cancel(rid_b)
        st = srv.stats()
        assert st["refused"] == 1 and st["pending"] == 2 and st["admitted"] == 0
        srv.resume()
        got = {}
        for _ in range(200):
            for r in srv.poll(wait_ms=20):
                got[r.id] = r
            if len(got) == 2:
                break
        assert got[rid_b].status == _native.ERR_CANCELLED
        assert rid_a in got  # ran (on a host without a GPU it reports a device error)
        with pytest.raises(Exception):
            srv.cancel(rid_a)  # no longer pending
    finally:
        srv.close()
