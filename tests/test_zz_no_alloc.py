"""The measurement entry point that allocates nothing.

ev_measure_qubit_noalloc serves callers that cannot call cudaMalloc (their
device memory belongs to their own allocator, or an allocation's implicit
device synchronisation is not acceptable where they call it).  This test plays
such a caller: it owns a device buffer (allocated here through the CUDA
runtime, outside the engine), measures it in place through the C ABI twice in
a row, and checks outcome and amplitudes against the CPU oracle's
measure_qubit (measure.rs:15-51) and against the state-owned
ev_measure_qubit on the same amplitudes and uniforms, within the 1e-12
amplitude tolerance of the measurement parity tests.  It does so on the
legacy default stream and on a stream the caller created, and checks that
buffers the kernels could not use are refused before any launch.  This file
is collected last so that a failure here cannot hide another test's result.
"""
import ctypes as C
import ctypes.util
import os

import numpy as np
import pytest

import oracle as O
from everett_gb300 import State, _native

pytestmark = pytest.mark.gpu


def _cudart():
    names = [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so"),
             "libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")]
    for name in names:
        if not name:
            continue
        try:
            rt = C.CDLL(name)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
        rt.cudaStreamDestroy.argtypes = [C.c_void_p]
        return rt
    pytest.fail("CUDA runtime library not found")


H2D, D2H = 1, 2


def _measure_twice(rt, lib, buf, amps, n, stream):
    """Two measurements in a row on the caller's buffer, each checked against
    the oracle and the state-owned path."""
    ref = State.from_amplitudes(amps)
    want = amps.copy()
    for k, u in ((3, 0.41), (n - 1, 0.77)):
        out = C.c_int32(-1)
        _native.check(lib.ev_measure_qubit_noalloc(buf, n, k, u, stream, C.byref(out)))
        want_bit = O.measure_qubit(want, k, u)
        assert bool(out.value) == want_bit
        assert ref.measure_qubit(k, u) == want_bit
        got = np.empty_like(amps)
        assert rt.cudaMemcpy(got.ctypes.data, buf, amps.nbytes, D2H) == 0
        assert np.max(np.abs(got - want)) < 1e-12
        assert np.max(np.abs(got - ref.amplitudes())) < 1e-12


@pytest.mark.parametrize("n", [10, 21])
def test_noalloc_measure_matches_oracle(gpu, n):
    rng = np.random.default_rng(n)
    amps = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    amps /= np.linalg.norm(amps)
    rt = _cudart()
    lib = _native.lib()
    buf = C.c_void_p()
    stream = C.c_void_p()
    assert rt.cudaMalloc(C.byref(buf), amps.nbytes) == 0
    try:
        # the legacy default stream
        assert rt.cudaMemcpy(buf, amps.ctypes.data, amps.nbytes, H2D) == 0
        _measure_twice(rt, lib, buf, amps, n, None)
        # a stream the caller created
        assert rt.cudaStreamCreate(C.byref(stream)) == 0
        assert rt.cudaMemcpy(buf, amps.ctypes.data, amps.nbytes, H2D) == 0
        _measure_twice(rt, lib, buf, amps, n, stream)
        # sizes beyond the maximum are refused with a clear error
        out = C.c_int32()
        rc = lib.ev_measure_qubit_noalloc(buf, 41, 0, 0.5, None, C.byref(out))
        assert rc == _native.ERR_INVALID_ARGUMENT
        assert "maximum" in _native.last_error()
    finally:
        if stream.value:
            rt.cudaStreamDestroy(stream)
        rt.cudaFree(buf)


def test_noalloc_refuses_unusable_buffers(gpu):
    """A misaligned device pointer, host memory and a buffer holding fewer
    than 2^n amplitudes from the given address are refused with
    EV_ERR_INVALID_ARGUMENT before any launch; the caller's data are
    untouched and the next valid call works."""
    n = 17  # a 2 MiB buffer
    amps = O.sample_state(n)
    amps /= np.linalg.norm(amps)
    rt = _cudart()
    lib = _native.lib()
    buf = C.c_void_p()
    assert rt.cudaMalloc(C.byref(buf), amps.nbytes) == 0
    try:
        assert rt.cudaMemcpy(buf, amps.ctypes.data, amps.nbytes, H2D) == 0
        out = C.c_int32(-1)
        half = amps.nbytes // 2
        for ptr, nq, why in ((buf.value + 8, n, "aligned"),
                             (amps.ctypes.data, n, "device memory"),
                             (buf.value + half, n, "fewer than")):
            rc = lib.ev_measure_qubit_noalloc(C.c_void_p(ptr), nq, 0, 0.5, None, C.byref(out))
            assert rc == _native.ERR_INVALID_ARGUMENT, why
            msg = _native.last_error()
            assert why in msg or (why == "device memory" and "allocation" in msg), (why, msg)
        got = np.empty_like(amps)
        assert rt.cudaMemcpy(got.ctypes.data, buf, amps.nbytes, D2H) == 0
        assert np.array_equal(got, amps)
        want = amps.copy()
        _native.check(lib.ev_measure_qubit_noalloc(buf, n, 2, 0.3, None, C.byref(out)))
        assert bool(out.value) == O.measure_qubit(want, 2, 0.3)
        # the second half of the buffer, as a register of n - 1 qubits, fits
        assert rt.cudaMemcpy(buf, amps.ctypes.data, amps.nbytes, H2D) == 0
        sub = amps[1 << (n - 1):].copy()
        sub /= np.linalg.norm(sub)
        assert rt.cudaMemcpy(C.c_void_p(buf.value + half), sub.ctypes.data, sub.nbytes, H2D) == 0
        _native.check(lib.ev_measure_qubit_noalloc(C.c_void_p(buf.value + half), n - 1, 4, 0.6,
                                                   None, C.byref(out)))
        assert bool(out.value) == O.measure_qubit(sub, 4, 0.6)
        got = np.empty_like(sub)
        assert rt.cudaMemcpy(got.ctypes.data, C.c_void_p(buf.value + half), sub.nbytes, D2H) == 0
        assert np.max(np.abs(got - sub)) < 1e-12
    finally:
        rt.cudaFree(buf)
