"""The measurement entry point that allocates nothing.

ev_measure_qubit_noalloc serves callers that cannot call cudaMalloc (their
device memory belongs to their own allocator, or an allocation's implicit
device synchronisation is not acceptable where they call it).  This test plays
such a caller: it owns a device buffer (allocated here through the CUDA
runtime, outside the engine), measures it in place through the C ABI twice in
a row, and checks outcome and amplitudes against the state-owned
ev_measure_qubit on the same amplitudes and uniforms, within the 1e-12
amplitude tolerance of the measurement parity tests.  This file is collected
last so that a failure here cannot hide another test's result.
"""
import ctypes as C
import ctypes.util
import os

import numpy as np
import pytest

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
        return rt
    pytest.fail("CUDA runtime library not found")


H2D, D2H = 1, 2


@pytest.mark.parametrize("n", [10, 21])
def test_noalloc_measure_matches_state_measure(gpu, n):
    rng = np.random.default_rng(n)
    amps = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    amps /= np.linalg.norm(amps)
    rt = _cudart()
    buf = C.c_void_p()
    assert rt.cudaMalloc(C.byref(buf), amps.nbytes) == 0
    try:
        assert rt.cudaMemcpy(buf, amps.ctypes.data, amps.nbytes, H2D) == 0
        ref = State.from_amplitudes(amps)
        lib = _native.lib()
        for k, u in ((3, 0.41), (n - 1, 0.77)):  # two calls in a row
            out = C.c_int32(-1)
            _native.check(lib.ev_measure_qubit_noalloc(buf, n, k, u, None, C.byref(out)))
            want = ref.measure_qubit(k, u)
            assert bool(out.value) == want
            got = np.empty_like(amps)
            assert rt.cudaMemcpy(got.ctypes.data, buf, amps.nbytes, D2H) == 0
            assert np.max(np.abs(got - ref.amplitudes())) < 1e-12
        # sizes beyond the maximum are refused with a clear error
        out = C.c_int32()
        rc = lib.ev_measure_qubit_noalloc(buf, 41, 0, 0.5, None, C.byref(out))
        assert rc == _native.ERR_INVALID_ARGUMENT
        assert "maximum" in _native.last_error()
    finally:
        rt.cudaFree(buf)
