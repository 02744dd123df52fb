"""The digit-sliced f64 product of the complex128 fused passes (the Ozaki
scheme, everett_gb300/csrc/ev_ozaki.cuh), restated on the host with the
kernel's own slicing and recombination routines (ev_ozaki_gemm_host_digits),
against exact rational products.  Bars, relative to 8 x the row's largest
value x the matrix's largest entry: seven digits 2^-50 (FP64-class; the
plain f64 sum of 64 products errs by up to ~64 ulps of the same scale), six
digits 2^-42 (the error bound of a 47-bit fixed point with the diagonals
d >= 6 dropped: 256 times the seven-digit one)."""
import ctypes as C
from fractions import Fraction

import numpy as np
import pytest

from everett_gb300 import _native as N

P = C.POINTER(C.c_double)


DIGITS = pytest.mark.parametrize("digits", [7, 6])
BAR = {7: 2.0 ** -50, 6: 2.0 ** -42}


def oz(x, w, digits=7):
    x = np.ascontiguousarray(x, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    y = np.empty((x.shape[0], 64))
    N.check(N.lib().ev_ozaki_gemm_host_digits(x.ctypes.data_as(P), x.shape[0],
                                              w.ctypes.data_as(P), y.ctypes.data_as(P), digits))
    if digits == 7:  # the original entry point is the seven-digit one
        y7 = np.empty_like(y)
        N.check(N.lib().ev_ozaki_gemm_host(x.ctypes.data_as(P), x.shape[0], w.ctypes.data_as(P),
                                           y7.ctypes.data_as(P)))
        assert np.array_equal(y, y7)
    return y


def exact(x, w):
    out = np.empty((x.shape[0], 64))
    fw = [[Fraction(float(w[k, n])) for n in range(64)] for k in range(64)]
    for r in range(x.shape[0]):
        fx = [Fraction(float(v)) for v in x[r]]
        for n in range(64):
            out[r, n] = float(sum(fx[k] * fw[k][n] for k in range(64) if fx[k]))
    return out


def unitary_w(rng):
    """The real 64 x 64 embedding of a random 32 x 32 unitary, as the fused
    planner builds it (y = x W on interleaved [re, im] rows)."""
    a = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    q, r = np.linalg.qr(a)
    u = q * (np.diag(r) / np.abs(np.diag(r)))
    w = np.zeros((64, 64))
    for i in range(32):
        for f in range(32):
            v = u[i, f]
            w[2 * f, 2 * i], w[2 * f + 1, 2 * i] = v.real, -v.imag
            w[2 * f, 2 * i + 1], w[2 * f + 1, 2 * i + 1] = v.imag, v.real
    return w


def check(x, w, digits=7):
    y, e = oz(x, w, digits), exact(x, w)
    scale = np.abs(x).max(axis=1) * np.abs(w).max() * 8
    scale[scale == 0] = 1
    err = (np.abs(y - e).max(axis=1) / scale).max()
    assert err <= BAR[digits], (digits, err)
    return y, e


@DIGITS
def test_unitary_rows_of_every_scale(digits):
    rng = np.random.default_rng(1)
    x = rng.normal(size=(8, 64)) * np.array([1, 1e-5, 3e-12, 1e3, 1, 1, 2 ** -600, 1e-290])[:, None]
    x[4, ::3] = 0.0
    x[5, 5] = 1e-200  # 190 orders below its row: contributes nothing above the bar
    check(x, unitary_w(rng), digits)


@DIGITS
def test_identity_and_basis_rows(digits):
    """W = I and single-entry rows: outputs within a few units of the last
    kept bit of the row's and column's power-of-two bounds."""
    rng = np.random.default_rng(2)
    x = rng.normal(size=(5, 64))
    y, e = check(x, np.eye(64), digits)
    last = 2.0 ** -51 if digits == 7 else 2.0 ** -43
    assert np.all(np.abs(y - x) <= last * np.abs(x).max(axis=1, keepdims=True))
    x = np.zeros((3, 64))
    x[0, 0], x[1, 63], x[2, 7] = 1.0, -0.5, 2.0 ** -30
    check(x, unitary_w(rng), digits)


@DIGITS
def test_zero_rows_and_columns(digits):
    rng = np.random.default_rng(3)
    w = unitary_w(rng)
    w[:, 5] = 0.0
    x = rng.normal(size=(3, 64))
    x[1] = 0.0
    y, e = check(x, w, digits)
    assert np.all(y[1] == 0) and np.all(y[:, 5] == 0)


@DIGITS
def test_digit_sums_at_their_bounds(digits):
    """Rows and columns whose digits are all at the balanced extremes drive
    every diagonal sum to its largest magnitude (up to digits * 2^20): the
    f32 sums and the conversions stay exact."""
    for xv, wv in [(1 - 2 ** -53, 1 - 2 ** -53), (-(1 - 2 ** -53), 1 - 2 ** -53),
                   (0.75 + 2 ** -40, -0.999), (2 ** -1 + 2 ** -9 + 2 ** -17, 0.5 + 2 ** -9)]:
        x = np.full((2, 64), xv)
        x[1, ::2] *= -1
        w = np.full((64, 64), wv)
        check(x, w, digits)


@DIGITS
@pytest.mark.parametrize("seed", range(3))
def test_random_matrices(seed, digits):
    rng = np.random.default_rng(10 + seed)
    w = rng.normal(size=(64, 64)) * np.exp(rng.uniform(-20, 20, size=(1, 64)))
    x = rng.normal(size=(4, 64)) * np.exp(rng.uniform(-30, 30, size=(4, 1)))
    check(x, w, digits)
