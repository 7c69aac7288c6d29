"""The split-precision tensor-core tile kernel on dense complex products,
against an FP64 product: the three-part BF16 split (BF16x6) must reach
FP32-level accuracy (error < 2e-6 of max|A| max|B| sqrt(K)), the two-part
split (BF16x3, dropped terms ~2^-16 per product) < 2e-5."""
import ctypes as C

import numpy as np
import pytest

from hofstadter_hubbard_tsc_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = {_lib.HH_PREC_BF16X6: 2e-6, _lib.HH_PREC_BF16X3: 2e-5}


def _run(device, M, N, K, seed, precision):
    rng = np.random.default_rng(seed)
    A = (rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K)))
    B = (rng.normal(size=(K, N)) + 1j * rng.normal(size=(K, N)))
    a = np.asfortranarray(A).ravel(order="F").view(np.float64).copy()
    b = np.asfortranarray(B).ravel(order="F").view(np.float64).copy()
    c = np.zeros(2 * M * N)
    dp = C.POINTER(C.c_double)
    device.check(device.lib.hh_tc_selftest(device.h, M, N, K, a.ctypes.data_as(dp), b.ctypes.data_as(dp),
                                           c.ctypes.data_as(dp), precision))
    got = c.view(np.complex128).reshape((M, N), order="F")
    ref = A @ B
    return np.abs(got - ref).max() / (np.abs(A).max() * np.abs(B).max() * np.sqrt(K))


@pytest.mark.parametrize("precision", [_lib.HH_PREC_BF16X6, _lib.HH_PREC_BF16X3])
@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (128, 128, 64), (40, 24, 37), (300, 200, 150), (8, 8, 8)])
def test_tc_tile_product(device, M, N, K, precision):
    err = _run(device, M, N, K, seed=M + N + K, precision=precision)
    assert err < TOL[precision], err


def test_tc_selftest_rejects_fp64(device):
    z = np.zeros(2 * 64)
    dp = C.POINTER(C.c_double)
    st = device.lib.hh_tc_selftest(device.h, 8, 8, 8, z.ctypes.data_as(dp), z.ctypes.data_as(dp),
                                   z.ctypes.data_as(dp), _lib.HH_PREC_FP64)
    assert st == -1


@pytest.mark.parametrize("precision", [_lib.HH_PREC_BF16X6, _lib.HH_PREC_BF16X3])
def test_bounded_wait_reports_timeout(device, precision):
    """A tile whose copy barrier is announced bytes that never arrive: the
    kernel's bounded waits run out, it unwinds and reports HH_ERR_TIMEOUT,
    and the context keeps working (the next product is correct)."""
    import time
    t0 = time.perf_counter()
    st = device.lib.hh_tc_selftest_hold(device.h, precision)
    dt = time.perf_counter() - t0
    assert st == -5, st
    assert "bounded" in device.lib.hh_last_error(device.h).decode()
    assert dt < 30.0, dt
    err = _run(device, 40, 24, 37, seed=1, precision=precision)
    assert err < TOL[precision], err
