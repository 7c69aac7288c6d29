"""The split-precision tensor-core tile kernel on dense complex products,
against an FP64 product: the BF16 three-way split must reach FP32-level
accuracy (relative error < 2e-6 of ||A|| ||B||)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(device, M, N, K, seed):
    rng = np.random.default_rng(seed)
    A = (rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K)))
    B = (rng.normal(size=(K, N)) + 1j * rng.normal(size=(K, N)))
    a = np.asfortranarray(A).ravel(order="F").view(np.float64).copy()
    b = np.asfortranarray(B).ravel(order="F").view(np.float64).copy()
    c = np.zeros(2 * M * N)
    dp = C.POINTER(C.c_double)
    device.check(device.lib.hh_tc_selftest(device.h, M, N, K, a.ctypes.data_as(dp), b.ctypes.data_as(dp),
                                           c.ctypes.data_as(dp)))
    got = c.view(np.complex128).reshape((M, N), order="F")
    ref = A @ B
    return np.abs(got - ref).max() / (np.abs(A).max() * np.abs(B).max() * np.sqrt(K))


@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (128, 128, 64), (40, 24, 37), (300, 200, 150), (8, 8, 8)])
def test_tc_tile_product(device, M, N, K):
    err = _run(device, M, N, K, seed=M + N + K)
    assert err < 2e-6, err
