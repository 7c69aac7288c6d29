"""The library's own FP64 eigensolver of density-matrix sectors (Householder
reduction on a thread-block cluster, bisection, inverse iteration, Newton-
Schulz orthonormalisation, back-transformation) against numpy's eigh, and
against the cuSOLVER zheevd path it replaces, through the C ABI."""
import ctypes as C

import numpy as np
import pytest

from hofstadter_hubbard_tsc_gb300 import _lib, step
from hofstadter_hubbard_tsc_gb300.device import DWave
from oracle.blocks import SSector, WSub, Wave
from oracle.density import get_density_matrix_sys, get_density_matrix_env, get_truncation_operator
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _selftest(device, a):
    n = a.shape[0]
    A = np.asfortranarray(a.astype(np.complex128))
    w = np.zeros(n)
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    dp = C.POINTER(C.c_double)
    device.check(device.lib.hh_eig_selftest(device.h, n, A.ctypes.data_as(dp), w.ctypes.data_as(dp),
                                            V.ctypes.data_as(dp)))
    return w, V


def _canonical(v):
    top = v[np.argmax(np.abs(v), axis=0), np.arange(v.shape[1])]
    return v * (np.conj(top) / np.abs(top))[None, :]


def _hermitian(rng, lam):
    n = len(lam)
    q, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    a = (q * lam[None, :]) @ q.conj().T
    return 0.5 * (a + a.conj().T)


def _check(a, w, V):
    """Backward-stable FP64 accuracy: eigenvalues, residuals and the
    orthonormality of the columns within 4 eps max(n, 64) ||A||."""
    n = a.shape[0]
    w_ref = np.linalg.eigvalsh(a)
    nrm = max(np.abs(w_ref).max(), 1e-300)
    tol = 4e-16 * max(n, 64)
    np.testing.assert_allclose(w, w_ref, atol=tol * nrm, rtol=0)
    assert np.all(np.diff(w) >= 0)
    # eigenpairs, orthonormal columns, canonical phase
    np.testing.assert_allclose(a @ V - V * w[None, :], 0.0, atol=tol * nrm)
    np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=tol)
    top = V[np.argmax(np.abs(V), axis=0), np.arange(n)]
    np.testing.assert_allclose(top.imag, 0.0, atol=1e-14)
    assert np.all(top.real > 0)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 33, 100, 257, 512, 1024])
def test_random_hermitian(device, n):
    rng = np.random.default_rng(n)
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    a = a + a.conj().T
    w, V = _selftest(device, a)
    _check(a, w, V)
    # columns of well-separated eigenvalues equal numpy's (canonical phase)
    wr, vr = np.linalg.eigh(a)
    vr = _canonical(vr)
    gap = np.minimum(np.r_[np.inf, np.diff(wr)], np.r_[np.diff(wr), np.inf])
    sep = gap > 1e-3 * np.abs(wr).max()
    np.testing.assert_allclose(V[:, sep], vr[:, sep], atol=1e-10)


@pytest.mark.parametrize("n", [40, 160, 400])
def test_density_spectra(device, n):
    """Spectra of density matrices: decaying over tens of decades, exact zeros
    (rank-deficient sectors) and exactly degenerate triples."""
    rng = np.random.default_rng(7 + n)
    lam = 10.0 ** (-np.arange(n) / (n / 14.0))
    lam[n // 2:] = 0.0                                  # null space
    lam[3:6] = lam[3]                                   # degenerate triple
    lam[n // 4:n // 4 + 3] = lam[n // 4]
    lam /= lam.sum()
    a = _hermitian(rng, lam)
    w, V = _selftest(device, a)
    _check(a, w, V)


def _wave(dims, side, seed, decay=6.0):
    rng = np.random.default_rng(seed)
    subs = []
    for k, (a, b) in enumerate(dims):
        ss = SSector(2 * k, k % 3, 60 - 2 * k, k % 3, a, b)
        d = np.exp(-np.arange(max(a, b)) / decay)
        v = rng.normal(size=(a, b)) + 1j * rng.normal(size=(a, b))
        v *= (d[:a, None] if side == 0 else d[None, :b]) * np.exp(-k / 3.0)
        subs.append(WSub(ss, v))
    psi = Wave(3, 3, subs)
    nrm = np.sqrt(sum(np.vdot(s.vec, s.vec).real for s in subs))
    for s in subs:
        s.vec /= nrm
    return psi


def _dwave(device, ow):
    w = H.wave(ow)
    dw = DWave(device, w.layout(), w.sys_len, w.env_len)
    dw.upload(w.flat())
    return dw


@pytest.mark.parametrize("kept", [(300, 500), (20, 40)])
@pytest.mark.parametrize("side", [0, 1])
def test_own_matches_cusolver_and_oracle(device, side, kept):
    """hh_density_truncate with the library's own eigensolver and with
    cuSOLVER zheevd: the same kept states, discarded weight, entropy and
    spectrum, and the same kept subspace in every sector, both equal to the
    oracle; sectors of 5 to 512 states, a rank-deficient one among them."""
    dims = [(5, 7), (33, 40), (64, 20), (120, 150), (257, 300), (512, 480)]
    psi = _wave(dims, side, 30 + side, decay=20.0)
    den = get_density_matrix_sys(psi) if side == 0 else get_density_matrix_env(psi)
    kmin, kmax = kept
    o_trun, o_ns, o_err, o_ent, o_spec = get_truncation_operator(den, kmin, kmax, 1e-12)
    res = {}
    for solver in (_lib.HH_EIG_OWN, _lib.HH_EIG_CUSOLVER):
        device.check(device.lib.hh_ctx_set_eigensolver(device.h, solver))
        try:
            res[solver] = step.density_truncate(device, _dwave(device, psi), side, kmin, kmax, 1e-12)
        finally:
            device.check(device.lib.hh_ctx_set_eigensolver(device.h, _lib.HH_EIG_OWN))
    rho = {(s.num_up, s.num_down): s.mat for s in den.subs}
    po = {(s.num_up, s.num_down): s.mat @ s.mat.conj().T for s in o_trun.subs}
    # the kept subspace is unique to ~eps / gap when the cut is in a gap
    cut_gap = o_spec[o_ns - 1] - o_spec[o_ns] if o_ns < len(o_spec) else 1.0
    for solver, (trun, ns, err, ent, spec) in res.items():
        assert ns == o_ns, solver
        assert err == pytest.approx(o_err, abs=1e-12)
        assert ent == pytest.approx(o_ent, abs=1e-12)
        np.testing.assert_allclose(spec, o_spec, atol=5e-14)
        g = trun.download()
        assert [(s.num_up, s.num_down, s.row_dim, s.sdim) for s in g.subs] == \
               [(s.num_up, s.num_down, s.row_dim, s.sdim) for s in o_trun.subs]
        for sg in g.subs:
            v = sg.mat
            r = rho[(sg.num_up, sg.num_down)]
            lam = np.einsum("ij,ik,kj->j", v.conj(), r, v).real
            np.testing.assert_allclose(r @ v - v * lam, 0.0, atol=5e-14)
            np.testing.assert_allclose(v.conj().T @ v, np.eye(sg.sdim), atol=1e-12)
            if cut_gap > 1e-7:
                p = v @ v.conj().T
                np.testing.assert_allclose(p, po[(sg.num_up, sg.num_down)], atol=1e-8)


def test_rejects_unknown_solver(device):
    assert device.lib.hh_ctx_set_eigensolver(device.h, 7) == _lib.HH_ERR_INVALID
