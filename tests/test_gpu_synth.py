"""Synthetic mid-chain superblocks of the matvec configurations (Hubbard and
t-J, the shapes of the m = 2000 / 4000 / 6000 workloads at small m): the GPU
FP64 model_wave against the oracle's, and both split precisions against the
FP64 path."""
import numpy as np
import pytest

import bench
from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.superblock import Superblock
from hofstadter_hubbard_tsc_gb300.synth import Workload

pytestmark = pytest.mark.gpu

CASES = {
    "hubbard-4x6": dict(W=4, L=6, n_elec=20, m=60, phi=1.0 / 3.0),
    "tj-2x12": dict(W=2, L=12, n_elec=20, m=160, model="tj", J=0.4, phi=1.0 / 6.0),
    "tj-4x6": dict(W=4, L=6, n_elec=22, m=60, model="tj", J=0.4, phi=1.0 / 6.0),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_synthetic_matvec(device, name):
    wl = Workload(**CASES[name])
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    rng = np.random.default_rng(5)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    sb.w_in.upload(psi)
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
    gpu = sb.w_out.download()
    _, ref = bench.cpu_matvec_timer(wl, psi, 1)
    assert np.linalg.norm(gpu - ref) / np.linalg.norm(ref) < 1e-12
    for prec, tol in ((_lib.HH_PREC_BF16X6, 5e-6), (_lib.HH_PREC_BF16X3, 2e-5)):
        device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, prec))
        got = sb.w_out.download()
        assert np.linalg.norm(got - gpu) / np.linalg.norm(gpu) < tol, (prec, name)
    sb.free()


def test_batched_matvec(device):
    """A wave of several vectors (the batched psi of the synthetic
    configuration): every vector equals its own single-vector product, in
    FP64 and split precision; mismatched batches are rejected."""
    from hofstadter_hubbard_tsc_gb300.device import DWave
    wl = Workload(**CASES["tj-2x12"])
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    nb = 3
    rng = np.random.default_rng(8)
    psi = rng.normal(size=(nb, wl.sup.dim)) + 1j * rng.normal(size=(nb, wl.sup.dim))
    lay = sb.w_in.layout
    win = DWave(device, lay, sb.w_in.sys_len, sb.w_in.env_len, nbatch=nb)
    wout = DWave(device, lay, sb.w_in.sys_len, sb.w_in.env_len, nbatch=nb)
    win.upload(psi)
    for prec in (_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3):
        device.check(device.lib.hh_matvec(sb.plan, win.h, wout.h, prec))
        got = wout.download().reshape(nb, -1)
        for b in range(nb):
            sb.w_in.upload(psi[b])
            device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, prec))
            ref = sb.w_out.download()
            assert np.linalg.norm(got[b] - ref) / np.linalg.norm(ref) < 1e-13, (prec, b)
    assert device.lib.hh_matvec(sb.plan, win.h, sb.w_out.h, _lib.HH_PREC_FP64) == -1
    win.free()
    wout.free()
    sb.free()


def test_lognormal_batched_uneven(device):
    """The synthetic block-sparse configuration at small scale (6-wide
    cylinder: 12 terms; 24 lognormal sectors per block, median 8, max 32):
    the GPU FP64 matvec equals the oracle's, and a batch of 8 uneven
    wavefunctions (per-sector lognormal weights, norms over eight decades) in
    one hh_matvec call equals the single-vector products (FP64) and stays
    within 2e-5 of FP64 per vector in BF16x3."""
    from hofstadter_hubbard_tsc_gb300.device import DWave
    from hofstadter_hubbard_tsc_gb300.synth import uneven_batch
    wl = Workload(W=6, L=8, n_elec=42, U=8.0, phi=1.0 / 3.0, lognormal=(24, 8, 32))
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    assert len(sb.terms) == 12
    nb = 8
    psi = uneven_batch([s.sys_dim * s.env_dim for s in wl.sup.subs], nb, np.random.default_rng(4))
    sb.w_in.upload(psi[2])
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
    _, ref = bench.cpu_matvec_timer(wl, psi[2], 1)
    assert np.linalg.norm(sb.w_out.download() - ref) / np.linalg.norm(ref) < 1e-12
    lay = sb.w_in.layout
    win = DWave(device, lay, sb.w_in.sys_len, sb.w_in.env_len, nbatch=nb)
    wout = DWave(device, lay, sb.w_in.sys_len, sb.w_in.env_len, nbatch=nb)
    win.upload(psi)
    device.check(device.lib.hh_matvec(sb.plan, win.h, wout.h, _lib.HH_PREC_FP64))
    fp64 = wout.download().reshape(nb, -1)
    device.check(device.lib.hh_matvec(sb.plan, win.h, wout.h, _lib.HH_PREC_BF16X3))
    x3 = wout.download().reshape(nb, -1)
    for b in range(nb):
        sb.w_in.upload(psi[b])
        device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
        one = sb.w_out.download()
        assert np.linalg.norm(fp64[b] - one) / np.linalg.norm(one) < 1e-13, b
        assert np.linalg.norm(x3[b] - one) / np.linalg.norm(one) < 2e-5, b
    win.free()
    wout.free()
    sb.free()


def test_full_size_properties(device):
    """The 4x32 Hubbard cylinder at m = 2000 (wave dimension 1.94 M, the
    headline workload), where the oracle is too slow: the FP64 matvec is
    Hermitian and linear, and BF16x3 stays within 2e-5 of FP64."""
    wl = Workload()
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    rng = np.random.default_rng(11)
    n = wl.sup.dim
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    y = rng.normal(size=n) + 1j * rng.normal(size=n)

    def hv(v, prec=_lib.HH_PREC_FP64):
        sb.w_in.upload(v)
        device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, prec))
        return sb.w_out.download()

    hx, hy = hv(x), hv(y)
    lhs, rhs = np.vdot(x, hy), np.conj(np.vdot(y, hx))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    a, b = 0.6 - 0.3j, -1.2 + 0.5j
    hz = hv(a * x + b * y)
    assert np.linalg.norm(hz - (a * hx + b * hy)) < 1e-12 * np.linalg.norm(hz)
    x3 = hv(x, _lib.HH_PREC_BF16X3)
    assert np.linalg.norm(x3 - hx) / np.linalg.norm(hx) < 2e-5
    sb.free()
