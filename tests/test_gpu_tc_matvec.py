"""Split-precision (BF16x6: three BF16 parts, BF16x3: two; tcgen05) model_wave
against the FP64 path on oracle DMRG superblocks, and its Lanczos energy
against the FP64 Lanczos."""
import ctypes as C

import numpy as np
import pytest

from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.superblock import Superblock
from tests import helpers as H

pytestmark = pytest.mark.gpu

# BF16x6: 24-bit split operands, FP32 accumulation (FP32 level); BF16x3:
# dropped x1 y1 terms and 16-bit operands, about 2^-16 per product
RTOL = {_lib.HH_PREC_BF16X6: 5e-6, _lib.HH_PREC_BF16X3: 2e-5}
SPLITS = [_lib.HH_PREC_BF16X6, _lib.HH_PREC_BF16X3]


@pytest.mark.parametrize("precision", SPLITS)
def test_tc_matvec_matches_fp64(device, precision):
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    for idx, rec in enumerate(d.record[::2]):
        sys, env, sys_bs, env_bs, geo, sup, _ = rec
        sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                        H.superbasis(sup), plat.geometry(sys.len, env.len))
        x = H.wave(H.random_wave(sup, idx))
        a = sb.model_wave(x, precision=_lib.HH_PREC_FP64).flat()
        b = sb.model_wave(x, precision=precision).flat()
        err = np.linalg.norm(a - b) / np.linalg.norm(a)
        assert err < RTOL[precision], (idx, err)
        sb.free()


@pytest.mark.parametrize("precision", SPLITS)
def test_tc_matvec_synthetic_m200(device, precision):
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    wl = Workload(W=4, L=8, n_elec=28, m=200)
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    rng = np.random.default_rng(3)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    sb.w_in.upload(psi)
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
    ref = sb.w_out.download()
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, precision))
    got = sb.w_out.download()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < RTOL[precision]
    # switching precision on one plan re-captures the matvec graph
    for pr in (precision, SPLITS[0] if precision != SPLITS[0] else SPLITS[1], precision):
        device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, pr))
        got = sb.w_out.download()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < RTOL[pr]
    assert device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, 7) == -1
    sb.free()


def test_tc_tile_shapes_and_tuner(device):
    """Every stage-2 tile shape (128 x 64, near-equal stacked tiles of at most
    64 rows, the mixed split, 128 x 128) gives the FP64 product within the
    split precision's tolerance, eagerly and on graph replay; the autotuner
    times every shape and launch variant and keeps one whose products agree."""
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    wl = Workload(W=4, L=8, n_elec=28, m=300)
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    rng = np.random.default_rng(11)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    sb.w_in.upload(psi)
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
    ref = sb.w_out.download()
    for shape in range(_lib.HH_TILE_SHAPES):
        device.check(device.lib.hh_plan_set_tiles(sb.plan, shape))
        for pr in SPLITS:
            for _ in range(3):  # eager first call, then graph capture and replay
                device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, pr))
                got = sb.w_out.download()
                assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < RTOL[pr], (shape, pr)
    assert device.lib.hh_plan_set_tiles(sb.plan, _lib.HH_TILE_SHAPES) == -1
    ms = np.zeros(_lib.HH_TUNE_VARIANTS)
    choice = C.c_int(-1)
    device.check(device.lib.hh_plan_tune(sb.plan, _lib.HH_PREC_BF16X3, 1, ms.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.byref(choice)))
    assert 0 <= choice.value < _lib.HH_TUNE_VARIANTS and np.all(ms > 0)
    assert ms[choice.value] == ms.min()
    for _ in range(2):
        device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_BF16X3))
        got = sb.w_out.download()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < RTOL[_lib.HH_PREC_BF16X3]
    sb.free()


@pytest.mark.parametrize("precision", SPLITS)
def test_tc_lanczos_energy(device, precision):
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    rec = d.record[-3]
    sys, env, sys_bs, env_bs, geo, sup, _ = rec
    sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                    H.superbasis(sup), plat.geometry(sys.len, env.len))
    start = H.wave(H.random_wave(sup, 9))
    e64, _, _ = sb.lanczos_memo_new(H.wave(H.random_wave(sup, 9)), 1e-10, precision=_lib.HH_PREC_FP64)
    emx, _, _ = sb.lanczos_memo_new(start, 1e-8, precision=precision)
    assert abs(emx - e64) / abs(e64) < 1e-8, (emx, e64)
    sb.free()


def test_fp32x2_matvec_and_restart(device):
    """The double-float product (HH_PREC_FP32X2: FP64 operands as sums of two
    floats, exact FMA residuals and TwoSum on the FP32 pipe) equals the FP64
    product to FP64-class accuracy on oracle superblocks and a synthetic
    m = 200 superblock; the split Lanczos with its restart product in
    double-float (the default) or FP64 gives the FP64 energy, and a Lanczos run
    wholly in double-float too."""
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    for idx, rec in enumerate(d.record[::3]):
        sys, env, sys_bs, env_bs, geo, sup, _ = rec
        sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                        H.superbasis(sup), plat.geometry(sys.len, env.len))
        x = H.wave(H.random_wave(sup, idx))
        a = sb.model_wave(x, precision=_lib.HH_PREC_FP64).flat()
        b = sb.model_wave(x, precision=_lib.HH_PREC_FP32X2).flat()
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-13, idx
        sb.free()
    wl = Workload(W=4, L=8, n_elec=28, m=200)
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    rng = np.random.default_rng(4)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    sb.w_in.upload(psi)
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
    ref = sb.w_out.download()
    device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP32X2))
    got = sb.w_out.download()
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    # N(0,1) operators, sums of several hundred products per element: a few
    # 2^-48 roundings each
    assert err < 5e-13, err
    sb.free()

    assert device.lib.hh_ctx_set_restart_precision(device.h, _lib.HH_PREC_BF16X3) == -1
    rec = d.record[-3]
    sys, env, sys_bs, env_bs, geo, sup, _ = rec
    sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                    H.superbasis(sup), plat.geometry(sys.len, env.len))
    e64, _, _ = sb.lanczos_memo_new(H.wave(H.random_wave(sup, 9)), 1e-10, precision=_lib.HH_PREC_FP64)
    edf, _, _ = sb.lanczos_memo_new(H.wave(H.random_wave(sup, 9)), 1e-10, precision=_lib.HH_PREC_FP32X2)
    assert abs(edf - e64) / abs(e64) < 1e-11, (edf, e64)
    try:
        for rp in (_lib.HH_PREC_FP64, _lib.HH_PREC_FP32X2):
            for ks in (_lib.HH_PREC_FP64, _lib.HH_PREC_FP32):  # first pass's Krylov basis
                device.check(device.lib.hh_ctx_set_restart_precision(device.h, rp))
                device.check(device.lib.hh_ctx_set_krylov_storage(device.h, ks))
                emx, _, _ = sb.lanczos_memo_new(H.wave(H.random_wave(sup, 9)), 1e-10, precision=_lib.HH_PREC_BF16X3)
                assert abs(emx - e64) / abs(e64) < 1e-10, (rp, ks, emx, e64)
    finally:
        device.check(device.lib.hh_ctx_set_restart_precision(device.h, _lib.HH_PREC_FP32X2))
        device.check(device.lib.hh_ctx_set_krylov_storage(device.h, _lib.HH_PREC_FP32))
    assert device.lib.hh_ctx_set_krylov_storage(device.h, _lib.HH_PREC_BF16X3) == -1
    sb.free()
