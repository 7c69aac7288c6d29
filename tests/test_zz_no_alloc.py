"""hh_matvec_noalloc, the allocation-free matvec for callers that cannot call
cudaMalloc at multiplication time (a Fortran code whose own pool already owns
the GPU's memory, or one that reserves a fixed device budget), gives the same
H psi as hh_matvec and reserves no device memory while it runs.

Both entry points are called through the C ABI on the same plan and input,
twice in a row (the static scratch keeps the previous call's contents, which
must not leak into the next result), on single waves and on a wave of two
vectors.  The file sorts last so that a run that stops at the first failure
has already run every other test; it also passes alone in a fresh process."""
import numpy as np
import pytest

from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.device import DWave
from hofstadter_hubbard_tsc_gb300.superblock import Superblock
from tests import helpers as H

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _superblocks(device):
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    for rec in (d.record[-3], d.record[-2]):
        sys, env, sys_bs, env_bs, geo, sup, _ = rec
        sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                        H.superbasis(sup), plat.geometry(sys.len, env.len))
        yield sb, sup
        sb.free()


def test_noalloc_matches_matvec(device):
    lib = device.lib
    for sb, sup in _superblocks(device):
        w_ref = DWave(device, sb.layout, sup.sys_len, sup.env_len)
        w_na = DWave(device, sb.layout, sup.sys_len, sup.env_len)
        for call in range(2):
            psi = H.wave(H.random_wave(sup, 100 + call)).flat()
            sb.w_in.upload(psi)
            device.check(lib.hh_matvec(sb.plan, sb.w_in.h, w_ref.h, _lib.HH_PREC_FP64))
            device.check(lib.hh_matvec_noalloc(sb.plan, sb.w_in.h, w_na.h))
            device.sync()
            a, b = w_na.download(), w_ref.download()
            err = np.linalg.norm(a - b) / np.linalg.norm(b)
            assert err < RTOL, (call, err)
        w_ref.free()
        w_na.free()


def test_noalloc_batched_wave(device):
    """A wave of two vectors: both products equal hh_matvec's, on two calls in
    a row; waves holding different numbers of vectors are rejected."""
    lib = device.lib
    for sb, sup in _superblocks(device):
        n = sb.w_in.nelem
        w_in = DWave(device, sb.layout, sup.sys_len, sup.env_len, nbatch=2)
        w_ref = DWave(device, sb.layout, sup.sys_len, sup.env_len, nbatch=2)
        w_na = DWave(device, sb.layout, sup.sys_len, sup.env_len, nbatch=2)
        for call in range(2):
            psi = np.concatenate([H.wave(H.random_wave(sup, 200 + 2 * call + k)).flat() for k in range(2)])
            w_in.upload(psi)
            device.check(lib.hh_matvec(sb.plan, w_in.h, w_ref.h, _lib.HH_PREC_FP64))
            device.check(lib.hh_matvec_noalloc(sb.plan, w_in.h, w_na.h))
            device.sync()
            a, b = w_na.download(), w_ref.download()
            for k in range(2):
                ak, bk = a[k * n:(k + 1) * n], b[k * n:(k + 1) * n]
                err = np.linalg.norm(ak - bk) / np.linalg.norm(bk)
                assert err < RTOL, (call, k, err)
        assert lib.hh_matvec_noalloc(sb.plan, w_in.h, sb.w_out.h) == _lib.HH_ERR_INVALID
        for w in (w_in, w_ref, w_na):
            w.free()


def test_noalloc_reserves_no_memory(device):
    """Free device memory is the same before and after calls of the entry
    point, the first one included (the static array's module is loaded by
    hh_init, when the context is created)."""
    import torch
    torch.cuda.init()
    torch.cuda.mem_get_info()
    lib = device.lib
    for sb, sup in _superblocks(device):
        w_na = DWave(device, sb.layout, sup.sys_len, sup.env_len)
        sb.w_in.upload(H.wave(H.random_wave(sup, 300)).flat())
        device.sync()
        before, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            device.check(lib.hh_matvec_noalloc(sb.plan, sb.w_in.h, w_na.h))
        device.sync()
        after, _ = torch.cuda.mem_get_info()
        assert after == before, (before, after)
        w_na.free()


def test_noalloc_rejects_oversized_plan(device):
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    wl = Workload(m=2000)
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    if sb.stats()["scratch_bytes"] <= (64 << 20):
        pytest.skip("this plan fits the static scratch")
    st = device.lib.hh_matvec_noalloc(sb.plan, sb.w_in.h, sb.w_out.h)
    assert st == _lib.HH_ERR_INVALID
    assert b"static buffer" in device.lib.hh_last_error(device.h)
    sb.free()
