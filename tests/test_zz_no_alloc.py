"""hh_matvec_noalloc, the allocation-free matvec for callers that cannot call
cudaMalloc at multiplication time, gives the same H psi as hh_matvec.

Both entry points are called through the C ABI on the same plan and input,
twice in a row (the static scratch keeps the previous call's contents, which
must not leak into the next result).  The file sorts last so that a run that
stops at the first failure has already run every other test; it also passes
alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.device import DWave
from hofstadter_hubbard_tsc_gb300.superblock import Superblock
from tests import helpers as H

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def test_noalloc_matches_matvec(device):
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    lib = device.lib
    for rec in (d.record[-3], d.record[-2]):
        sys, env, sys_bs, env_bs, geo, sup, _ = rec
        sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                        H.superbasis(sup), plat.geometry(sys.len, env.len))
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
        sb.free()


def test_noalloc_rejects_oversized_plan(device):
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    wl = Workload(m=2000)
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    if sb.stats()["scratch_bytes"] <= (64 << 20):
        pytest.skip("this plan fits the static scratch")
    st = device.lib.hh_matvec_noalloc(sb.plan, sb.w_in.h, sb.w_out.h)
    assert st == -1
    assert b"static buffer" in device.lib.hh_last_error(device.h)
    sb.free()
