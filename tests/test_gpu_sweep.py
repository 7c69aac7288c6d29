"""Whole DMRG on the GPU (enlargement, Lanczos, truncation, renormalisation,
wave transforms all in libhh_dmrg.so) against exact diagonalisation and the
oracle DMRG."""
import numpy as np
import pytest

from oracle import ed
from oracle.lattice import Lattice
from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice
from hofstadter_hubbard_tsc_gb300.sweep import GPUDMRG

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (4, 2, 6, 8.0, 0.25)])
def test_gpu_dmrg_exact(device, W, L, ne, U, phi):
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11)
    e = d.run(sweeps=1)
    es, _ = ed.singlet_ground_energy(Lattice(W, L, U=U, phi=phi), ne)
    assert e == pytest.approx(es, abs=1e-8)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X6, _lib.HH_PREC_BF16X3])
def test_gpu_dmrg_tj_exact(device, precision):
    lat = SquareLattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0)
    d = GPUDMRG(device, lat, 6, kept_min=300, kept_max=300, trun_err=1e-14, lanzero=1e-11, precision=precision)
    e = d.run(sweeps=1)
    es = ed.tj_singlet_ground_energy(Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0), 6)
    assert e == pytest.approx(es, abs=1e-8)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_BF16X6, _lib.HH_PREC_BF16X3])
def test_gpu_dmrg_split_precision(device, precision):
    lat = SquareLattice(2, 6, U=8.0, phi=0.25)
    d64 = GPUDMRG(device, lat, 10, kept_min=48, kept_max=48, trun_err=1e-14, lanzero=1e-10)
    e64 = d64.run(sweeps=1)
    dmx = GPUDMRG(device, lat, 10, kept_min=48, kept_max=48, trun_err=1e-14, lanzero=1e-8,
                  precision=precision)
    emx = dmx.run(sweeps=1)
    assert abs(emx - e64) / abs(e64) < 1e-8, (emx, e64)


def test_checkpoint_resume(device, tmp_path):
    """save after the half sweeps, load into a fresh driver, sweep both: the
    resumed run reproduces the uninterrupted one."""
    lat = SquareLattice(2, 6, U=8.0, phi=0.25)
    kw = dict(kept_min=32, kept_max=32, trun_err=1e-12, lanzero=1e-10, precision=_lib.HH_PREC_BF16X3)
    a = GPUDMRG(device, lat, 10, **kw)
    a.run(sweeps=0)
    a.save(str(tmp_path / "ckpt"))
    b = GPUDMRG(device, lat, 10, **kw)
    b.load(str(tmp_path / "ckpt"))
    a.sweep()
    b.sweep()
    ea = [r[2] for r in a.energies[-2 * (lat.N - 3):]]
    eb = [r[2] for r in b.energies[-2 * (lat.N - 3):]]
    np.testing.assert_allclose(eb, ea, rtol=0, atol=1e-12)
