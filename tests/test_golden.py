"""Committed golden fixtures (tests/golden/, written by make_golden.py):
known answers of the independent exact diagonalisation and the oracle's
model_wave on seeded synthetic superblocks.  The CPU tests pin the oracle to
them; the GPU tests hold the library to them."""
import json
import os

import numpy as np
import pytest

from oracle import ed
from oracle.lattice import Lattice
from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.synth import Workload
from tests.golden.make_golden import MATVEC_CASES

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ed():
    with open(os.path.join(HERE, "ed_known_answers.json")) as f:
        return json.load(f)


def _green(g):
    return np.array(g["green_re"]) + 1j * np.array(g["green_im"])


def _pair(g):
    return np.array(g["pair_re"]) + 1j * np.array(g["pair_im"])


def _matvec(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    return z["psi"], z["hpsi"]


def test_ed_reproduces_fixture():
    g = _ed()["hubbard_2x4_U8_phi0.25_Ne6"]
    hub = Lattice(2, 4, U=8.0, phi=0.25)
    e, _ = ed.singlet_ground_energy(hub, 6)
    assert e == pytest.approx(g["energy"], abs=1e-12)
    _, ss, _ = ed.hubbard_spin_correlations(hub, 3, 3)
    np.testing.assert_allclose(ss, np.array(g["ss"]), atol=1e-12)
    _, G = ed.hubbard_green(hub, 3, 3)
    np.testing.assert_allclose(G, _green(g), atol=1e-12)
    _, P = ed.hubbard_pair_correlations(hub, 3, 3, [tuple(b) for b in g["pair_bonds"]])
    np.testing.assert_allclose(P, _pair(g), atol=1e-12)
    h = _ed()["tj_2x4_J0.4_phi1/6_Ne6"]
    tj = Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0)
    _, Gt, Pt = ed.tj_singlet_correlations(tj, 6, [tuple(b) for b in h["pair_bonds"]])
    np.testing.assert_allclose(Gt, _green(h), atol=1e-12)
    np.testing.assert_allclose(Pt, _pair(h), atol=1e-12)
    np.testing.assert_allclose(ed.tj_singlet_spin_correlations(tj, 6)[1], np.array(h["ss"]), atol=1e-12)


def test_oracle_dmrg_reproduces_fixture():
    from oracle.dmrg import DMRG
    from oracle import measure as om
    g = _ed()
    d = DMRG(Lattice(2, 4, U=8.0, phi=0.25), 6, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, seed=3)
    assert d.run(sweeps=1) == pytest.approx(g["hubbard_2x4_U8_phi0.25_Ne6"]["energy"], abs=1e-9)
    d.left_to_right(1, 3)
    np.testing.assert_allclose(om.density_correlations(d), np.array(g["hubbard_2x4_U8_phi0.25_Ne6"]["nn"]), atol=1e-6)
    np.testing.assert_allclose(om.electron_correlations_all(d), _green(g["hubbard_2x4_U8_phi0.25_Ne6"]), atol=1e-6)
    h = g["hubbard_2x4_U8_phi0.25_Ne6"]
    bonds = [tuple(b) for b in h["pair_bonds"]]
    np.testing.assert_allclose(om.pairing_correlations(d, bonds[:1], bonds[1:]), _pair(h)[:1, 1:], atol=1e-6)
    t = DMRG(Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0), 6, kept_min=300, kept_max=300, trun_err=1e-14,
             lanzero=1e-11, seed=3)
    assert t.run(sweeps=1) == pytest.approx(g["tj_2x4_J0.4_phi1/6_Ne6"]["energy"], abs=1e-9)
    t.left_to_right(1, 3)
    h = g["tj_2x4_J0.4_phi1/6_Ne6"]
    bonds = [tuple(b) for b in h["pair_bonds"]]
    np.testing.assert_allclose(om.spin_correlations_all(t), np.array(h["ss"]), atol=1e-6)
    np.testing.assert_allclose(om.electron_correlations_all(t), _green(h), atol=1e-6)
    np.testing.assert_allclose(om.pairing_correlations(t, bonds[:1], bonds[1:]), _pair(h)[:1, 1:], atol=1e-6)


@pytest.mark.parametrize("name", sorted(MATVEC_CASES))
def test_oracle_matvec_reproduces_fixture(name):
    import bench
    psi, hpsi = _matvec(name)
    _, got = bench.cpu_matvec_timer(Workload(**MATVEC_CASES[name]), psi, 1)
    assert np.linalg.norm(got - hpsi) / np.linalg.norm(hpsi) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MATVEC_CASES))
def test_gpu_matvec_golden(device, name):
    from hofstadter_hubbard_tsc_gb300.superblock import Superblock
    psi, hpsi = _matvec(name)
    wl = Workload(**MATVEC_CASES[name])
    sb = Superblock(device, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo)
    sb.w_in.upload(psi)
    for prec, tol in ((_lib.HH_PREC_FP64, 1e-12), (_lib.HH_PREC_BF16X6, 5e-6), (_lib.HH_PREC_BF16X3, 2e-5)):
        device.check(device.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, prec))
        got = sb.w_out.download()
        assert np.linalg.norm(got - hpsi) / np.linalg.norm(hpsi) < tol, (name, prec)
    sb.free()


@pytest.mark.gpu
def test_gpu_dmrg_golden(device):
    from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice
    from hofstadter_hubbard_tsc_gb300.measure import Measurement
    from hofstadter_hubbard_tsc_gb300.sweep import GPUDMRG
    g = _ed()["hubbard_2x4_U8_phi0.25_Ne6"]
    lat = SquareLattice(2, 4, U=8.0, phi=0.25)
    d = GPUDMRG(device, lat, 6, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11,
                precision=_lib.HH_PREC_BF16X3)
    assert d.run(sweeps=1) == pytest.approx(g["energy"], abs=1e-8)
    d.left_to_right(1, 3)
    m = Measurement(d)
    np.testing.assert_allclose(m.density_correlations(), np.array(g["nn"]), atol=1e-6)
    np.testing.assert_allclose(m.spin_correlations_all(), np.array(g["ss"]), atol=1e-6)
    np.testing.assert_allclose(m.electron_correlations_all(), _green(g), atol=1e-6)
    bonds = [tuple(b) for b in g["pair_bonds"]]
    np.testing.assert_allclose(m.pairing_correlations(bonds[:1], bonds[1:]), _pair(g)[:1, 1:], atol=1e-6)
