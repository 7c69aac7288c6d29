"""Measurements on the GPU DMRG state (measure_operator_dia and the cross-cut
part of Get_density_cor) against the exact ground state, and the sum rule on a
truncated run."""
import numpy as np
import pytest

from oracle import ed
from oracle.lattice import Lattice
from hofstadter_hubbard_tsc_gb300 import _lib
from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice
from hofstadter_hubbard_tsc_gb300.measure import Measurement
from hofstadter_hubbard_tsc_gb300.sweep import GPUDMRG

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_density_profile_and_correlations_exact(device, precision):
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, dens, corr = ed.hubbard_density_correlations(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2)
    m = Measurement(d)
    prof = m.site_profile("num_elec")
    assert prof.sum() == pytest.approx(ne, abs=1e-9)
    np.testing.assert_allclose(prof, dens, atol=1e-6)
    sa, sb, c = m.cross_correlations("num_elec", "num_elec")
    np.testing.assert_allclose(c, corr[np.ix_(np.array(sa) - 1, np.array(sb) - 1)], atol=1e-6)


def test_profile_sum_rules_truncated(device):
    """m = 48 on a 2x8 ladder: <n_i> sums to N_e, <n_a n_b> summed over the
    environment half equals <n_a N_env>, and double occupancy stays in [0, <n_i>/2]."""
    lat = SquareLattice(2, 8, U=8.0, phi=0.25)
    d = GPUDMRG(device, lat, 14, kept_min=48, kept_max=48, trun_err=1e-12, lanzero=1e-10)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    m = Measurement(d)
    n = m.site_profile("num_elec")
    assert n.sum() == pytest.approx(14.0, abs=1e-8)
    dbl = m.site_profile("double")
    assert np.all(dbl >= -1e-10) and np.all(dbl <= n / 2 + 1e-10)
    sa, sb, c = m.cross_correlations()
    assert np.all(np.isfinite(c))
    # sum_b <n_a n_b> <= <n_a> * max particles on the environment side
    assert np.all(c.sum(axis=1) <= n[np.array(sa) - 1] * 2 * len(sb) + 1e-8)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_spin_correlations_exact(device, precision):
    """Cross-cut <S_a . S_b> on the GPU state (rank-1 operators carried with
    the ndia embeddings, one-term S.S plans) against exact diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, ss, _ = ed.hubbard_spin_correlations(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2)
    sa, sb, m = Measurement(d).spin_correlations()
    np.testing.assert_allclose(m, ss[np.ix_(np.array(sa) - 1, np.array(sb) - 1)], atol=1e-6)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_density_correlations_all_pairs(device, precision):
    """<n_i n_j> for every pair (same-side carried products, cross-cut,
    diagonal) on the GPU state against exact diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, _, corr = ed.hubbard_density_correlations(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2)
    np.testing.assert_allclose(Measurement(d).density_correlations(), corr, atol=1e-6)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_spin_correlations_all_pairs(device, precision):
    """<S_i . S_j> for every pair on the GPU state against exact
    diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, ss, _ = ed.hubbard_spin_correlations(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2)
    np.testing.assert_allclose(Measurement(d).spin_correlations_all(), ss, atol=1e-6)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_electron_correlations_exact(device, precision):
    """Cross-cut G_ab = sum_s <c+_as c_bs> on the GPU state (fermion
    operators carried with the 'F' ndia embeddings, one-term hopping plans
    with coefficients 1 and i) against exact diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, G = ed.hubbard_green(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2)
    sa, sb, m = Measurement(d).electron_correlations()
    np.testing.assert_allclose(m, G[np.ix_(np.array(sa) - 1, np.array(sb) - 1)], atol=1e-6)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_electron_correlations_all_pairs(device, precision):
    """G_ij = sum_s <c+_is c_js> for every pair on the GPU state against exact
    diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, G = ed.hubbard_green(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2)
    np.testing.assert_allclose(Measurement(d).electron_correlations_all(), G, atol=1e-6)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_pairing_correlations_exact(device, precision):
    """Cross-cut singlet-pair correlations on the GPU state (pair creators
    from hh_block_product, one-term block-block plans with coefficients 1 and
    i) against exact diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    sys_bonds = [(1, 2)]
    env_bonds = [(8, 7), (7, 6), (6, 5), (8, 6), (7, 5), (8, 5)]
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    _, P = ed.hubbard_pair_correlations(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2, sys_bonds + env_bonds)
    m = Measurement(d)
    np.testing.assert_allclose(m.pairing_correlations(sys_bonds, env_bonds), P[:1, 1:], atol=1e-6)
    with pytest.raises(ValueError):
        m.pairing_correlations([(2, 3)], env_bonds)


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_pairing_correlations_same_side_exact(device, precision):
    """Same-side singlet-pair correlations on the GPU state (products of the
    pair creator with two elec_down operators by hh_block_product, the scalar
    measured by block_vec_dia plans) against exact diagonalisation."""
    W, L, ne, U, phi = 2, 4, 6, 8.0, 0.25
    lat = SquareLattice(W, L, U=U, phi=phi)
    d = GPUDMRG(device, lat, ne, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, precision=precision)
    d.run(sweeps=1)
    d.left_to_right(1, 5)
    _, P = ed.hubbard_pair_correlations(Lattice(W, L, U=U, phi=phi), ne // 2, ne // 2, [(1, 2), (3, 4)])
    m = Measurement(d)
    assert m.Ls == 4
    np.testing.assert_allclose(m.pairing_correlations_sys([(1, 2)], [(3, 4)]), P[:1, 1:], atol=1e-6)
    with pytest.raises(ValueError):
        m.pairing_correlations_sys([(1, 3)], [(2, 4)])


@pytest.mark.parametrize("precision", [_lib.HH_PREC_FP64, _lib.HH_PREC_BF16X3])
def test_tj_electron_and_pairing_correlations_exact(device, precision):
    """t-J ladder (projected site operators) on the GPU: electron and spin
    correlations for all pairs, cross-cut and same-side singlet-pair
    correlations against the exact singlet ground state."""
    lat_o = Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0)
    sys_bonds, env_bonds = [(1, 2)], [(8, 7), (7, 6), (6, 5), (8, 6), (7, 5), (8, 5)]
    _, G, P = ed.tj_singlet_correlations(lat_o, 6, sys_bonds + env_bonds + [(3, 4)])

    def state(end):
        d = GPUDMRG(device, SquareLattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0), 6, kept_min=300,
                    kept_max=300, trun_err=1e-14, lanzero=1e-11, precision=precision)
        d.run(sweeps=1)
        d.left_to_right(1, end)
        return Measurement(d)

    m = state(lat_o.N // 2 - 1)
    np.testing.assert_allclose(m.electron_correlations_all(), G, atol=1e-6)
    _, ss = ed.tj_singlet_spin_correlations(lat_o, 6)
    np.testing.assert_allclose(m.spin_correlations_all(), ss, atol=1e-6)
    np.testing.assert_allclose(m.pairing_correlations(sys_bonds, env_bonds), P[:1, 1:7], atol=1e-6)
    m = state(5)
    np.testing.assert_allclose(m.pairing_correlations_sys([(1, 2)], [(3, 4)]), P[:1, 7:], atol=1e-6)
