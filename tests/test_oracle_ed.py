"""Pins the oracle: DMRG with m above the exact dimension reproduces exact
diagonalisation singlet energies of small flux ladders and cylinders, and the
free-fermion energy at U=0."""
import numpy as np
import pytest

from oracle import ed
from oracle.lattice import Lattice
from oracle.dmrg import DMRG


def _dmrg(lat, ne, m=256, sweeps=2):
    d = DMRG(lat, ne, kept_min=m, kept_max=m, trun_err=1e-14, lanzero=1e-11, seed=3)
    return d.run(sweeps=sweeps), d


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 3, 4, 0.0, 0.25), (2, 4, 6, 0.0, 0.2)])
def test_free_fermions(W, L, ne, U, phi):
    lat = Lattice(W, L, U=U, phi=phi)
    e, _ = _dmrg(lat, ne)
    assert e == pytest.approx(ed.free_fermion_energy(lat, ne), abs=1e-10)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (4, 2, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_hubbard_exact(W, L, ne, U, phi):
    lat = Lattice(W, L, U=U, phi=phi)
    e, d = _dmrg(lat, ne)
    es, _ = ed.singlet_ground_energy(lat, ne)
    assert e == pytest.approx(es, abs=1e-9)
    # every finite-sweep step sees the same ground state
    finals = [r[2] for r in d.energies[-4:]]
    assert np.ptp(finals) < 1e-9


@pytest.mark.parametrize("W,L,ne,phi", [(2, 3, 4, 1.0 / 6.0), (2, 4, 6, 1.0 / 6.0), (4, 2, 6, 0.25)])
def test_tj_exact(W, L, ne, phi):
    """t-J model (J = 0.4, the t-J configuration's coupling): the oracle DMRG
    against a Fock-basis t-J diagonalisation with no double occupancy and
    J (S_i.S_j - n_i n_j / 4) on every bond."""
    lat = Lattice(W, L, model="tj", J=0.4, U=0.0, phi=phi)
    e, _ = _dmrg(lat, ne, m=300, sweeps=1)
    assert e == pytest.approx(ed.tj_singlet_ground_energy(lat, ne), abs=1e-9)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_measurements_exact(W, L, ne, U, phi):
    """measure_operator_dia and the cross-cut density correlations of the
    oracle against the exact ground state (Fock basis)."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    _, dens, corr = ed.hubbard_density_correlations(lat, ne // 2, ne // 2)
    _, d = _dmrg(lat, ne, sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    prof = om.site_profile(d)
    assert prof.sum() == pytest.approx(ne, abs=1e-10)
    np.testing.assert_allclose(prof, dens, atol=1e-6)
    sa, sb, m = om.cross_correlations(d)
    np.testing.assert_allclose(m, corr[np.ix_(np.array(sa) - 1, np.array(sb) - 1)], atol=1e-6)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_spin_correlations_exact(W, L, ne, U, phi):
    """Cross-cut <S_a . S_b> of the oracle (carried rank-1 operators, the S.S
    bond kernels, -sqrt(3) normalisation) against the exact ground state; the
    exact state is a singlet (<S.S> = 3 <Sz Sz>)."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    _, ss, szsz3 = ed.hubbard_spin_correlations(lat, ne // 2, ne // 2)
    np.testing.assert_allclose(ss, szsz3, atol=1e-12)
    _, d = _dmrg(lat, ne, sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    sa, sb, m = om.spin_correlations(d)
    np.testing.assert_allclose(m, ss[np.ix_(np.array(sa) - 1, np.array(sb) - 1)], atol=1e-6)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_density_correlations_all_pairs(W, L, ne, U, phi):
    """<n_i n_j> for every pair (same-side products, cross-cut and diagonal)
    of the oracle against the exact ground state."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    _, _, corr = ed.hubbard_density_correlations(lat, ne // 2, ne // 2)
    _, d = _dmrg(lat, ne, sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    np.testing.assert_allclose(om.density_correlations(d), corr, atol=1e-6)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_spin_correlations_all_pairs(W, L, ne, U, phi):
    """<S_i . S_j> for every pair (same-side bond products, block-site terms,
    cross-cut, diagonal) of the oracle against the exact ground state."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    _, ss, _ = ed.hubbard_spin_correlations(lat, ne // 2, ne // 2)
    _, d = _dmrg(lat, ne, sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    np.testing.assert_allclose(om.spin_correlations_all(d), ss, atol=1e-6)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_electron_correlations_exact(W, L, ne, U, phi):
    """Cross-cut G_ab = sum_s <c+_as c_bs> of the oracle (fermion operators
    carried with the 'F' ndia embeddings, the hopping kernels with
    coefficients 1 and i) against the exact ground state; the exact G is
    Hermitian with trace N_e and carries the flux phases (complex)."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    e0, G = ed.hubbard_green(lat, ne // 2, ne // 2)
    np.testing.assert_allclose(G, G.conj().T, atol=1e-12)
    assert np.trace(G).real == pytest.approx(ne, abs=1e-10)
    assert np.abs(G.imag).max() > 1e-3
    e, d = _dmrg(lat, ne, sweeps=1)
    assert e == pytest.approx(e0, rel=1e-10)
    d.left_to_right(1, lat.N // 2 - 1)
    sa, sb, m = om.electron_correlations(d)
    np.testing.assert_allclose(m, G[np.ix_(np.array(sa) - 1, np.array(sb) - 1)], atol=1e-6)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 3, 4, 4.0, 0.3)])
def test_electron_correlations_all_pairs(W, L, ne, U, phi):
    """G_ij = sum_s <c+_is c_js> for every pair (same-side hopping bonds
    formed in the enlarged basis, block-middle-site hopping terms, cross-cut,
    diagonal) of the oracle against the exact ground state."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    _, G = ed.hubbard_green(lat, ne // 2, ne // 2)
    _, d = _dmrg(lat, ne, sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    m = om.electron_correlations_all(d)
    np.testing.assert_allclose(m, m.conj().T, atol=1e-12)
    np.testing.assert_allclose(m, G, atol=1e-6)


PAIR_SYS = [(1, 2)]
PAIR_ENV = [(8, 7), (7, 6), (6, 5), (8, 6), (7, 5), (8, 5)]


@pytest.mark.parametrize("W,L,nu,phi", [(2, 3, 2, 0.0), (2, 4, 3, 0.25)])
def test_exact_pair_correlations_wick(W, L, nu, phi):
    """At U = 0 (a single Slater determinant per spin) the exact singlet-pair
    correlation is <D+_ab D_cd> = g_ac g_bd + g_ad g_bc with the per-spin
    one-body matrix g = G / 2."""
    lat = Lattice(W, L, U=0.0, phi=phi)
    bonds = [(1, 2), (1, 3), (2, 4), (3, 5), (4, 6), (5, 6)]
    _, P = ed.hubbard_pair_correlations(lat, nu, nu, bonds)
    _, G = ed.hubbard_green(lat, nu, nu)
    g = G / 2
    wick = np.array([[g[a - 1, c - 1] * g[b - 1, d - 1] + g[a - 1, d - 1] * g[b - 1, c - 1] for (c, d) in bonds]
                     for (a, b) in bonds])
    np.testing.assert_allclose(P, wick, atol=1e-12)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 4, 4, 4.0, 0.3), (2, 4, 8, 4.0, 0.0)])
def test_pairing_correlations_exact(W, L, ne, U, phi):
    """Cross-cut singlet-pair correlations of the oracle (pair creators as
    rank-0 products of two elec_up operators, block_mul_block_ndia; the
    measurement of sys_block_env_block_cor_ndia) against the exact ground
    state: the reference's reduced normalisation is <D+_x D_y> with
    D+_ij = (c+_i,up c+_j,dn - c+_i,dn c+_j,up) / sqrt(2)."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    e0, P = ed.hubbard_pair_correlations(lat, ne // 2, ne // 2, PAIR_SYS + PAIR_ENV)
    e, d = _dmrg(lat, ne, sweeps=1)
    assert e == pytest.approx(e0, rel=1e-10)
    d.left_to_right(1, lat.N // 2 - 1)
    m = om.pairing_correlations(d, PAIR_SYS, PAIR_ENV)
    np.testing.assert_allclose(m, P[:len(PAIR_SYS), len(PAIR_SYS):], atol=1e-6)
    with pytest.raises(ValueError):
        om.pairing_correlations(d, [(2, 3)], PAIR_ENV)


@pytest.mark.parametrize("W,L,ne,U,phi", [(2, 4, 6, 8.0, 0.25), (2, 4, 8, 4.0, 0.0)])
def test_pairing_correlations_same_side_exact(W, L, ne, U, phi):
    """Same-side singlet-pair correlations of the oracle (the pair creator of
    the first bond multiplied by the second bond's two elec_down operators,
    ranks 1/2 then 0, measured with measure_sys_block) against the exact
    ground state, on a superblock with four system block sites."""
    from oracle import measure as om
    lat = Lattice(W, L, U=U, phi=phi)
    _, P = ed.hubbard_pair_correlations(lat, ne // 2, ne // 2, [(1, 2), (3, 4)])
    _, d = _dmrg(lat, ne, sweeps=1)
    d.left_to_right(1, 5)
    assert d.wave.sys_len == 5
    m = om.pairing_correlations_sys(d, [(1, 2)], [(3, 4)])
    np.testing.assert_allclose(m, P[:1, 1:], atol=1e-6)
    with pytest.raises(ValueError):
        om.pairing_correlations_sys(d, [(1, 3)], [(2, 4)])


def test_tj_electron_and_pairing_correlations_exact():
    """t-J ladder (projected site operators): the oracle's electron
    correlations for all pairs and its cross-cut and same-side singlet-pair
    correlations against the exact singlet ground state."""
    from oracle import measure as om
    lat = Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0)
    bonds = PAIR_SYS + PAIR_ENV + [(3, 4)]
    e0, G, P = ed.tj_singlet_correlations(lat, 6, bonds)
    np.testing.assert_allclose(G, G.conj().T, atol=1e-12)
    assert np.trace(G).real == pytest.approx(6.0, abs=1e-10)
    e, d = _dmrg(lat, 6, m=300, sweeps=1)
    assert e == pytest.approx(e0, abs=1e-9)
    d.left_to_right(1, lat.N // 2 - 1)
    np.testing.assert_allclose(om.electron_correlations_all(d), G, atol=1e-6)
    np.testing.assert_allclose(om.pairing_correlations(d, PAIR_SYS, PAIR_ENV), P[:1, 1:7], atol=1e-6)
    _, d = _dmrg(lat, 6, m=300, sweeps=1)
    d.left_to_right(1, 5)
    np.testing.assert_allclose(om.pairing_correlations_sys(d, [(1, 2)], [(3, 4)]), P[:1, 7:], atol=1e-6)


@pytest.mark.parametrize("W,L,cut", [(2, 4, 0), (2, 6, 1), (4, 5, 1), (3, 4, 0)])
def test_structure_factor_matches_oracle(W, L, cut):
    """The host structure factor (vectorised) equals the oracle's restatement
    of Get_structure_factor_cut on a random complex matrix (real part used);
    a diagonal C = c 1 gives S = c at every k."""
    from oracle import measure as om
    from hofstadter_hubbard_tsc_gb300.measure import structure_factor
    rng = np.random.default_rng(W * 100 + L * 10 + cut)
    N = W * L
    C = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    kx, ky, S = structure_factor(C, W, L, cut)
    np.testing.assert_allclose(S, om.structure_factor_cut(C, W, L, cut), atol=1e-12)
    assert kx[0] == 0.0 and kx[-1] == pytest.approx(2.0) and ky[-1] == pytest.approx(2.0)
    _, _, S1 = structure_factor(0.7 * np.eye(N), W, L, cut)
    np.testing.assert_allclose(S1, 0.7, atol=1e-12)
    with pytest.raises(ValueError):
        structure_factor(C[:-1, :-1], W, L, cut)


def test_spin_structure_factor_sum_rule():
    """For the exact singlet, sum_j <S_i . S_j> = 0 for every i (total spin
    zero), so the spin structure factor at k = 0 over the whole ladder
    vanishes."""
    from hofstadter_hubbard_tsc_gb300.measure import structure_factor
    lat = Lattice(2, 4, U=8.0, phi=0.25)
    _, ss, _ = ed.hubbard_spin_correlations(lat, 3, 3)
    _, _, S = structure_factor(ss, 2, 4, 0)
    assert abs(S[0, 0]) < 1e-10
    assert S.max() > 0.1


def test_tj_spin_correlations_all_pairs():
    """t-J ladder: the oracle's <S_i . S_j> for every pair against the exact
    singlet ground state (rows sum to zero: total spin 0)."""
    from oracle import measure as om
    lat = Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0)
    _, ss = ed.tj_singlet_spin_correlations(lat, 6)
    np.testing.assert_allclose(ss.sum(axis=1), 0.0, atol=1e-10)
    _, d = _dmrg(lat, 6, m=300, sweeps=1)
    d.left_to_right(1, lat.N // 2 - 1)
    np.testing.assert_allclose(om.spin_correlations_all(d), ss, atol=1e-6)
