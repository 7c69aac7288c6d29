"""SU(2) -> Fock-basis expansion of the oracle's reduced states: a known answer
for model_wave vector by vector.

Every reduced multiplet state of a block is expanded into the Fock space of
its sites, recursively over the enlargements and truncations of an oracle
DMRG run: an enlarged state of total spin S, projection M, is
sum CG(S_b m_b, S_s m_s | S M) |block; S_b m_b> |site; S_s m_s>, and a
block state is a column of the truncation operator over the enlarged states.
Conventions that reproduce the reference's reduced matrices (found by
requiring the block Hamiltonians to match, and then fixed here):
  * site multiplets |0>, (c+_up|0>, c+_dn|0>) for (M = 1/2, -1/2), c+_up c+_dn|0>;
  * fermion modes in ascending site order, up before down within a site,
    no extra sign between a block and its new site;
  * environment basis vectors are the complex conjugates of the recursion's,
    and an environment block stores the complex conjugate of its matrix
    elements in that basis (its operators act from the right, psi O^H, in
    vec_block_dia and its siblings, code/mat_vec.f90:218-267);
  * the superblock singlet is sum_m CG(S m, S -m | 0 0) |sys; S m> |env; S -m>.
The superblock H psi of the oracle then equals the dense Fock-space
Hamiltonian applied to the expanded psi."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import ed
from oracle.su2 import cg
from tests import helpers as H


def _site_states():
    e = np.eye(4)
    return {(0, 0): e[0][None, :, None], (1, 1): np.stack([e[1], e[2]])[:, :, None], (2, 0): e[3][None, :, None]}


def _enlarge(block, basis, trun, site, nb, block_low):
    """Components (2S+1, 4^(nb+1), dim) of every enlarged sector, truncated
    with trun when it is given."""
    enl = {}
    for sec in basis.sectors:
        S2 = sec.new_num_down
        arr = np.zeros((S2 + 1, 4 ** (nb + 1), sec.dim), dtype=complex)
        for sb in sec.subs:
            B = block[(sb.bl_num_up, sb.bl_num_down)]
            X = site[(sb.st_num_up, sb.st_num_down)][:, :, 0]
            jb, js = sb.bl_num_down, sb.st_num_down
            for k in range(S2 + 1):
                M = S2 - 2 * k
                for kb in range(jb + 1):
                    mb = jb - 2 * kb
                    ms = M - mb
                    if abs(ms) > js or (js - ms) % 2:
                        continue
                    c = cg(jb, mb, js, ms, S2, M)
                    if c == 0.0:
                        continue
                    ks = (js - ms) // 2
                    for j in range(sb.sdim):
                        if block_low:   # block sites below the new site
                            v = np.outer(X[ks], B[kb][:, j]).ravel()
                        else:           # new site below the block sites
                            v = np.outer(B[kb][:, j], X[ks]).ravel()
                        arr[k, :, sb.spos + j] += c * v
        enl[(sec.new_num_up, S2)] = arr
    if trun is None:
        return enl
    return {(s.num_up, s.num_down): np.einsum("kfb,bc->kfc", enl[(s.num_up, s.num_down)], s.mat) for s in trun.subs}


def _expand(bases, truns, length, block_low, truncate_last, last_basis=None):
    """Block states of `length` sites (truncate_last) or the enlarged basis
    of that length (last_basis, default bases[length])."""
    site = _site_states()
    blk = dict(site)
    for nb in range(1, length):
        last = nb + 1 == length
        trun = truns[nb + 1] if (truncate_last or not last) else None
        basis = last_basis if (last and last_basis is not None) else bases[nb + 1]
        blk = _enlarge(blk, basis, trun, site, nb, block_low)
    return blk


def _fock_hamiltonian(lat, sites, n_elec=None):
    """-t sum (phase c+_i c_j + h.c.) + U sum n_up n_dn on the bonds inside
    `sites` (ascending), modes 2 k + spin for the k-th site."""
    sites = sorted(sites)
    pos = {s: k for k, s in enumerate(sites)}
    bonds = [(i, j) for (i, j) in ed._bonds(lat) if i in pos and j in pos]
    dim = 4 ** len(sites)
    rows, cols, vals = [], [], []
    for c in range(dim):
        if n_elec is not None and bin(c).count("1") != n_elec:
            continue
        for (i, j) in bonds:
            amp = -lat.t * lat.phase(i, j)
            for s in (0, 1):
                for a, b, am in ((i, j, amp), (j, i, np.conj(amp))):
                    ma, mb = 2 * pos[a] + s, 2 * pos[b] + s
                    if not (c >> mb) & 1 or (c >> ma) & 1:
                        continue
                    n1 = bin(c & ((1 << mb) - 1)).count("1")
                    c1 = c ^ (1 << mb)
                    n2 = bin(c1 & ((1 << ma) - 1)).count("1")
                    rows.append(c1 | (1 << ma)); cols.append(c); vals.append(am * (-1) ** (n1 + n2))
        u = sum((c >> (2 * k)) & (c >> (2 * k + 1)) & 1 for k in range(len(sites)))
        if u:
            rows.append(c); cols.append(c); vals.append(lat.U * u)
    return sp.csr_matrix((vals, (rows, cols)), shape=(dim, dim), dtype=complex)


def _fock_hamiltonian_tj(lat, sites, n_elec):
    """-t sum P (phase c+_i c_j + h.c.) P + J sum (S_i . S_j - n_i n_j / 4)
    on the bonds inside `sites` (no double occupancy), same mode order as
    _fock_hamiltonian; a spin flip S+_i = c+_i,up c_i,dn moves one electron
    between two adjacent modes and carries no sign."""
    sites = sorted(sites)
    pos = {s: k for k, s in enumerate(sites)}
    bonds = [(i, j) for (i, j) in ed._bonds(lat) if i in pos and j in pos]
    n = len(sites)
    rows, cols, vals = [], [], []

    def occ(c, k):
        return (c >> (2 * k)) & 1, (c >> (2 * k + 1)) & 1

    for c in range(4 ** n):
        if bin(c).count("1") != n_elec or any(occ(c, k) == (1, 1) for k in range(n)):
            continue
        for (i, j) in bonds:
            a, b = pos[i], pos[j]
            amp = -lat.t * lat.phase(i, j)
            for s in (0, 1):
                for p_, q_, am in ((a, b, amp), (b, a, np.conj(amp))):
                    ma, mb = 2 * p_ + s, 2 * q_ + s
                    if not (c >> mb) & 1 or (c >> ma) & 1 or (c >> (2 * p_ + 1 - s)) & 1:
                        continue
                    n1 = bin(c & ((1 << mb) - 1)).count("1")
                    c1 = c ^ (1 << mb)
                    n2 = bin(c1 & ((1 << ma) - 1)).count("1")
                    rows.append(c1 | (1 << ma)); cols.append(c); vals.append(am * (-1) ** (n1 + n2))
            (ua, da), (ub, db) = occ(c, a), occ(c, b)
            diag = lat.J * (0.25 * (ua - da) * (ub - db) - 0.25 * (ua + da) * (ub + db))
            if diag:
                rows.append(c); cols.append(c); vals.append(diag)
            if (ua, da, ub, db) in ((0, 1, 1, 0), (1, 0, 0, 1)):
                c2 = c ^ (3 << (2 * a)) ^ (3 << (2 * b))
                rows.append(c2); cols.append(c); vals.append(0.5 * lat.J)
    return sp.csr_matrix((vals, (rows, cols)), shape=(4 ** n, 4 ** n), dtype=complex)


def _expand_wave(w, S, E, N):
    v = np.zeros(4 ** N, dtype=complex)
    for ws in w.subs:
        A, B = S[(ws.sys_num_up, ws.sys_num_down)], E[(ws.env_num_up, ws.env_num_down)]
        j = ws.sys_num_down
        for k in range(j + 1):
            m = j - 2 * k
            v += cg(j, m, j, -m, 0, 0) * np.einsum("sb,eb->es", A[k] @ ws.vec, B[j - k]).ravel()
    return v


def _reduce_wave(v, template, S, E, N, nsys):
    """The adjoint of _expand_wave: the reduced coefficients of the Fock
    vector v on the expanded superblock basis."""
    out = template.zeros_like()
    Vm = v.reshape(4 ** (N - nsys), 4 ** nsys).T      # [sys configuration, env configuration]
    for ws in out.subs:
        A, B = S[(ws.sys_num_up, ws.sys_num_down)], E[(ws.env_num_up, ws.env_num_down)]
        j = ws.sys_num_down
        for k in range(j + 1):
            m = j - 2 * k
            ws.vec += cg(j, m, j, -m, 0, 0) * (A[k].conj().T @ Vm @ B[j - k].conj())
    return out


@pytest.fixture(scope="module")
def run():
    lat, d = H.record_superblocks(2, 4, 6, 256, U=8.0, phi=0.25)
    d.left_to_right(1, lat.N // 2 - 1)
    return lat, d


def test_block_hamiltonians_expand_to_dense(run):
    """The reduced block Hamiltonians (sqrt(2S+1) times the regular element;
    conjugated on the environment side) of both halves equal the dense
    Hamiltonian of their sites in the expanded basis; the expansion is an
    isometry."""
    lat, d = run
    sysm, envm, sys_bs, env_bs = d.record[-1][:4]
    N = lat.N
    nbs, nbe = sys_bs.len - 1, env_bs.len - 1
    Sb = _expand(d.sys_bases, d.sys_truns, nbs, True, True)
    Eb = _expand(d.env_bases, d.env_truns, nbe, False, True)
    Hs = _fock_hamiltonian(lat, range(1, nbs + 1))
    He = _fock_hamiltonian(lat, range(N - nbe + 1, N + 1))
    for blk, ham, Hd, conj in ((Sb, sysm.ham, Hs, False), (Eb, envm.ham, He, True)):
        for s in ham.subs:
            F = blk[(s.num_up, s.num_down)][0]
            if conj:
                F = F.conj()
            np.testing.assert_allclose(F.conj().T @ F, np.eye(F.shape[1]), atol=1e-12)
            red = np.sqrt(1.0 + s.num_down) * (F.conj().T @ (Hd @ F))
            np.testing.assert_allclose(red.conj() if conj else red, s.mat, atol=1e-12)


@pytest.mark.parametrize("which", [-1, -2])
def test_model_wave_equals_dense_hamiltonian(run, which):
    """On the last two superblocks of a left-to-right pass (whose blocks the
    stored bases and truncations still describe), the oracle's H psi
    (hmerge + model_wave) is the dense Fock-space H projected on the expanded
    superblock basis, V^H H V psi, for a random psi; on the first (no block
    truncated) H V psi stays in that basis and equals V H psi."""
    lat, d = run
    rec = d.record[which]
    sys_bs, env_bs, sup = rec[2], rec[3], rec[5]
    N = lat.N
    S = _expand(d.sys_bases, d.sys_truns, sys_bs.len, True, False, sys_bs)
    E = {k: np.conj(v) for k, v in _expand(d.env_bases, d.env_truns, env_bs.len, False, False, env_bs).items()}
    psi = H.random_wave(sup, 5)
    phi = H.oracle_hpsi(rec, d.st, psi)
    HF = _fock_hamiltonian(lat, range(1, N + 1), n_elec=sum(w.sys_num_up + w.env_num_up for w in psi.subs[:1]))
    pf, hf = _expand_wave(psi, S, E, N), _expand_wave(phi, S, E, N)
    assert np.linalg.norm(pf) == pytest.approx(np.sqrt(sum(np.vdot(w.vec, w.vec).real for w in psi.subs)), rel=1e-12)
    red = _reduce_wave(HF @ pf, psi, S, E, N, sys_bs.len).flat()
    np.testing.assert_allclose(red, phi.flat(), atol=1e-12 * np.abs(phi.flat()).max())
    if which == -1:
        assert np.linalg.norm(HF @ pf - hf) < 1e-12 * np.linalg.norm(hf)


def test_model_wave_tj_equals_dense_hamiltonian():
    """The t-J branch of model_wave (projected hopping, S.S and n n bond
    terms on blocks and sites): on an untruncated superblock of a t-J ladder
    the oracle's H psi equals the dense projected t-J Hamiltonian applied to
    the expanded psi."""
    lat, d = H.record_superblocks(2, 4, 6, 300, U=0.0, phi=1.0 / 6.0, model="tj", J=0.4)
    d.left_to_right(1, lat.N // 2 - 1)
    rec = d.record[-1]
    sys_bs, env_bs, sup = rec[2], rec[3], rec[5]
    N = lat.N
    S = _expand(d.sys_bases, d.sys_truns, sys_bs.len, True, False, sys_bs)
    E = {k: np.conj(v) for k, v in _expand(d.env_bases, d.env_truns, env_bs.len, False, False, env_bs).items()}
    psi = H.random_wave(sup, 6)
    phi = H.oracle_hpsi(rec, d.st, psi)
    HF = _fock_hamiltonian_tj(lat, range(1, N + 1), 6)
    pf, hf = _expand_wave(psi, S, E, N), _expand_wave(phi, S, E, N)
    assert np.linalg.norm(pf) == pytest.approx(np.sqrt(sum(np.vdot(w.vec, w.vec).real for w in psi.subs)), rel=1e-12)
    assert np.linalg.norm(HF @ pf - hf) < 1e-12 * np.linalg.norm(hf)


def test_wave_transforms_preserve_the_state(run):
    """wave_trans_LR and wave_trans_RL (code/warm_up.f90:1855-2170) carry the
    converged psi of one superblock to the guess on the next as the same
    Fock-space state: left to right (nothing truncated in between) the
    expansions are equal; right to left (the environment block grows and is
    truncated) the guess is the old state's coefficients on the new basis,
    V_new^H V_old psi."""
    from oracle.blocks import allocate_wave
    from oracle.dmrg import wave_trans_lr, wave_trans_rl

    def exp(d, rec):
        S = _expand(d.sys_bases, d.sys_truns, rec[2].len, True, False, rec[2])
        E = {k: np.conj(v) for k, v in _expand(d.env_bases, d.env_truns, rec[3].len, False, False, rec[3]).items()}
        return S, E

    lat, d = run
    N = lat.N
    old, new = d.record[-2], d.record[-1]
    guess = allocate_wave(new[5])
    wave_trans_lr(new[2], d.env_bases[old[3].len], d.sys_truns[old[2].len], d.env_truns[new[3].len], old[6], guess)
    vo, vn = _expand_wave(old[6], *exp(d, old), N), _expand_wave(guess, *exp(d, new), N)
    assert np.linalg.norm(vn - vo) < 1e-12

    lat, d = H.record_superblocks(2, 4, 6, 256, U=8.0, phi=0.25)
    old, new = d.record[-2], d.record[-1]
    label = new[2].len
    guess = allocate_wave(new[5])
    wave_trans_rl(d.sys_bases[label + 1], new[3], d.sys_truns[label], d.env_truns[N - label - 1], old[6], guess)
    Sn, En = exp(d, new)
    red = _reduce_wave(_expand_wave(old[6], *exp(d, old), N), guess, Sn, En, N, label).flat()
    g = guess.flat()
    assert np.linalg.norm(red / np.linalg.norm(red) - g / np.linalg.norm(g)) < 1e-12


def test_density_matrix_spectra_are_schmidt_spectra(run):
    """Get_density_matrix_sys / _env (code/get_den.f90:4-177): every
    eigenvalue x of a sector (2S) density matrix, spread as x / (2S+1) over
    the multiplet's 2S+1 states, gives the spectrum of the Fock-space reduced
    density matrix of that half of the expanded ground state (the Schmidt
    spectrum, the same on both halves)."""
    from oracle.density import get_density_matrix_env, get_density_matrix_sys
    lat, d = run
    N = lat.N
    rec = d.record[-1]
    psi = rec[6]
    S = _expand(d.sys_bases, d.sys_truns, rec[2].len, True, False, rec[2])
    E = {k: np.conj(v) for k, v in _expand(d.env_bases, d.env_truns, rec[3].len, False, False, rec[3]).items()}
    M = _expand_wave(psi, S, E, N).reshape(4 ** (N - rec[2].len), 4 ** rec[2].len).T
    schmidt = np.sort(np.linalg.svd(M, compute_uv=False) ** 2)[::-1]
    for den in (get_density_matrix_sys(psi), get_density_matrix_env(psi)):
        spread = np.sort(np.concatenate([np.repeat(np.linalg.eigvalsh(s.mat) / (s.num_down + 1), s.num_down + 1)
                                         for s in den.subs]))[::-1]
        spread = spread / spread.sum()
        k = min(len(spread), len(schmidt))
        np.testing.assert_allclose(spread[:k], schmidt[:k], atol=1e-13)
        assert abs(spread[k:]).sum() < 1e-13 and schmidt[k:].sum() < 1e-13
