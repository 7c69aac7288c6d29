"""Site profiles and cross-cut correlations of diagonal (rank-0) site operators
(test infrastructure, restating code/measure.f90).

measure_operator_dia (code/measure.f90:3-62): <O_i> for every site.  The
operator of block site i is carried to the block of the superblock the way
Get_sys_oper_dia / Get_env_oper_dia (code/get_ham.f90:1244-1380) do: embedded
in the enlarged basis of length i (update_site_dia) and truncated, then for each
longer block embedded as a block operator (update_block_dia) and truncated;
<O_i> = <psi|(O_i x 1)|psi> is measure_sys_block / measure_env_block
(code/measure.f90:611-862), and the two middle sites are site terms.

Cross-cut correlations <O_a O_b> with a on the system side and b on the
environment side (the cross part of Get_density_cor, code/correlation.f90:43):
with phi_a = (O_a x 1) psi and chi_b = (1 x O_b) psi, <psi|O_a O_b|psi> =
Re <phi_a|chi_b>, since the two operators act on different halves and are
Hermitian.  Sites are numbered like the reference's output: system block site
i is site i, environment block site j is site N - j + 1.

Same-side density correlations <n_a n_b> (a < b on one half, the rest of
Get_density_cor): n_a is carried to the block of length b - 1 and embedded in
the enlarged basis of length b (update_block_dia), n_b embedded as the new
site (update_site_dia), and their product formed in that basis the way
Get_hamiltonian_dia forms the n.n bond (code/get_ham.f90:852-941:
coef/sqrt(2S+1) O1 O2 per sector); the product is truncated and carried to
the current block like a site operator and measured with block_vec_dia /
vec_block_dia.  A block site with the middle site of its half is the
block_site_vec_dia / vec_block_site_dia term; <n_i n_i> = <n_i> + 2 <d_i>.

Cross-cut spin correlations <S_a . S_b> (the spin part of Get_spin_cor,
code/correlation.f90): the rank-1 operator sd of site a is carried to its
block with update_site_ndia / update_block_ndia / update_trun_ndia, and the
pair is applied by the kernel of the Hamiltonian's own S.S bond term of that
geometry (block_vec_block_ndia, block_vec_site_ndia, site_vec_block_ndia,
site_vec_site_ndia with the environment block through block_transfer_trans,
code/mat_vec.f90:3509-3600), which carries J S.S as jd = -sqrt(3) J times
the unit-coefficient term: <S_a . S_b> = -sqrt(3) <psi|T_ab psi>.
"""
import numpy as np

from .blocks import (Block, Sub, update_site_dia, update_block_dia, update_trun_dia, wave_product,
                     update_site_ndia, update_block_ndia, update_trun_ndia, block_transfer_trans,
                     block_mul_block_ndia, SU)
from .su2 import w6j
from .enlarge import get_hamiltonian_dia, get_hamiltonian_ndia
from .matvec import (block_vec_dia, vec_block_dia, site_vec_site_dia, block_vec_block_ndia, block_vec_site_ndia,
                     site_vec_block_ndia, site_vec_site_ndia, block_site_vec_dia, vec_block_site_dia,
                     block_site_vec_ndia, vec_block_site_ndia)


def _carry(op, i, length, bases, truns):
    """Operator of block site i in the truncated block of `length` sites."""
    cur = op.copy() if i <= 1 else update_trun_dia(update_site_dia(op, bases[i]), truns[i])
    for L in range(i + 1, length + 1):
        cur = update_trun_dia(update_block_dia(cur, bases[L]), truns[L])
    return cur


def site_vectors(d, name):
    """{site: (side, phi)} with phi = O_site psi on the current superblock of an
    oracle DMRG ``d`` (side 0 system half, 1 environment half)."""
    wave = d.wave
    N = d.lat.N
    st = d.st
    op, one = getattr(st, name), st.si
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    out = {}
    for i in range(1, Ls + 1):
        o = _carry(op, i, Ls, d.sys_bases, d.sys_truns)
        phi = wave.zeros_like()
        block_vec_dia(o, sys_bs, wave, phi, 1.0)
        out[i] = (0, phi)
    phi = wave.zeros_like()
    site_vec_site_dia(op, one, sys_bs, env_bs, wave, phi, 1.0)
    out[Ls + 1] = (0, phi)
    phi = wave.zeros_like()
    site_vec_site_dia(one, op, sys_bs, env_bs, wave, phi, 1.0)
    out[N - Le] = (1, phi)
    for j in range(1, Le + 1):
        o = _carry(op, j, Le, d.env_bases, d.env_truns)
        phi = wave.zeros_like()
        vec_block_dia(o, env_bs, wave, phi, 1.0)
        out[N - j + 1] = (1, phi)
    return out


def site_profile(d, name="num_elec"):
    """measure_operator_dia: <O_i>, i = 1..N."""
    vec = site_vectors(d, name)
    prof = np.zeros(d.lat.N)
    for s, (_, phi) in vec.items():
        prof[s - 1] = wave_product(d.wave, phi)
    return prof


def cross_correlations(d, name_a="num_elec", name_b="num_elec"):
    """<O_a O_b> for a on the system half and b on the environment half:
    (sites_a, sites_b, matrix)."""
    va, vb = site_vectors(d, name_a), site_vectors(d, name_b)
    sa = sorted(s for s, (side, _) in va.items() if side == 0)
    sb = sorted(s for s, (side, _) in vb.items() if side == 1)
    m = np.array([[wave_product(va[a][1], vb[b][1]) for b in sb] for a in sa])
    return sa, sb, m


def _carry_ndia(op, i, length, bases, truns, side):
    """Rank-1 (boson) operator of block site i in the truncated block of
    `length` sites (the ndia counterpart of _carry)."""
    cur = op.copy() if i <= 1 else update_trun_ndia(update_site_ndia(op, bases[i], "B", side), truns[i])
    for L in range(i + 1, length + 1):
        cur = update_trun_ndia(update_block_ndia(cur, bases[L], "B", side), truns[L])
    return cur


SPIN_NORM = -np.sqrt(3.0)  # <S_a . S_b> per unit-coefficient sd x sd term


def spin_correlations(d):
    """<S_a . S_b> for a on the system half and b on the environment half of
    the current superblock of an oracle DMRG ``d``: (sites_a, sites_b, matrix)."""
    wave = d.wave
    N = d.lat.N
    sd = d.st.sd
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    # (site, block operator or None for the middle site)
    a_ops = [(i, _carry_ndia(sd, i, Ls, d.sys_bases, d.sys_truns, "sys")) for i in range(1, Ls + 1)]
    a_ops.append((Ls + 1, None))
    b_ops = [(N - Le, None)]
    b_ops += [(N - j + 1, block_transfer_trans(_carry_ndia(sd, j, Le, d.env_bases, d.env_truns, "env")))
              for j in range(1, Le + 1)]
    sa = [a for a, _ in a_ops]
    sb = sorted(b for b, _ in b_ops)
    m = np.zeros((len(sa), len(sb)))
    for ia, (a, oa) in enumerate(a_ops):
        for b, ob in b_ops:
            phi = wave.zeros_like()
            if oa is not None and ob is not None:
                block_vec_block_ndia(oa, "B", ob, "B", sys_bs, env_bs, wave, phi, 1.0)
            elif oa is not None:
                block_vec_site_ndia(oa, "B", sd, "B", sys_bs, env_bs, wave, phi, 1.0)
            elif ob is not None:
                site_vec_block_ndia(sd, "B", ob, "B", sys_bs, env_bs, wave, phi, 1.0)
            else:
                site_vec_site_ndia(sd, "B", sd, "B", sys_bs, env_bs, wave, phi, 1.0)
            m[ia, sb.index(b)] = SPIN_NORM * wave_product(wave, phi)
    return sa, sb, m


def _pair_operator(op, a, b, length, bases, truns):
    """n_a n_b (block sites a < b <= length) in the truncated block of
    `length` sites."""
    basis = bases[b]
    A = update_block_dia(_carry(op, a, b - 1, bases, truns), basis)
    B = update_site_dia(op, basis)
    P = Block(b, 0, 0, [Sub(sec.new_num_up, sec.new_num_down, 0, sec.dim, sec.dim) for sec in basis.sectors])
    get_hamiltonian_dia(A, B, 1.0, P)
    cur = update_trun_dia(P, truns[b])
    for L in range(b + 1, length + 1):
        cur = update_trun_dia(update_block_dia(cur, bases[L]), truns[L])
    return cur


def density_correlations(d, name="num_elec"):
    """<n_i n_j> for all sites i, j (N x N, sites numbered as in the
    reference's output) on the current superblock of an oracle DMRG ``d``:
    cross-cut pairs from cross_correlations, same-side pairs from carried
    products, the diagonal from the site profiles of n and of the double
    occupancy (Hubbard)."""
    wave = d.wave
    N = d.lat.N
    op = getattr(d.st, name)
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    m = np.zeros((N, N))
    sa, sb, cross = cross_correlations(d, name, name)
    for ia, a in enumerate(sa):
        for ib, b in enumerate(sb):
            m[a - 1, b - 1] = m[b - 1, a - 1] = cross[ia, ib]

    def measure(fn, *args):
        phi = wave.zeros_like()
        fn(*args, wave, phi, 1.0)
        return wave_product(wave, phi)

    # system half: block sites 1..Ls and the middle site Ls + 1
    for b in range(2, Ls + 1):
        for a in range(1, b):
            v = measure(block_vec_dia, _pair_operator(op, a, b, Ls, d.sys_bases, d.sys_truns), sys_bs)
            m[a - 1, b - 1] = m[b - 1, a - 1] = v
    for a in range(1, Ls + 1):
        v = measure(block_site_vec_dia, _carry(op, a, Ls, d.sys_bases, d.sys_truns), op, sys_bs)
        m[a - 1, Ls] = m[Ls, a - 1] = v
    # environment half: block sites j = 1..Le (site N - j + 1) and the middle site N - Le
    for jb in range(2, Le + 1):
        for ja in range(1, jb):
            v = measure(vec_block_dia, _pair_operator(op, ja, jb, Le, d.env_bases, d.env_truns), env_bs)
            i, j = N - ja, N - jb
            m[i, j] = m[j, i] = v
    for ja in range(1, Le + 1):
        v = measure(vec_block_site_dia, _carry(op, ja, Le, d.env_bases, d.env_truns), op, env_bs)
        i, j = N - ja, N - Le - 1
        m[i, j] = m[j, i] = v
    n = site_profile(d, name)
    dbl = site_profile(d, "double") if hasattr(d.st, "double") else np.zeros(N)
    for i in range(N):
        m[i, i] = n[i] + 2.0 * dbl[i]
    return m


def _spin_pair_operator(sd, a, b, length, bases, truns, side):
    """S_a . S_b (block sites a < b <= length) in the truncated block of
    `length` sites: S_a carried (rank 1) to the block of length b - 1, the
    scalar product with the new site's sd added in the enlarged basis of
    length b as the S.S bond of Get_hamiltonian_ndia (with -sqrt(3), the
    inverse of jd / J), then truncated and carried."""
    basis = bases[b]
    Sa = _carry_ndia(sd, a, b - 1, bases, truns, side)
    P = Block(b, 0, 0, [Sub(sec.new_num_up, sec.new_num_down, 0, sec.dim, sec.dim) for sec in basis.sectors])
    get_hamiltonian_ndia(Sa, sd, basis, SPIN_NORM, P, "B", "S" if side == "sys" else "E")
    cur = update_trun_dia(P, truns[b])
    for L in range(b + 1, length + 1):
        cur = update_trun_dia(update_block_dia(cur, bases[L]), truns[L])
    return cur


def spin_correlations_all(d):
    """<S_i . S_j> for all sites i, j (N x N): cross-cut pairs from
    spin_correlations, same-side pairs from carried bond products, a block
    site with its half's middle site as the block-site S.S term, and
    <S_i . S_i> = 3/4 (<n_i> - 2 <d_i>) (Hubbard)."""
    wave = d.wave
    N = d.lat.N
    sd = d.st.sd
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    m = np.zeros((N, N))
    sa, sb, cross = spin_correlations(d)
    for ia, a in enumerate(sa):
        for ib, b in enumerate(sb):
            m[a - 1, b - 1] = m[b - 1, a - 1] = cross[ia, ib]

    def measure(fn, *args, coef=1.0):
        phi = wave.zeros_like()
        fn(*args, wave, phi, coef)
        return wave_product(wave, phi)

    for b in range(2, Ls + 1):
        for a in range(1, b):
            v = measure(block_vec_dia, _spin_pair_operator(sd, a, b, Ls, d.sys_bases, d.sys_truns, "sys"), sys_bs)
            m[a - 1, b - 1] = m[b - 1, a - 1] = v
    for a in range(1, Ls + 1):
        v = SPIN_NORM * measure(block_site_vec_ndia, _carry_ndia(sd, a, Ls, d.sys_bases, d.sys_truns, "sys"), "B",
                                sd, "B", sys_bs)
        m[a - 1, Ls] = m[Ls, a - 1] = v
    for jb in range(2, Le + 1):
        for ja in range(1, jb):
            v = measure(vec_block_dia, _spin_pair_operator(sd, ja, jb, Le, d.env_bases, d.env_truns, "env"), env_bs)
            i, j = N - ja, N - jb
            m[i, j] = m[j, i] = v
    for ja in range(1, Le + 1):
        v = SPIN_NORM * measure(vec_block_site_ndia, _carry_ndia(sd, ja, Le, d.env_bases, d.env_truns, "env"), "B",
                                sd, "B", env_bs)
        i, j = N - ja, N - Le - 1
        m[i, j] = m[j, i] = v
    n = site_profile(d, "num_elec")
    dbl = site_profile(d, "double")
    for i in range(N):
        m[i, i] = 0.75 * (n[i] - 2.0 * dbl[i])
    return m


def _carry_fermion(op, i, length, bases, truns, side):
    """Rank-1/2 (fermion) operator of block site i in the truncated block of
    `length` sites."""
    cur = op.copy() if i <= 1 else update_trun_ndia(update_site_ndia(op, bases[i], "F", side), truns[i])
    for L in range(i + 1, length + 1):
        cur = update_trun_ndia(update_block_ndia(cur, bases[L], "F", side), truns[L])
    return cur


def electron_correlations(d):
    """G_ab = sum_s <c+_as c_bs> for a on the system half and b on the
    environment half (the electron part of Get_density_cor, flag 'F'):
    (sites_a, sites_b, complex matrix).  Each pair is the hopping kernel of
    that geometry (the environment operator through block_transfer_trans),
    which holds X + X^+ with X = sum_s c+_as c_bs / sqrt(2); with the
    coefficients 1 and i it gives Re G = <T_1> / sqrt(2), Im G = -<T_i> /
    sqrt(2)."""
    wave = d.wave
    N = d.lat.N
    up, dn = d.st.elec_up, d.st.elec_down
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    a_ops = [(i, _carry_fermion(up, i, Ls, d.sys_bases, d.sys_truns, "sys")) for i in range(1, Ls + 1)]
    a_ops.append((Ls + 1, None))
    b_ops = [(N - Le, None)]
    b_ops += [(N - j + 1, block_transfer_trans(_carry_fermion(dn, j, Le, d.env_bases, d.env_truns, "env")))
              for j in range(1, Le + 1)]
    dn_t = block_transfer_trans(dn)
    sa = [a for a, _ in a_ops]
    sb = sorted(b for b, _ in b_ops)
    m = np.zeros((len(sa), len(sb)), dtype=np.complex128)
    for ia, (a, oa) in enumerate(a_ops):
        for b, ob in b_ops:
            t = []
            for coef in (1.0, 1j):
                phi = wave.zeros_like()
                if oa is not None and ob is not None:
                    block_vec_block_ndia(oa, "F", ob, "F", sys_bs, env_bs, wave, phi, coef)
                elif oa is not None:
                    block_vec_site_ndia(oa, "F", dn_t, "F", sys_bs, env_bs, wave, phi, coef)
                elif ob is not None:
                    site_vec_block_ndia(up, "F", ob, "F", sys_bs, env_bs, wave, phi, coef)
                else:
                    site_vec_site_ndia(up, "F", dn_t, "F", sys_bs, env_bs, wave, phi, coef)
                t.append(wave_product(wave, phi))
            m[ia, sb.index(b)] = (t[0] - 1j * t[1]) / np.sqrt(2.0)
    return sa, sb, m


def _hop_pair_operators(op, site, a, b, length, bases, truns, side):
    """The hopping bond of Get_hamiltonian_ndia between block site a (op:
    elec_up on the system side, elec_down on the environment side, carried
    to the block of length b - 1) and the new site b (site operator through
    block_transfer_trans), formed with coefficients 1 and i in the enlarged
    basis of length b and carried as scalars to the block of `length`
    sites."""
    basis = bases[b]
    out = []
    for coef in (1.0, 1j):
        Ca = _carry_fermion(op, a, b - 1, bases, truns, side)
        P = Block(b, 0, 0, [Sub(sec.new_num_up, sec.new_num_down, 0, sec.dim, sec.dim) for sec in basis.sectors])
        get_hamiltonian_ndia(Ca, block_transfer_trans(site), basis, coef, P, "F", "S" if side == "sys" else "E")
        cur = update_trun_dia(P, truns[b])
        for L in range(b + 1, length + 1):
            cur = update_trun_dia(update_block_dia(cur, bases[L]), truns[L])
        out.append(cur)
    return out


def electron_correlations_all(d):
    """G_ij = sum_s <c+_is c_js> for all sites i, j (N x N, complex,
    Hermitian): cross-cut pairs from electron_correlations; same-side pairs
    from the hopping bond formed in the enlarged basis (system side: block
    elec_up with the new site's elec_down, giving G_ab, a < b; environment
    side: block elec_down with the new site's elec_up, giving G for the
    outer site first); a block site with its half's middle site from the
    block-site hopping kernels; the diagonal <n_i>.  Every term holds
    X + X^+ with X = G / sqrt(2): G = (<T_1> - i <T_i>) / sqrt(2)."""
    wave = d.wave
    N = d.lat.N
    up, dn = d.st.elec_up, d.st.elec_down
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    G = np.zeros((N, N), dtype=np.complex128)

    def put(i, j, v):
        G[i, j] = v
        G[j, i] = np.conj(v)

    sa, sb, cross = electron_correlations(d)
    for ia, a in enumerate(sa):
        for ib, b in enumerate(sb):
            put(a - 1, b - 1, cross[ia, ib])

    def scalar(ops, fn, bs):
        t = []
        for cur in ops:
            phi = wave.zeros_like()
            fn(cur, bs, wave, phi, 1.0)
            t.append(wave_product(wave, phi))
        return (t[0] - 1j * t[1]) / np.sqrt(2.0)

    def term(fn, *args):
        t = []
        for coef in (1.0, 1j):
            phi = wave.zeros_like()
            fn(*args, wave, phi, coef)
            t.append(wave_product(wave, phi))
        return (t[0] - 1j * t[1]) / np.sqrt(2.0)

    dn_t = block_transfer_trans(dn)
    for b in range(2, Ls + 1):
        for a in range(1, b):
            ops = _hop_pair_operators(up, dn, a, b, Ls, d.sys_bases, d.sys_truns, "sys")
            put(a - 1, b - 1, scalar(ops, block_vec_dia, sys_bs))
    for a in range(1, Ls + 1):
        oa = _carry_fermion(up, a, Ls, d.sys_bases, d.sys_truns, "sys")
        put(a - 1, Ls, term(block_site_vec_ndia, oa, "F", dn_t, "F", sys_bs))
    for jb in range(2, Le + 1):
        for ja in range(1, jb):
            ops = _hop_pair_operators(dn, up, ja, jb, Le, d.env_bases, d.env_truns, "env")
            put(N - ja, N - jb, scalar(ops, vec_block_dia, env_bs))
    for ja in range(1, Le + 1):
        oa = _carry_fermion(up, ja, Le, d.env_bases, d.env_truns, "env")
        put(N - ja, N - Le - 1, term(vec_block_site_ndia, oa, "F", dn_t, "F", env_bs))
    n = site_profile(d, "num_elec")
    for i in range(N):
        G[i, i] = n[i]
    return G


def _fermion_in_basis(op, a, b, bases, truns, side):
    """Get_sys_oper_ndia / Get_env_oper_ndia with Truns = .false.
    (code/get_ham.f90:1631-1695): the operator of site a in the enlarged,
    untruncated basis of length b >= a."""
    if a == b:
        return op.copy() if b <= 1 else update_site_ndia(op, bases[b], "F", side)
    cur = _carry_fermion(op, a, b - 1, bases, truns, side)
    return update_block_ndia(cur, bases[b], "F", side)


def pair_creator(d, a, b, side):
    """Singlet pair creator [c+_a c+_b]^0 of block sites a < b (Get_SCOP_Operator_Sys /
    Get_SCOP_Operator_Env with 'S0', code/correlation.f90:2659-2772):
    elec_up of both sites in the enlarged basis of length b, their product
    coupled to rank 0 (block_mul_block_ndia), truncated, then carried as a
    boson operator to the block of the current superblock (Change_sys_oper_ndia,
    code/get_ham.f90:1767-1818)."""
    if side == "sys":
        bases, truns, length = d.sys_bases, d.sys_truns, d.wave.sys_len - 1
    else:
        bases, truns, length = d.env_bases, d.env_truns, d.wave.env_len - 1
    up = d.st.elec_up
    P = block_mul_block_ndia(_fermion_in_basis(up, a, b, bases, truns, side),
                             _fermion_in_basis(up, b, b, bases, truns, side), 0, bases[b])
    cur = update_trun_ndia(P, truns[b])
    for L in range(b + 1, length + 1):
        cur = update_trun_ndia(update_block_ndia(cur, bases[L], "B", side), truns[L])
    return cur


def sys_block_env_block_cor_ndia(sys_bl, env_bl, sys_bs, env_bs, wave):
    """<(A x 1) psi | (1 x B) psi> for a system block operator A and an
    environment block operator B of the same rank k and the same up_dif,
    boson sign (sys_block_env_block_cor_ndia with 'B',
    code/correlation.f90:1666-1929): each operator re-coupled into its
    enlarged basis with the 6j of its block and site, times
    sqrt((2S'+1)(2S+1)/(k+1)) and the phase of the two recouplings."""
    up_dif, k = sys_bl.up_dif, sys_bl.down_dif
    value = 0.0 + 0.0j
    for w in wave.subs:
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        for m in ss.subs:
            for n in es.subs:
                for dd in range(-k, k + 1, SU):
                    sid = sys_bl.find(m.bl_num_up, m.bl_num_down, dd)
                    nsbu, nsbd = m.bl_num_up + up_dif, m.bl_num_down + dd
                    for edd in range(-k, k + 1, SU):
                        nebu, nebd = n.bl_num_up - up_dif, n.bl_num_down - edd
                        eid = env_bl.find(nebu, nebd, edd)
                        if sid is None or eid is None:
                            continue
                        for nsd in range(abs(w.sys_num_down - k), w.sys_num_down + k + 1, SU):
                            nsu, neu, ned = w.sys_num_up + up_dif, w.env_num_up - up_dif, nsd
                            ts, te = sys_bs.find(nsu, nsd), env_bs.find(neu, ned)
                            ms = ts.find_full(nsbu, nsbd, m.st_num_up, m.st_num_down) if ts else None
                            me = te.find_full(nebu, nebd, n.st_num_up, n.st_num_down) if te else None
                            kk = wave.find(nsu, nsd, neu, ned)
                            if ms is None or me is None or kk is None:
                                continue
                            c1 = w6j(nsd, k, w.sys_num_down, m.bl_num_down, m.st_num_down, nsbd)
                            if c1 == 0.0:
                                continue
                            c1 *= w6j(ned, k, w.env_num_down, n.bl_num_down, n.st_num_down, nebd)
                            if c1 == 0.0:
                                continue
                            c1 *= np.sqrt((1.0 + ned) * (1.0 + w.env_num_down) / (1.0 + k))
                            if ((nsbd + m.st_num_down + w.sys_num_down + k) // 2
                                    + (nebd + n.st_num_down + w.env_num_down + k) // 2) % 2 == 1:
                                c1 = -c1
                            x = w.vec[m.spos:m.spos + m.sdim, n.spos:n.spos + n.sdim]
                            y = wave.subs[kk].vec[ms.spos:ms.spos + ms.sdim, me.spos:me.spos + me.sdim]
                            m1 = sys_bl.subs[sid].mat @ x
                            m2 = c1 * (y @ env_bl.subs[eid].mat.conj().T)
                            value += np.vdot(m1, m2)
    return value


def pairing_correlations(d, sys_bonds, env_bonds):
    """Cross-cut singlet-pair correlations of Get_mSCOP_Operator_cor0
    (code/correlation.f90:198-327): for a bond (a, a') inside the system
    block and a bond (b, b') inside the environment block (sites in the
    output numbering), the conjugate of sys_block_env_block_cor_ndia of the
    two pair creators, <D+_(a,a') D_(b,b')> in the reference's reduced
    normalisation.  Returns the (len(sys_bonds), len(env_bonds)) complex
    matrix."""
    wave = d.wave
    N = d.lat.N
    Ls, Le = wave.sys_len - 1, wave.env_len - 1
    for a, b in sys_bonds:
        if not (1 <= min(a, b) < max(a, b) <= Ls):
            raise ValueError(f"bond ({a}, {b}) is not inside the system block")
    for a, b in env_bonds:
        if not (N - Le + 1 <= min(a, b) < max(a, b) <= N):
            raise ValueError(f"bond ({a}, {b}) is not inside the environment block")
    sys_bs, env_bs = d.sys_bases[wave.sys_len], d.env_bases[wave.env_len]
    A = [pair_creator(d, min(a, b), max(a, b), "sys") for a, b in sys_bonds]
    B = []
    for a, b in env_bonds:
        ea, eb = N - a + 1, N - b + 1
        B.append(pair_creator(d, min(ea, eb), max(ea, eb), "env"))
    return np.array([[np.conj(sys_block_env_block_cor_ndia(x, y, sys_bs, env_bs, wave)) for y in B] for x in A])


def _carry_untruncated(op, a, b, bases, truns, side, flag):
    """Change_sys_oper_ndia with Truns = .false. (code/get_ham.f90:1767-1818):
    a block operator of the truncated block of length a embedded in the
    enlarged, untruncated basis of length b > a (truncated at the lengths in
    between)."""
    cur = op
    for L in range(a + 1, b):
        cur = update_trun_ndia(update_block_ndia(cur, bases[L], flag, side), truns[L])
    return update_block_ndia(cur, bases[b], flag, side)


def pair_pair_operator(d, bond_x, bond_y):
    """The scalar D+_x D_y of two bonds inside the system block, bond x before
    bond y (Get_sys_two and Get_sys_two1, code/correlation.f90:331-428): the
    pair creator of x truncated at its later site, embedded up to the first
    site of y, multiplied by that site's elec_down (rank 1/2) and truncated,
    embedded (fermion) up to the second site of y and multiplied by its
    elec_down to rank 0, then truncated and carried as a scalar to the
    block of the superblock (Change_sys_oper_dia)."""
    a1, a2 = sorted(bond_x)
    a3, a4 = sorted(bond_y)
    bases, truns, length = d.sys_bases, d.sys_truns, d.wave.sys_len - 1
    up, dn = d.st.elec_up, d.st.elec_down
    P = block_mul_block_ndia(_fermion_in_basis(up, a1, a2, bases, truns, "sys"),
                             _fermion_in_basis(up, a2, a2, bases, truns, "sys"), 0, bases[a2])
    P = update_trun_ndia(P, truns[a2])
    X = block_mul_block_ndia(_carry_untruncated(P, a2, a3, bases, truns, "sys", "B"),
                             _fermion_in_basis(dn, a3, a3, bases, truns, "sys"), 1, bases[a3])
    X = update_trun_ndia(X, truns[a3])
    X = block_mul_block_ndia(_carry_untruncated(X, a3, a4, bases, truns, "sys", "F"),
                             _fermion_in_basis(dn, a4, a4, bases, truns, "sys"), 0, bases[a4])
    X = update_trun_dia(X, truns[a4])
    for L in range(a4 + 1, length + 1):
        X = update_trun_dia(update_block_dia(X, bases[L]), truns[L])
    return X


def measure_sys_block(op, sys_bs, wave):
    """<psi|(O x 1)|psi>, complex (measure_sys_block, code/measure.f90:611-673)."""
    phi = wave.zeros_like()
    block_vec_dia(op, sys_bs, wave, phi, 1.0)
    return sum(np.vdot(w.vec, p.vec) for w, p in zip(wave.subs, phi.subs))


def pairing_correlations_sys(d, bonds_x, bonds_y):
    """Same-side singlet-pair correlations of Get_mSCOP_Operator_cor0
    (code/correlation.f90:226-262): measure_sys_block of pair_pair_operator
    for bonds x and y inside the system block, every site of x before every
    site of y.  Returns the (len(bonds_x), len(bonds_y)) complex matrix."""
    Ls = d.wave.sys_len - 1
    for x in bonds_x:
        for y in bonds_y:
            if not (1 <= min(x) and max(x) < min(y) and max(y) <= Ls):
                raise ValueError(f"bonds {x}, {y} are not ordered inside the system block")
    sys_bs = d.sys_bases[d.wave.sys_len]
    return np.array([[measure_sys_block(pair_pair_operator(d, x, y), sys_bs, d.wave) for y in bonds_y]
                     for x in bonds_x])


def structure_factor_cut(corr, W, L, nx_cut):
    """Get_structure_factor_cut (code/measure.f90:2159-2236): for the sites
    outside nx_cut columns at either end, S(kx, ky) = (sum_x C_xx +
    sum_{x != y} exp(i (kx (X_x - X_y) + ky (Y_x - Y_y))) C_xy) / N' with
    C the real part of the correlation matrix, kx = 2 pi i / (L - 2 nx_cut),
    i = 0..L - 2 nx_cut, ky = 2 pi j / W, j = 0..W; site s sits at
    X = (s - 1) // W + 1, Y = (s - 1) % W + 1.  Returns the real part,
    indexed [i, j]."""
    C = np.real(np.asarray(corr))
    N = W * L
    kxn, kyn = L - 2 * nx_cut, W
    lo, hi = nx_cut * W + 1, N - nx_cut * W
    out = np.zeros((kxn + 1, kyn + 1))
    for i in range(kxn + 1):
        kx = 2.0 * np.pi * i / kxn
        for j in range(kyn + 1):
            ky = 2.0 * np.pi * j / kyn
            s = 0.0 + 0.0j
            for x in range(lo, hi + 1):
                s += C[x - 1, x - 1]
            for x in range(lo, hi + 1):
                for y in range(lo, hi + 1):
                    if x != y:
                        dx = (x - 1) // W - (y - 1) // W
                        dy = (x - 1) % W - (y - 1) % W
                        s += np.exp(1j * (kx * dx + ky * dy)) * C[x - 1, y - 1]
            out[i, j] = (s / (N - 2 * nx_cut * W)).real
    return out
