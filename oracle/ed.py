"""Exact diagonalisation of small flux ladders in the Fock basis (known-answer tests).

H = sum_<ij>,s (-t pint(i,j) c+_is c_js + h.c.) + U sum_i n_i,up n_i,dn with the
same bonds and Peierls factors as ``oracle.lattice``.  The spectrum is invariant
under phi -> -phi and t -> -t on these bipartite lattices, so the comparison does
not depend on the orientation convention of the reference's coefficients.
"""
from itertools import combinations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _bonds(lat):
    nb = lat._neib(lat.L)
    out = []
    for i, d in nb.items():
        for k, j in d.items():
            if k in (1, 3):
                out.append((i, j))
    return out


def _configs(nsite, nel):
    return [sum(1 << b for b in c) for c in combinations(range(nsite), nel)]


def _spin_hop(lat, confs):
    idx = {c: n for n, c in enumerate(confs)}
    rows, cols, vals = [], [], []
    for (i, j) in _bonds(lat):
        a, b = i - 1, j - 1
        amp = -lat.t * lat.phase(i, j)
        lo, hi = min(a, b), max(a, b)
        mask = ((1 << hi) - 1) & ~((1 << (lo + 1)) - 1)
        for n, c in enumerate(confs):
            # c+_a c_b
            if (c >> b) & 1 and not (c >> a) & 1:
                c2 = c ^ (1 << a) ^ (1 << b)
                s = -1.0 if bin(c & mask).count("1") % 2 else 1.0
                rows.append(idx[c2]); cols.append(n); vals.append(s * amp)
            # h.c.: c+_b c_a
            if (c >> a) & 1 and not (c >> b) & 1:
                c2 = c ^ (1 << a) ^ (1 << b)
                s = -1.0 if bin(c & mask).count("1") % 2 else 1.0
                rows.append(idx[c2]); cols.append(n); vals.append(s * np.conj(amp))
    m = len(confs)
    return sp.csr_matrix((vals, (rows, cols)), shape=(m, m), dtype=np.complex128)


def hubbard_ground_energy(lat, n_up, n_dn, k=1):
    N = lat.N
    cu = _configs(N, n_up)
    cd = _configs(N, n_dn)
    hu = _spin_hop(lat, cu)
    hd = _spin_hop(lat, cd)
    H = sp.kron(hu, sp.identity(len(cd)), format="csr") + sp.kron(sp.identity(len(cu)), hd, format="csr")
    if lat.U != 0.0:
        au = np.array(cu, dtype=np.int64)
        ad = np.array(cd, dtype=np.int64)
        dbl = np.array([[bin(int(x & y)).count("1") for y in ad] for x in au], dtype=np.float64).ravel()
        H = H + sp.diags(lat.U * dbl)
    dim = H.shape[0]
    if dim <= 400:
        w = np.linalg.eigvalsh(H.toarray())
        return w[:k]
    w = spla.eigsh(H, k=k, which="SA", return_eigenvectors=False, tol=1e-12)
    return np.sort(w)


def singlet_ground_energy(lat, n_elec, k=10, tol=1e-7):
    """Lowest S=0 energy and the lowest Sz=1 energy.

    Every S>=1 multiplet has an Sz=1 member, so the lowest Sz=0 level that is
    not matched (with multiplicity) by an Sz=1 level is the singlet ground state.
    """
    e0 = list(hubbard_ground_energy(lat, n_elec // 2, n_elec // 2, k=k))
    e1 = list(hubbard_ground_energy(lat, n_elec // 2 + 1, n_elec // 2 - 1, k=k))
    pool = list(e1)
    for e in e0:
        hit = [i for i, f in enumerate(pool) if abs(f - e) < tol]
        if hit:
            pool.pop(hit[0])
            continue
        return float(e), float(e1[0])
    raise RuntimeError("no singlet among the lowest levels; raise k")


def free_fermion_energy(lat, n_elec):
    """U=0 singlet energy: both spins fill the lowest n_elec/2 single-particle levels."""
    N = lat.N
    h = np.zeros((N, N), dtype=np.complex128)
    for (i, j) in _bonds(lat):
        amp = -lat.t * lat.phase(i, j)
        h[i - 1, j - 1] += amp
        h[j - 1, i - 1] += np.conj(amp)
    eps = np.linalg.eigvalsh(h)
    return 2.0 * float(np.sum(eps[:n_elec // 2]))


# ---------------------------------------------------------------- t-J model
def _tj_apply(state, ops, nsite):
    """Apply fermion operators right to left; ops = [(mode, dagger)], mode =
    site (up) or nsite + site (down).  Returns (sign, state) or (0, None)."""
    sign = 1.0
    for mode, dag in reversed(ops):
        occ = (state >> mode) & 1
        if dag == occ:
            return 0.0, None
        if bin(state & ((1 << mode) - 1)).count("1") % 2:
            sign = -sign
        state ^= 1 << mode
    return sign, state


def tj_ground_energies(lat, n_up, n_dn, k=1):
    """Lowest k levels of H = -t sum P(c+_is c_js + h.c.)P + J sum_<ij> (S_i.S_j - n_i n_j / 4)
    in the (n_up, n_dn) sector, no double occupancy, same bonds and Peierls
    factors as the Hubbard case."""
    H, _ = _tj_hamiltonian(lat, n_up, n_dn)
    m = H.shape[0]
    if m <= 400:
        return np.linalg.eigvalsh(H.toarray())[:k]
    w = spla.eigsh(H, k=k, which="SA", return_eigenvectors=False, tol=1e-12)
    return np.sort(w)


def _tj_hamiltonian(lat, n_up, n_dn):
    """The t-J Hamiltonian of tj_ground_energies on the (n_up, n_dn) sector
    and its configurations (bit s: up electron on site s + 1; bit N + s:
    down electron)."""
    N = lat.N
    confs = []
    for ups in combinations(range(N), n_up):
        u = sum(1 << b for b in ups)
        for dns in combinations([x for x in range(N) if not (u >> x) & 1], n_dn):
            confs.append(u | (sum(1 << b for b in dns) << N))
    idx = {c: n for n, c in enumerate(confs)}
    rows, cols, vals = [], [], []

    def add(c, ops, amp):
        s, c2 = _tj_apply(c, ops, N)
        if c2 is None:
            return
        u, d = c2 & ((1 << N) - 1), c2 >> N
        if u & d:
            return  # projected out: double occupancy
        rows.append(idx[c2]); cols.append(idx[c]); vals.append(s * amp)

    for c in confs:
        for (i, j) in _bonds(lat):
            a, b = i - 1, j - 1
            amp = -lat.t * lat.phase(i, j)
            for sh in (0, N):
                add(c, [(a + sh, 1), (b + sh, 0)], amp)
                add(c, [(b + sh, 1), (a + sh, 0)], np.conj(amp))
            # J (S_a.S_b - n_a n_b / 4): diagonal part Sz Sz - n n / 4
            ua, da = (c >> a) & 1, (c >> (a + N)) & 1
            ub, db = (c >> b) & 1, (c >> (b + N)) & 1
            szz = 0.25 * (ua - da) * (ub - db)
            nn = (ua + da) * (ub + db)
            if szz - 0.25 * nn != 0.0:
                rows.append(idx[c]); cols.append(idx[c]); vals.append(lat.J * (szz - 0.25 * nn))
            # (S+_a S-_b + S-_a S+_b) / 2
            add(c, [(a, 1), (a + N, 0), (b + N, 1), (b, 0)], 0.5 * lat.J)
            add(c, [(a + N, 1), (a, 0), (b, 1), (b + N, 0)], 0.5 * lat.J)
    m = len(confs)
    return sp.csr_matrix((vals, (rows, cols)), shape=(m, m), dtype=np.complex128), confs


def tj_singlet_ground_energy(lat, n_elec, k=10, tol=1e-7):
    """Lowest S=0 energy of the t-J model (Sz=0 levels not matched by Sz=1 ones)."""
    e0 = list(tj_ground_energies(lat, n_elec // 2, n_elec // 2, k=k))
    e1 = list(tj_ground_energies(lat, n_elec // 2 + 1, n_elec // 2 - 1, k=k))
    pool = list(e1)
    for e in e0:
        hit = [i for i, f in enumerate(pool) if abs(f - e) < tol]
        if hit:
            pool.pop(hit[0])
            continue
        return float(e)
    raise RuntimeError("no singlet among the lowest levels; raise k")


def hubbard_density_correlations(lat, n_up, n_dn):
    """Lowest state of the (n_up, n_dn) sector: energy, <n_i> and <n_i n_j>
    (Fock-basis exact diagonalisation, sites in lattice order)."""
    N = lat.N
    cu = _configs(N, n_up)
    cd = _configs(N, n_dn)
    hu = _spin_hop(lat, cu)
    hd = _spin_hop(lat, cd)
    H = sp.kron(hu, sp.identity(len(cd)), format="csr") + sp.kron(sp.identity(len(cu)), hd, format="csr")
    au = np.array(cu, dtype=np.int64)
    ad = np.array(cd, dtype=np.int64)
    if lat.U != 0.0:
        dbl = np.array([[bin(int(x & y)).count("1") for y in ad] for x in au], dtype=np.float64).ravel()
        H = H + sp.diags(lat.U * dbl)
    if H.shape[0] <= 2000:
        w, v = np.linalg.eigh(H.toarray())
        e0, psi = w[0], v[:, 0]
    else:
        w, v = spla.eigsh(H, k=1, which="SA", tol=1e-13)
        e0, psi = w[0], v[:, 0]
    p = np.abs(psi) ** 2
    occ_u = np.array([[(c >> s) & 1 for s in range(N)] for c in au], dtype=np.float64)
    occ_d = np.array([[(c >> s) & 1 for s in range(N)] for c in ad], dtype=np.float64)
    n = (occ_u[:, None, :] + occ_d[None, :, :]).reshape(-1, N)   # occupation per basis state
    dens = p @ n
    corr = (n * p[:, None]).T @ n
    return float(e0), dens, corr


def _pair_hop(confs, a, b):
    """c+_a c_b (a != b) on one spin species' configurations, with the sign
    of the occupied sites strictly between a and b."""
    idx = {c: n for n, c in enumerate(confs)}
    lo, hi = min(a, b), max(a, b)
    mask = ((1 << hi) - 1) & ~((1 << (lo + 1)) - 1)
    rows, cols, vals = [], [], []
    for n, c in enumerate(confs):
        if (c >> b) & 1 and not (c >> a) & 1:
            c2 = c ^ (1 << a) ^ (1 << b)
            rows.append(idx[c2]); cols.append(n)
            vals.append(-1.0 if bin(c & mask).count("1") % 2 else 1.0)
    m = len(confs)
    return sp.csr_matrix((vals, (rows, cols)), shape=(m, m), dtype=np.complex128)


def hubbard_spin_correlations(lat, n_up, n_dn):
    """Lowest state of the (n_up, n_dn) sector: energy, <S_i.S_j> and
    3 <S^z_i S^z_j> (equal for a singlet), sites in lattice order.
    S_i.S_j = S^z_i S^z_j + (S^+_i S^-_j + S^-_i S^+_j) / 2 with
    S^+_i S^-_j = c+_iu c_id c+_jd c_ju = -(c+_iu c_ju)(c+_jd c_id) for i != j
    (the up bilinear acts on the up configurations, the down one on the down
    configurations, same ordering as the Hamiltonian here); for i = j,
    S_i.S_i = 3/4 (n_i,u - n_i,d)^2."""
    N = lat.N
    cu = _configs(N, n_up)
    cd = _configs(N, n_dn)
    hu = _spin_hop(lat, cu)
    hd = _spin_hop(lat, cd)
    H = sp.kron(hu, sp.identity(len(cd)), format="csr") + sp.kron(sp.identity(len(cu)), hd, format="csr")
    au = np.array(cu, dtype=np.int64)
    ad = np.array(cd, dtype=np.int64)
    if lat.U != 0.0:
        dbl = np.array([[bin(int(x & y)).count("1") for y in ad] for x in au], dtype=np.float64).ravel()
        H = H + sp.diags(lat.U * dbl)
    if H.shape[0] <= 2000:
        w, v = np.linalg.eigh(H.toarray())
        e0, psi = w[0], v[:, 0]
    else:
        w, v = spla.eigsh(H, k=1, which="SA", tol=1e-13)
        e0, psi = w[0], v[:, 0]
    p = np.abs(psi) ** 2
    occ_u = np.array([[(c >> s) & 1 for s in range(N)] for c in au], dtype=np.float64)
    occ_d = np.array([[(c >> s) & 1 for s in range(N)] for c in ad], dtype=np.float64)
    sz = 0.5 * (occ_u[:, None, :] - occ_d[None, :, :]).reshape(-1, N)
    szsz = (sz * p[:, None]).T @ sz
    ss = np.array(szsz, dtype=np.float64)
    for i in range(N):
        ss[i, i] = 3.0 * szsz[i, i]
        for j in range(N):
            if i == j:
                continue
            # S+_i S-_j and its conjugate S-_i S+_j = -(c+_id c_jd)(c+_ju c_iu)
            pm = -sp.kron(_pair_hop(cu, i, j), _pair_hop(cd, j, i), format="csr")
            mp = -sp.kron(_pair_hop(cu, j, i), _pair_hop(cd, i, j), format="csr")
            ss[i, j] += 0.5 * float(np.real(np.vdot(psi, (pm + mp) @ psi)))
    return float(e0), ss, 3.0 * szsz


def _hubbard_ground(lat, n_up, n_dn):
    """Lowest state of the (n_up, n_dn) sector of the Hubbard model: energy,
    state (up configuration major), up and down configurations."""
    N = lat.N
    cu = _configs(N, n_up)
    cd = _configs(N, n_dn)
    hu = _spin_hop(lat, cu)
    hd = _spin_hop(lat, cd)
    H = sp.kron(hu, sp.identity(len(cd)), format="csr") + sp.kron(sp.identity(len(cu)), hd, format="csr")
    au = np.array(cu, dtype=np.int64)
    ad = np.array(cd, dtype=np.int64)
    if lat.U != 0.0:
        dbl = np.array([[bin(int(x & y)).count("1") for y in ad] for x in au], dtype=np.float64).ravel()
        H = H + sp.diags(lat.U * dbl)
    if H.shape[0] <= 2000:
        w, v = np.linalg.eigh(H.toarray())
        e0, psi = w[0], v[:, 0]
    else:
        w, v = spla.eigsh(H, k=1, which="SA", tol=1e-13)
        e0, psi = w[0], v[:, 0]
    return float(e0), psi, cu, cd


def hubbard_green(lat, n_up, n_dn):
    """Lowest state of the (n_up, n_dn) sector: energy and
    G_ij = sum_s <c+_is c_js> (complex, sites in lattice order)."""
    N = lat.N
    e0, psi, cu, cd = _hubbard_ground(lat, n_up, n_dn)
    au = np.array(cu, dtype=np.int64)
    ad = np.array(cd, dtype=np.int64)
    G = np.zeros((N, N), dtype=np.complex128)
    Iu, Id = sp.identity(len(cu), format="csr"), sp.identity(len(cd), format="csr")
    occ_u = np.array([[(c >> s) & 1 for s in range(N)] for c in au], dtype=np.float64)
    occ_d = np.array([[(c >> s) & 1 for s in range(N)] for c in ad], dtype=np.float64)
    n = (occ_u[:, None, :] + occ_d[None, :, :]).reshape(-1, N)
    p = np.abs(psi) ** 2
    for i in range(N):
        G[i, i] = p @ n[:, i]
        for j in range(N):
            if i != j:
                op = sp.kron(_pair_hop(cu, i, j), Id, format="csr") + sp.kron(Iu, _pair_hop(cd, i, j), format="csr")
                G[i, j] = np.vdot(psi, op @ psi)
    return float(e0), G


def _annihilate(src, dst, site):
    """c_site from configurations src to dst of one spin species, with the
    sign of the occupied sites below site."""
    idx = {c: n for n, c in enumerate(dst)}
    low = (1 << site) - 1
    rows, cols, vals = [], [], []
    for n, c in enumerate(src):
        if (c >> site) & 1:
            rows.append(idx[c ^ (1 << site)]); cols.append(n)
            vals.append(-1.0 if bin(c & low).count("1") % 2 else 1.0)
    return sp.csr_matrix((vals, (rows, cols)), shape=(len(dst), len(src)), dtype=np.complex128)


def hubbard_pair_correlations(lat, n_up, n_dn, bonds):
    """Lowest state of the (n_up, n_dn) sector: energy and the singlet-pair
    correlations P[x, y] = <D+_x D_y> for the given bonds (i, j) (sites in
    lattice order, 1-based), D+_ij = (c+_i,up c+_j,dn - c+_i,dn c+_j,up) /
    sqrt(2).  Up operators are ordered before down operators."""
    N = lat.N
    e0, psi, cu, cd = _hubbard_ground(lat, n_up, n_dn)
    cu1, cd1 = _configs(N, n_up - 1), _configs(N, n_dn - 1)
    Psi = psi.reshape(len(cu), len(cd))
    up = [_annihilate(cu, cu1, s) for s in range(N)]
    dn = [_annihilate(cd, cd1, s) for s in range(N)]
    su0 = -1.0 if n_up % 2 else 1.0           # down operator passing the n_up up electrons
    su1 = -1.0 if (n_up - 1) % 2 else 1.0     # ... after one up electron was removed
    vecs = []
    for (i, j) in bonds:
        a, b = i - 1, j - 1
        # D_ij = (c_j,dn c_i,up - c_j,up c_i,dn) / sqrt(2)
        t1 = su1 * (up[a] @ Psi) @ dn[b].T
        t2 = up[b] @ (su0 * Psi @ dn[a].T)
        vecs.append(np.asarray(t1 - t2).ravel() / np.sqrt(2.0))
    P = np.array([[np.vdot(vx, vy) for vy in vecs] for vx in vecs])
    return e0, P


def tj_singlet_correlations(lat, n_elec, bonds, k=10):
    """The t-J singlet ground state (tj_singlet_ground_energy picked out of the
    lowest levels of the S_z = 0 sector): energy, G_ij = sum_s <c+_is c_js>
    with projected operators, and the singlet-pair correlations
    <D+_x D_y> of the given bonds, D+_ij = (c+_i,up c+_j,dn - c+_i,dn c+_j,up)
    / sqrt(2).  On a state without double occupancy the plain annihilators
    equal the projected ones; a creation that makes a double occupancy
    gives zero."""
    N = lat.N
    e_s = tj_singlet_ground_energy(lat, n_elec)
    H, confs = _tj_hamiltonian(lat, n_elec // 2, n_elec // 2)
    w, v = np.linalg.eigh(H.toarray()) if H.shape[0] <= 3000 else spla.eigsh(H, k=k, which="SA", tol=1e-13)
    order = np.argsort(w)
    w, v = w[order], v[:, order]
    i0 = int(np.argmin(np.abs(w - e_s)))
    if abs(w[i0] - e_s) > 1e-8 or (i0 + 1 < len(w) and abs(w[i0 + 1] - w[i0]) < 1e-8) or \
            (i0 > 0 and abs(w[i0] - w[i0 - 1]) < 1e-8):
        raise RuntimeError("singlet ground state not isolated in the S_z = 0 sector")
    psi = v[:, i0]
    amp = dict(zip(confs, psi))

    def apply(ops):
        out = {}
        for c, a in amp.items():
            sgn, c2 = _tj_apply(c, ops, N)
            if c2 is None or (c2 & ((1 << N) - 1)) & (c2 >> N):
                continue
            out[c2] = out.get(c2, 0.0) + sgn * a
        return out

    G = np.zeros((N, N), dtype=np.complex128)
    for i in range(N):
        for j in range(N):
            for sh in (0, N):
                phi = apply([(i + sh, 1), (j + sh, 0)])
                G[i, j] += sum(np.conj(amp.get(c, 0.0)) * a for c, a in phi.items())
    vecs = []
    for (i, j) in bonds:
        a, b = i - 1, j - 1
        t1 = apply([(b + N, 0), (a, 0)])
        t2 = apply([(b, 0), (a + N, 0)])
        vec = dict(t1)
        for c, x in t2.items():
            vec[c] = vec.get(c, 0.0) - x
        vecs.append({c: x / np.sqrt(2.0) for c, x in vec.items()})
    P = np.array([[sum(np.conj(vx.get(c, 0.0)) * y for c, y in vy.items()) for vy in vecs] for vx in vecs])
    return float(w[i0]), G, P


def tj_singlet_spin_correlations(lat, n_elec, k=10):
    """<S_i . S_j> (N x N) of the t-J singlet ground state of
    tj_singlet_correlations: S^z_i S^z_j + (S^+_i S^-_j + S^-_i S^+_j) / 2,
    with S^+_i = c+_i,up c_i,dn; the diagonal is 3/4 <n_i>."""
    N = lat.N
    e_s = tj_singlet_ground_energy(lat, n_elec)
    H, confs = _tj_hamiltonian(lat, n_elec // 2, n_elec // 2)
    w, v = np.linalg.eigh(H.toarray()) if H.shape[0] <= 3000 else spla.eigsh(H, k=k, which="SA", tol=1e-13)
    i0 = int(np.argmin(np.abs(w - e_s)))
    psi = v[:, i0]
    amp = dict(zip(confs, psi))
    ss = np.zeros((N, N))
    for i in range(N):
        for j in range(N):
            if i == j:
                ss[i, i] = sum(abs(a) ** 2 * 0.75 * (((c >> i) & 1) + ((c >> (i + N)) & 1)) for c, a in amp.items())
                continue
            val = 0.0
            for c, a in amp.items():
                szi = 0.5 * (((c >> i) & 1) - ((c >> (i + N)) & 1))
                szj = 0.5 * (((c >> j) & 1) - ((c >> (j + N)) & 1))
                val += abs(a) ** 2 * szi * szj
                for ops in ([(i, 1), (i + N, 0), (j + N, 1), (j, 0)], [(i + N, 1), (i, 0), (j, 1), (j + N, 0)]):
                    sgn, c2 = _tj_apply(c, ops, N)
                    if c2 is not None:
                        val += 0.5 * (np.conj(amp.get(c2, 0.0)) * sgn * a).real
            ss[i, j] = val
    return float(w[i0]), ss
