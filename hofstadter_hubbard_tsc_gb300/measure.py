"""Measurements on the GPU DMRG state: site profiles and cross-cut correlations
of diagonal (rank-0) site operators (code/measure.f90, code/correlation.f90).

measure_operator_dia (code/measure.f90:3-62): <O_i> for every site.  The
operator of block site i is carried to the block of the current superblock as
Get_sys_oper_dia / Get_env_oper_dia do (code/get_ham.f90:1244-1380): embedded
in the enlarged basis of length i (update_site_dia), truncated, then for each
longer block embedded as a block operator (update_block_dia) and truncated,
with the bases and truncation operators the sweep left on the device.  Then
phi_i = (O_i x 1) psi is one matvec of a one-term plan (the block_vec_dia /
vec_block_dia / site_vec_site_dia kernels of model_wave: measure_sys_block and
its siblings, code/measure.f90:611-862), and <O_i> = Re <psi|phi_i>.

Cross-cut correlations <O_a O_b>, a on the system half and b on the
environment half (the cross part of Get_density_cor, code/correlation.f90:43):
Re <phi_a|chi_b> with chi_b = (1 x O_b) psi, one dot product per pair on the
device.  Sites are numbered like the reference's output: system block site i
is site i, environment block site j is site N - j + 1.

Same-side density correlations <n_a n_b> (a < b on one half): n_a carried to
the block of length b - 1 and embedded in the enlarged basis of length b, n_b
embedded as the new site, their product formed there the way
Get_hamiltonian_dia forms the n.n bond (code/get_ham.f90:852-941), then
truncated and carried to the current block and measured with block_vec_dia /
vec_block_dia; a block site with its half's middle site is one
block_site_vec_dia / vec_block_site_dia term; <n_i n_i> = <n_i> + 2 <d_i>.

Same-side spin pairs: S_a carried (rank 1) to the block of length b - 1 and
the scalar product with the new site's S added in the enlarged basis as the
S.S bond of Get_hamiltonian_ndia (code/get_ham.f90:954-1152), then carried
like a scalar; a block site with its half's middle site is the
block_site_vec_ndia / vec_block_site_ndia S.S term.

Cross-cut spin correlations <S_a . S_b> (the spin part of Get_spin_cor,
code/correlation.f90): the rank-1 site operator sd is carried to its block
with the ndia embeddings and truncation (update_site_ndia, update_block_ndia,
update_trun_ndia, code/update.f90), and each pair is one matvec of a one-term
plan of the kernel that carries the Hamiltonian's S.S bond in that geometry
(block-block, block-site, site-block, site-site; the environment operator
through block_transfer_trans); that term holds J S.S as jd = -sqrt(3) J
times the unit-coefficient term, so <S_a . S_b> = -sqrt(3) <psi|T_ab psi>.

Cross-cut electron correlations G_ab = sum_s <c+_as c_bs> (the 'F' call of
Get_density_cor, code/quantum.f90:531): elec_up of site a and elec_down of
site b carried with the fermion ('F') ndia embeddings, each pair the hopping
kernel of its geometry (the Hamiltonian's own t term, code/mat_vec.f90:
3502-3615) with coefficient 1 and with i.  That term holds X + X^+ with
X = sum_s c+_as c_bs / sqrt(2), so Re G = <T_1> / sqrt(2) and
Im G = -<T_i> / sqrt(2).

Cross-cut singlet-pair correlations <D+_x D_y> (Get_mSCOP_Operator_cor0,
code/correlation.f90:198-327): the pair creator of a bond inside a block is
the product of the two sites' elec_up operators in the basis of the later
site, coupled to rank 0 (block_mul_block_ndia, hh_block_product), truncated
and carried as a boson operator.  sys_block_env_block_cor_ndia
(code/correlation.f90:1666-1929) has the coefficients of the block-block
term with the environment creator untransposed; that term also holds its
h.c., so with coefficients 1 and i, <D+_x D_y> = (<T_1> - i <T_i>) / 2.
Same-side pairs (x before y inside the system block) multiply the creator
of x by the two elec_down operators of y in turn (ranks 1/2, then 0) and
measure the scalar with block_vec_dia (no h.c.): <T_1> - i <T_i>.
"""
import ctypes as C

import numpy as np

from . import _lib
from .device import DBlock, DWave
from .step import update_trun
from .types import SubBlock, TotalBlock


def _embed(dev, mode, op, dbasis, side, flag="B"):
    h = C.c_void_p()
    dev.check(dev.lib.hh_enlarge_operator(dev.h, mode, op.h, dbasis.h, ord(flag), side, C.byref(h)))
    return DBlock.from_handle(dev, h)


def _carry(dev, op, i, length, bases, truns, side, rank1=False, flag="B"):
    """Operator of block site i in the truncated block of `length` sites
    (rank1: an operator of nonzero rank through the ndia embeddings, flag
    'B' boson or 'F' fermion)."""
    site_mode, block_mode = (3, 2) if rank1 else (1, 0)
    dia = not rank1
    cur = op if i <= 1 else update_trun(dev, _embed(dev, site_mode, op, bases[i][1], side, flag), truns[i], dia=dia)
    for L in range(i + 1, length + 1):
        cur = update_trun(dev, _embed(dev, block_mode, cur, bases[L][1], side, flag), truns[L], dia=dia)
    return cur


SPIN_NORM = -np.sqrt(3.0)  # <S_a . S_b> per unit-coefficient sd x sd term


def _spin_pair_operator(dev, sd, a, b, length, bases, truns, side):
    """S_a . S_b (block sites a < b <= length) in the truncated block of
    `length` sites: S_a carried (rank 1) to the block of length b - 1, the
    scalar product with the new site's sd added in the enlarged basis as the
    S.S bond of Get_hamiltonian_ndia (coefficient -sqrt(3)), then truncated
    and carried."""
    basis, dbasis = bases[b]
    Sa = _carry(dev, sd, a, b - 1, bases, truns, side, rank1=True)
    P = DBlock.upload(dev, TotalBlock(b, 0, 0, [SubBlock(sec.new_num_up, sec.new_num_down, 0,
                                                         np.zeros((sec.dim, sec.dim))) for sec in basis.sectors]))
    c = np.array([SPIN_NORM, 0.0])
    dev.check(dev.lib.hh_ham_add_bond(dev.h, P.h, Sa.h, sd.h, 0, dbasis.h, c.ctypes.data_as(C.POINTER(C.c_double)),
                                      ord("B"), ord("S") if side == 0 else ord("E")))
    cur = update_trun(dev, P, truns[b], dia=True)
    for L in range(b + 1, length + 1):
        cur = update_trun(dev, _embed(dev, 0, cur, bases[L][1], side), truns[L], dia=True)
    return cur


def _pair_operator(dev, op, a, b, length, bases, truns, side):
    """n_a n_b (block sites a < b <= length) in the truncated block of
    `length` sites."""
    basis, dbasis = bases[b]
    A = _embed(dev, 0, _carry(dev, op, a, b - 1, bases, truns, side), dbasis, side)
    B = _embed(dev, 1, op, dbasis, side)
    P = DBlock.upload(dev, TotalBlock(b, 0, 0, [SubBlock(sec.new_num_up, sec.new_num_down, 0,
                                                         np.zeros((sec.dim, sec.dim))) for sec in basis.sectors]))
    one = np.array([1.0, 0.0])
    dev.check(dev.lib.hh_ham_add_product(dev.h, P.h, A.h, B.h, one.ctypes.data_as(C.POINTER(C.c_double))))
    cur = update_trun(dev, P, truns[b], dia=True)
    for L in range(b + 1, length + 1):
        cur = update_trun(dev, _embed(dev, 0, cur, bases[L][1], side), truns[L], dia=True)
    return cur


def _hop_pair_operators(dev, op, site, a, b, length, bases, truns, side):
    """The hopping bond of Get_hamiltonian_ndia between block site a (op
    carried with the fermion ndia embeddings to the block of length b - 1)
    and the new site b (site operator through block_transfer_trans), formed
    with coefficients 1 and i in the enlarged basis of length b, each
    truncated and carried as a scalar to the block of `length` sites."""
    basis, dbasis = bases[b]
    out = []
    for coef in (1.0, 1j):
        Ca = _carry(dev, op, a, b - 1, bases, truns, side, rank1=True, flag="F")
        P = DBlock.upload(dev, TotalBlock(b, 0, 0, [SubBlock(sec.new_num_up, sec.new_num_down, 0,
                                                             np.zeros((sec.dim, sec.dim))) for sec in basis.sectors]))
        c = np.array([complex(coef).real, complex(coef).imag])
        dev.check(dev.lib.hh_ham_add_bond(dev.h, P.h, Ca.h, site.h, 1, dbasis.h,
                                          c.ctypes.data_as(C.POINTER(C.c_double)), ord("F"),
                                          ord("S") if side == 0 else ord("E")))
        cur = update_trun(dev, P, truns[b], dia=True)
        for L in range(b + 1, length + 1):
            cur = update_trun(dev, _embed(dev, 0, cur, bases[L][1], side), truns[L], dia=True)
        out.append(cur)
    return out


def _fermion_in_basis(dev, op, a, b, bases, truns, side):
    """Get_sys_oper_ndia / Get_env_oper_ndia with Truns = .false.
    (code/get_ham.f90:1631-1695): the fermion operator of site a in the
    enlarged, untruncated basis of length b >= a."""
    if a == b:
        return op if b <= 1 else _embed(dev, 3, op, bases[b][1], side, "F")
    cur = _carry(dev, op, a, b - 1, bases, truns, side, rank1=True, flag="F")
    return _embed(dev, 2, cur, bases[b][1], side, "F")


def _pair_creator(dev, up, a, b, length, bases, truns, side):
    """Singlet pair creator [c+_a c+_b]^0 of block sites a < b
    (Get_SCOP_Operator_Sys / _Env with 'S0', code/correlation.f90:2659-2772):
    the product of the two elec_up operators in the basis of length b
    (hh_block_product, rank 0), truncated, then carried as a boson operator
    to the block of `length` sites."""
    A = _fermion_in_basis(dev, up, a, b, bases, truns, side)
    Bo = _fermion_in_basis(dev, up, b, b, bases, truns, side)
    h = C.c_void_p()
    one = np.array([1.0, 0.0])
    dev.check(dev.lib.hh_block_product(dev.h, A.h, Bo.h, 0, bases[b][1].h, one.ctypes.data_as(C.POINTER(C.c_double)),
                                       C.byref(h)))
    cur = update_trun(dev, DBlock.from_handle(dev, h), truns[b], dia=False)
    for L in range(b + 1, length + 1):
        cur = update_trun(dev, _embed(dev, 2, cur, bases[L][1], side, "B"), truns[L], dia=False)
    return cur


def _product(dev, o1, o2, down_dif, dbasis):
    """hh_block_product: (o1 o2) coupled to rank down_dif / 2 in dbasis."""
    h = C.c_void_p()
    one = np.array([1.0, 0.0])
    dev.check(dev.lib.hh_block_product(dev.h, o1.h, o2.h, down_dif, dbasis.h, one.ctypes.data_as(C.POINTER(C.c_double)),
                                       C.byref(h)))
    return DBlock.from_handle(dev, h)


def _carry_untruncated(dev, op, a, b, bases, truns, side, flag):
    """Change_sys_oper_ndia with Truns = .false. (code/get_ham.f90:1767-1818):
    a block operator of the truncated block of length a embedded in the
    enlarged, untruncated basis of length b > a."""
    cur = op
    for L in range(a + 1, b):
        cur = update_trun(dev, _embed(dev, 2, cur, bases[L][1], side, flag), truns[L], dia=False)
    return _embed(dev, 2, cur, bases[b][1], side, flag)


def _pair_pair_operator(dev, up, dn, bond_x, bond_y, length, bases, truns):
    """The scalar D+_x D_y of two bonds inside the system block, x before y
    (Get_sys_two / Get_sys_two1, code/correlation.f90:331-428): the pair
    creator of x truncated at its later site, embedded up to the first site
    of y and multiplied by that site's elec_down (rank 1/2), truncated,
    embedded (fermion) up to the second site of y and multiplied by its
    elec_down to rank 0, then truncated and carried as a scalar."""
    a1, a2 = sorted(bond_x)
    a3, a4 = sorted(bond_y)
    P = _product(dev, _fermion_in_basis(dev, up, a1, a2, bases, truns, 0),
                 _fermion_in_basis(dev, up, a2, a2, bases, truns, 0), 0, bases[a2][1])
    P = update_trun(dev, P, truns[a2], dia=False)
    X = _product(dev, _carry_untruncated(dev, P, a2, a3, bases, truns, 0, "B"),
                 _fermion_in_basis(dev, dn, a3, a3, bases, truns, 0), 1, bases[a3][1])
    X = update_trun(dev, X, truns[a3], dia=False)
    X = _product(dev, _carry_untruncated(dev, X, a3, a4, bases, truns, 0, "F"),
                 _fermion_in_basis(dev, dn, a4, a4, bases, truns, 0), 0, bases[a4][1])
    X = update_trun(dev, X, truns[a4], dia=True)
    for L in range(a4 + 1, length + 1):
        X = update_trun(dev, _embed(dev, 0, X, bases[L][1], 0), truns[L], dia=True)
    return X


def structure_factor(corr, W, L, nx_cut=0):
    """Get_structure_factor_cut (code/measure.f90:2159-2236) on the host:
    S(kx, ky) = Re(f^T C f*) / N' over the sites outside nx_cut columns at
    either end, f_x = exp(i (kx X_x + ky Y_x)), C the real part of the
    correlation matrix (the diagonal enters with phase 1), kx = 2 pi i /
    (L - 2 nx_cut), i = 0..L - 2 nx_cut, ky = 2 pi j / W, j = 0..W.  Returns
    (kx / pi, ky / pi, S[i, j])."""
    C = np.real(np.asarray(corr, dtype=np.complex128))
    N = W * L
    if C.shape != (N, N) or not 0 <= 2 * nx_cut < L:
        raise ValueError("correlation matrix must be N x N and 2 nx_cut < L")
    kxn = L - 2 * nx_cut
    kx = 2.0 * np.pi * np.arange(kxn + 1) / kxn
    ky = 2.0 * np.pi * np.arange(W + 1) / W
    sites = np.arange(nx_cut * W, N - nx_cut * W)
    X, Y = sites // W, sites % W
    Cw = C[np.ix_(sites, sites)]
    f = np.exp(1j * (kx[:, None, None] * X[None, None, :] + ky[None, :, None] * Y[None, None, :]))
    S = np.einsum("ijx,xy,ijy->ij", f, Cw, np.conj(f)).real / len(sites)
    return kx / np.pi, ky / np.pi, S


class Measurement:
    """Measurements on the current superblock of a ``GPUDMRG`` (its last
    Lanczos state and the bases and truncations it keeps on the device)."""

    def __init__(self, dmrg):
        self.d = dmrg
        self.dev = dmrg.dev
        self.wave, sup = dmrg.wave
        self.N = dmrg.lat.N
        self.sys_bs = dmrg.sys_bases[sup.sys_len][1]
        self.env_bs = dmrg.env_bases[sup.env_len][1]
        self.Ls, self.Le = sup.sys_len - 1, sup.env_len - 1

    def _apply(self, kind, op0, op1=None, trans1=0, flag="B", coef=1.0):
        """(one term) psi as a new device wave."""
        dev, w = self.dev, self.wave
        t = (_lib.HHTerm * 1)()
        c = complex(coef)
        t[0] = _lib.HHTerm(kind, ord(flag), ord(flag), 0, trans1, op0.h, op1.h if op1 is not None else None, c.real,
                           c.imag)
        plan = C.c_void_p()
        dev.check(dev.lib.hh_plan_create(dev.h, self.sys_bs.h, self.env_bs.h, w.h, 1, t, C.byref(plan)))
        out = DWave(dev, w.layout, w.sys_len, w.env_len)
        try:
            dev.check(dev.lib.hh_matvec(plan, w.h, out.h, _lib.HH_PREC_FP64))
        finally:
            dev.lib.hh_plan_free(plan)
        return out

    def site_vectors(self, name):
        """{site: (side, phi)} with phi = O_site psi (side 0 system half, 1
        environment half); name is a site operator of the sweep ("num_elec",
        "double", ...)."""
        d, dev = self.d, self.dev
        op, one = d.d_st[name], d.d_st["si"]
        out = {}
        for i in range(1, self.Ls + 1):
            o = _carry(dev, op, i, self.Ls, d.sys_bases, d.sys_truns, 0)
            out[i] = (0, self._apply(_lib.BLOCK_VEC_DIA, o))
        out[self.Ls + 1] = (0, self._apply(_lib.SITE_VEC_SITE_DIA, op, one))
        out[self.N - self.Le] = (1, self._apply(_lib.SITE_VEC_SITE_DIA, one, op))
        for j in range(1, self.Le + 1):
            o = _carry(dev, op, j, self.Le, d.env_bases, d.env_truns, 1)
            out[self.N - j + 1] = (1, self._apply(_lib.VEC_BLOCK_DIA, o))
        return out

    def site_profile(self, name="num_elec"):
        """measure_operator_dia: <O_i>, i = 1..N."""
        prof = np.zeros(self.N)
        for s, (_, phi) in self.site_vectors(name).items():
            prof[s - 1] = self.wave.dot(phi)
            phi.free()
        return prof

    def cross_correlations(self, name_a="num_elec", name_b="num_elec"):
        """<O_a O_b>, a on the system half, b on the environment half:
        (sites_a, sites_b, matrix)."""
        va = self.site_vectors(name_a)
        vb = va if name_b == name_a else self.site_vectors(name_b)
        sa = sorted(s for s, (side, _) in va.items() if side == 0)
        sb = sorted(s for s, (side, _) in vb.items() if side == 1)
        m = np.array([[va[a][1].dot(vb[b][1]) for b in sb] for a in sa])
        for v in {id(x[1]): x[1] for x in list(va.values()) + list(vb.values())}.values():
            v.free()
        return sa, sb, m

    def spin_correlations(self):
        """<S_a . S_b>, a on the system half, b on the environment half:
        (sites_a, sites_b, matrix)."""
        d, dev, N = self.d, self.dev, self.N
        sd = d.d_st["sd"]
        a_ops = [(i, _carry(dev, sd, i, self.Ls, d.sys_bases, d.sys_truns, 0, rank1=True))
                 for i in range(1, self.Ls + 1)] + [(self.Ls + 1, None)]
        b_ops = [(N - self.Le, None)] + [(N - j + 1, _carry(dev, sd, j, self.Le, d.env_bases, d.env_truns, 1,
                                                            rank1=True)) for j in range(1, self.Le + 1)]
        sa = [a for a, _ in a_ops]
        sb = sorted(b for b, _ in b_ops)
        m = np.zeros((len(sa), len(sb)))
        for ia, (a, oa) in enumerate(a_ops):
            for b, ob in b_ops:
                if oa is not None and ob is not None:
                    phi = self._apply(_lib.BLOCK_VEC_BLOCK_NDIA, oa, ob, trans1=1)
                elif oa is not None:
                    phi = self._apply(_lib.BLOCK_VEC_SITE_NDIA, oa, sd)
                elif ob is not None:
                    phi = self._apply(_lib.SITE_VEC_BLOCK_NDIA, sd, ob, trans1=1)
                else:
                    phi = self._apply(_lib.SITE_VEC_SITE_NDIA, sd, sd)
                m[ia, sb.index(b)] = SPIN_NORM * self.wave.dot(phi)
                phi.free()
        return sa, sb, m

    def electron_correlations(self):
        """G_ab = sum_s <c+_as c_bs>, a on the system half, b on the
        environment half: (sites_a, sites_b, complex matrix)."""
        d, dev, N = self.d, self.dev, self.N
        up, dn = d.d_st["elec_up"], d.d_st["elec_down"]
        a_ops = [(i, _carry(dev, up, i, self.Ls, d.sys_bases, d.sys_truns, 0, rank1=True, flag="F"))
                 for i in range(1, self.Ls + 1)] + [(self.Ls + 1, None)]
        b_ops = [(N - self.Le, None)] + [(N - j + 1, _carry(dev, dn, j, self.Le, d.env_bases, d.env_truns, 1,
                                                            rank1=True, flag="F")) for j in range(1, self.Le + 1)]
        sa = [a for a, _ in a_ops]
        sb = sorted(b for b, _ in b_ops)
        m = np.zeros((len(sa), len(sb)), dtype=np.complex128)
        for ia, (a, oa) in enumerate(a_ops):
            for b, ob in b_ops:
                t = []
                for coef in (1.0, 1j):
                    if oa is not None and ob is not None:
                        phi = self._apply(_lib.BLOCK_VEC_BLOCK_NDIA, oa, ob, 1, "F", coef)
                    elif oa is not None:
                        phi = self._apply(_lib.BLOCK_VEC_SITE_NDIA, oa, dn, 1, "F", coef)
                    elif ob is not None:
                        phi = self._apply(_lib.SITE_VEC_BLOCK_NDIA, up, ob, 1, "F", coef)
                    else:
                        phi = self._apply(_lib.SITE_VEC_SITE_NDIA, up, dn, 1, "F", coef)
                    t.append(self.wave.dot(phi))
                    phi.free()
                m[ia, sb.index(b)] = (t[0] - 1j * t[1]) / np.sqrt(2.0)
        return sa, sb, m

    def pairing_correlations(self, sys_bonds, env_bonds):
        """Cross-cut singlet-pair correlations <D+_x D_y> of
        Get_mSCOP_Operator_cor0 (code/correlation.f90:198-327) for bonds x
        inside the system block and y inside the environment block (sites in
        the output numbering): (len(sys_bonds), len(env_bonds)) complex."""
        d, dev, N, w = self.d, self.dev, self.N, self.wave
        up = d.d_st["elec_up"]
        for a, b in sys_bonds:
            if not (1 <= min(a, b) < max(a, b) <= self.Ls):
                raise ValueError(f"bond ({a}, {b}) is not inside the system block (sites 1..{self.Ls})")
        for a, b in env_bonds:
            if not (N - self.Le + 1 <= min(a, b) < max(a, b) <= N):
                raise ValueError(f"bond ({a}, {b}) is not inside the environment block "
                                 f"(sites {N - self.Le + 1}..{N})")
        A = [_pair_creator(dev, up, min(a, b), max(a, b), self.Ls, d.sys_bases, d.sys_truns, 0) for a, b in sys_bonds]
        B = [_pair_creator(dev, up, min(N - a + 1, N - b + 1), max(N - a + 1, N - b + 1), self.Le, d.env_bases,
                           d.env_truns, 1) for a, b in env_bonds]
        m = np.zeros((len(A), len(B)), dtype=np.complex128)
        for i, x in enumerate(A):
            for j, y in enumerate(B):
                t = []
                for coef in (1.0, 1j):
                    phi = self._apply(_lib.BLOCK_VEC_BLOCK_NDIA, x, y, 0, "B", coef)
                    t.append(w.dot(phi))
                    phi.free()
                m[i, j] = (t[0] - 1j * t[1]) / 2.0
        return m

    def pairing_correlations_sys(self, bonds_x, bonds_y):
        """Same-side singlet-pair correlations <D+_x D_y> of
        Get_mSCOP_Operator_cor0 (code/correlation.f90:226-262) for bonds x
        and y inside the system block, every site of x before every site of
        y: measure_sys_block of the scalar D+_x D_y, as
        <T_1> - i <T_i> of one-term block_vec_dia plans with coefficients 1
        and i.  Returns the (len(bonds_x), len(bonds_y)) complex matrix."""
        d, dev, w = self.d, self.dev, self.wave
        for x in bonds_x:
            for y in bonds_y:
                if not (1 <= min(x) and max(x) < min(y) and max(y) <= self.Ls):
                    raise ValueError(f"bonds {x}, {y} are not ordered inside the system block (sites 1..{self.Ls})")
        up, dn = d.d_st["elec_up"], d.d_st["elec_down"]
        m = np.zeros((len(bonds_x), len(bonds_y)), dtype=np.complex128)
        for i, x in enumerate(bonds_x):
            for j, y in enumerate(bonds_y):
                O = _pair_pair_operator(dev, up, dn, x, y, self.Ls, d.sys_bases, d.sys_truns)
                t = []
                for coef in (1.0, 1j):
                    phi = self._apply(_lib.BLOCK_VEC_DIA, O, coef=coef)
                    t.append(w.dot(phi))
                    phi.free()
                m[i, j] = t[0] - 1j * t[1]
        return m

    def density_correlations(self, name="num_elec"):
        """<n_i n_j> for all sites i, j (N x N): cross-cut pairs, same-side
        pairs from carried products, the diagonal from <n_i> + 2 <d_i>."""
        d, dev, N, w = self.d, self.dev, self.N, self.wave
        op, st_op = d.d_st[name], d.d_st[name]
        Ls, Le = self.Ls, self.Le
        m = np.zeros((N, N))
        sa, sb, cross = self.cross_correlations(name, name)
        for ia, a in enumerate(sa):
            for ib, b in enumerate(sb):
                m[a - 1, b - 1] = m[b - 1, a - 1] = cross[ia, ib]

        def measure(kind, o0, o1=None):
            phi = self._apply(kind, o0, o1)
            v = w.dot(phi)
            phi.free()
            return v

        for b in range(2, Ls + 1):
            for a in range(1, b):
                v = measure(_lib.BLOCK_VEC_DIA, _pair_operator(dev, op, a, b, Ls, d.sys_bases, d.sys_truns, 0))
                m[a - 1, b - 1] = m[b - 1, a - 1] = v
        for a in range(1, Ls + 1):
            v = measure(_lib.BLOCK_SITE_VEC_DIA, _carry(dev, op, a, Ls, d.sys_bases, d.sys_truns, 0), st_op)
            m[a - 1, Ls] = m[Ls, a - 1] = v
        for jb in range(2, Le + 1):
            for ja in range(1, jb):
                v = measure(_lib.VEC_BLOCK_DIA, _pair_operator(dev, op, ja, jb, Le, d.env_bases, d.env_truns, 1))
                i, j = N - ja, N - jb
                m[i, j] = m[j, i] = v
        for ja in range(1, Le + 1):
            v = measure(_lib.VEC_BLOCK_SITE_DIA, _carry(dev, op, ja, Le, d.env_bases, d.env_truns, 1), st_op)
            i, j = N - ja, N - Le - 1
            m[i, j] = m[j, i] = v
        n = self.site_profile(name)
        dbl = self.site_profile("double")
        for i in range(N):
            m[i, i] = n[i] + 2.0 * dbl[i]
        return m

    def spin_correlations_all(self):
        """<S_i . S_j> for all sites i, j (N x N): cross-cut pairs, same-side
        pairs from carried bond products, block-middle-site terms, diagonal
        3/4 (<n_i> - 2 <d_i>)."""
        d, dev, N, w = self.d, self.dev, self.N, self.wave
        sd = d.d_st["sd"]
        Ls, Le = self.Ls, self.Le
        m = np.zeros((N, N))
        sa, sb, cross = self.spin_correlations()
        for ia, a in enumerate(sa):
            for ib, b in enumerate(sb):
                m[a - 1, b - 1] = m[b - 1, a - 1] = cross[ia, ib]

        def measure(kind, o0, o1=None):
            phi = self._apply(kind, o0, o1)
            v = w.dot(phi)
            phi.free()
            return v

        for b in range(2, Ls + 1):
            for a in range(1, b):
                P = _spin_pair_operator(dev, sd, a, b, Ls, d.sys_bases, d.sys_truns, 0)
                m[a - 1, b - 1] = m[b - 1, a - 1] = measure(_lib.BLOCK_VEC_DIA, P)
        for a in range(1, Ls + 1):
            Sa = _carry(dev, sd, a, Ls, d.sys_bases, d.sys_truns, 0, rank1=True)
            m[a - 1, Ls] = m[Ls, a - 1] = SPIN_NORM * measure(_lib.BLOCK_SITE_VEC_NDIA, Sa, sd)
        for jb in range(2, Le + 1):
            for ja in range(1, jb):
                P = _spin_pair_operator(dev, sd, ja, jb, Le, d.env_bases, d.env_truns, 1)
                i, j = N - ja, N - jb
                m[i, j] = m[j, i] = measure(_lib.VEC_BLOCK_DIA, P)
        for ja in range(1, Le + 1):
            Sj = _carry(dev, sd, ja, Le, d.env_bases, d.env_truns, 1, rank1=True)
            i, j = N - ja, N - Le - 1
            m[i, j] = m[j, i] = SPIN_NORM * measure(_lib.VEC_BLOCK_SITE_NDIA, Sj, sd)
        n = self.site_profile("num_elec")
        dbl = self.site_profile("double")
        for i in range(N):
            m[i, i] = 0.75 * (n[i] - 2.0 * dbl[i])
        return m

    def electron_correlations_all(self):
        """G_ij = sum_s <c+_is c_js> for all sites i, j (N x N, complex,
        Hermitian): cross-cut pairs, same-side pairs from the hopping bond
        formed in the enlarged basis (system side: block elec_up with the new
        site's elec_down; environment side: block elec_down with the new
        site's elec_up), block-middle-site hopping terms, diagonal <n_i>."""
        d, dev, N, w = self.d, self.dev, self.N, self.wave
        up, dn = d.d_st["elec_up"], d.d_st["elec_down"]
        Ls, Le = self.Ls, self.Le
        G = np.zeros((N, N), dtype=np.complex128)

        def put(i, j, v):
            G[i, j] = v
            G[j, i] = np.conj(v)

        sa, sb, cross = self.electron_correlations()
        for ia, a in enumerate(sa):
            for ib, b in enumerate(sb):
                put(a - 1, b - 1, cross[ia, ib])

        def scalar(kind, ops):
            t = []
            for o in ops:
                phi = self._apply(kind, o)
                t.append(w.dot(phi))
                phi.free()
            return (t[0] - 1j * t[1]) / np.sqrt(2.0)

        def term(kind, o0, o1):
            t = []
            for coef in (1.0, 1j):
                phi = self._apply(kind, o0, o1, 1, "F", coef)
                t.append(w.dot(phi))
                phi.free()
            return (t[0] - 1j * t[1]) / np.sqrt(2.0)

        for b in range(2, Ls + 1):
            for a in range(1, b):
                ops = _hop_pair_operators(dev, up, dn, a, b, Ls, d.sys_bases, d.sys_truns, 0)
                put(a - 1, b - 1, scalar(_lib.BLOCK_VEC_DIA, ops))
        for a in range(1, Ls + 1):
            oa = _carry(dev, up, a, Ls, d.sys_bases, d.sys_truns, 0, rank1=True, flag="F")
            put(a - 1, Ls, term(_lib.BLOCK_SITE_VEC_NDIA, oa, dn))
        for jb in range(2, Le + 1):
            for ja in range(1, jb):
                ops = _hop_pair_operators(dev, dn, up, ja, jb, Le, d.env_bases, d.env_truns, 1)
                put(N - ja, N - jb, scalar(_lib.VEC_BLOCK_DIA, ops))
        for ja in range(1, Le + 1):
            oa = _carry(dev, up, ja, Le, d.env_bases, d.env_truns, 1, rank1=True, flag="F")
            put(N - ja, N - Le - 1, term(_lib.VEC_BLOCK_SITE_NDIA, oa, dn))
        n = self.site_profile("num_elec")
        for i in range(N):
            G[i, i] = n[i]
        return G
