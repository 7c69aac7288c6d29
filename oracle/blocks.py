"""Data model and block utilities of the reference, restated in numpy.

Types follow code/pubdata.f90:91-181:
  * ``Block``  = ``Total_Block``: list of ``Sub`` keyed by the ket sector
    (num_up=N, num_down=2S) and down_dif (change of 2S); ``mat`` is
    (row_dim x sdim) = (bra dim x ket dim).  ``up_dif`` is the change of N.
  * ``Basis``  = ``Total_Basis``: enlarged-block sectors, each a list of
    (block sector, site sector) sub-blocks with offsets ``spos``.
  * ``Super``  = ``Super_Basis`` and ``Wave`` = ``Wavefunction``.
Reference lookups are linear "first match" searches; with the unique keys the
reference produces, a dictionary of the first matching index is equivalent.
"""
import numpy as np

from .su2 import w3j, w6j, parity_sign

SU = 2  # code/pubdata.f90:11 (su=2: spin steps in doubled units)


class Sub:
    __slots__ = ("num_up", "num_down", "down_dif", "row_dim", "sdim", "mat")

    def __init__(self, num_up, num_down, down_dif, row_dim, sdim, mat=None):
        self.num_up = num_up
        self.num_down = num_down
        self.down_dif = down_dif
        self.row_dim = row_dim
        self.sdim = sdim
        self.mat = (np.zeros((row_dim, sdim), dtype=np.complex128) if mat is None
                    else mat)


class Block:
    """Total_Block (code/pubdata.f90:146-149)."""

    def __init__(self, len=0, up_dif=0, down_dif=0, subs=None):
        self.len = len
        self.up_dif = up_dif
        self.down_dif = down_dif
        self.subs = [] if subs is None else subs
        self._idx2 = None
        self._idx3 = None
        self._nbuilt = -1

    @property
    def num(self):
        return len(self.subs)

    @property
    def dim(self):
        return sum(s.sdim for s in self.subs)

    def _build(self):
        self._idx2, self._idx3 = {}, {}
        for i, s in enumerate(self.subs):
            self._idx2.setdefault((s.num_up, s.num_down), i)
            self._idx3.setdefault((s.num_up, s.num_down, s.down_dif), i)
        self._nbuilt = len(self.subs)

    def find(self, num_up, num_down, down_dif=None):
        """Index of the first sub with this ket sector (and down_dif), or None."""
        if self._idx2 is None or self._nbuilt != len(self.subs):
            self._build()
        if down_dif is None:
            return self._idx2.get((num_up, num_down))
        return self._idx3.get((num_up, num_down, down_dif))

    def invalidate(self):
        self._idx2 = None
        self._idx3 = None
        self._nbuilt = -1

    def copy(self):
        b = Block(self.len, self.up_dif, self.down_dif,
                  [Sub(s.num_up, s.num_down, s.down_dif, s.row_dim, s.sdim, s.mat.copy())
                   for s in self.subs])
        return b

    def zeros_like(self):
        """block_pass_info (code/space_info.f90:131-158)."""
        return Block(self.len, self.up_dif, self.down_dif,
                     [Sub(s.num_up, s.num_down, s.down_dif, s.row_dim, s.sdim)
                      for s in self.subs])


def block_transfer_trans(inmat, realcode=False):
    """Conjugate-transpose view of a block (code/space_info.f90:32-63).

    The output is keyed by the input's bra sector; up_dif flips sign while the
    total rank ``down_dif`` is kept; every sub-matrix becomes mat^H.
    """
    out = Block(inmat.len, -inmat.up_dif, inmat.down_dif)
    for s in inmat.subs:
        m = s.mat.T.copy()
        if not realcode:
            m = np.conj(m)
        out.subs.append(Sub(s.num_up + inmat.up_dif, s.num_down + s.down_dif,
                            -s.down_dif, s.sdim, s.row_dim, m))
    return out


def block_add_block_two(block1, coef1, new_block):
    """new_block += coef1*block1 sub by sub (code/space_info.f90:176-214).

    The reference searches ``block1`` from the position after the last match;
    both blocks share one sector order, so the scan is a forward merge.
    """
    x1 = 0
    for ns in new_block.subs:
        idx = None
        for x in range(x1, block1.num):
            s = block1.subs[x]
            if (s.num_up == ns.num_up and s.num_down == ns.num_down
                    and s.down_dif == ns.down_dif):
                idx = x
                x1 = x + 1
                break
        if idx is not None:
            ns.mat += coef1 * block1.subs[idx].mat


# ---------------------------------------------------------------------------
# Bases
# ---------------------------------------------------------------------------
def _odd(n):
    return -1.0 if n % 2 else 1.0


def block_mul_block_ndia(op1, op2, down_dif, basis, coef=1.0):
    """(op1 op2)^K, K = down_dif / 2: the product of two operators of one
    block coupled to rank K (block_mul_block_ndia with flags 'N', 'N',
    code/space_info.f90:373-631).  For each sector (N, 2S) of the basis and
    each 2S' = |2S - down_dif| .. 2S + down_dif whose sector (N + up_dif,
    2S') exists, the reduced matrix of the product is the regular matrix
    element at the stretched projections M' = S', M = S, built by the
    Wigner-Eckart theorem (<S' M'|T^k_q|S M> = (-1)^(S'-M') (S' k S; -M' q M)
    <S'||T^k||S>) from the two factors summed over the intermediate
    projection with the Clebsch-Gordan coefficient of the coupling
    (-1)^(-k1+k2+q) sqrt(2K+1) (k1 k2 K; q1 q2 -q), divided by the 3j of the
    product at the same projections.  Intermediate spins run over
    |2S - k2| .. 2S + k2; a product term needs both factor sub-blocks."""
    up_dif = op1.up_dif + op2.up_dif
    k1, k2, K = op1.down_dif, op2.down_dif, down_dif
    subs = []
    for sec in basis.sectors:
        nu, nd = sec.new_num_up, sec.new_num_down
        for nnd in range(abs(nd - K), nd + K + 1, SU):
            tgt = basis.find(nu + up_dif, nnd)
            if tgt is None:
                continue
            sub = Sub(nu, nd, nnd - nd, tgt.dim, sec.dim)
            subs.append(sub)
            q = nnd - nd
            norm = w3j(nnd, K, nd, -nnd, q, nd)
            for md in range(abs(nd - k2), nd + k2 + 1, SU):
                ib = op2.find(nu, nd, md - nd)
                ia = op1.find(nu + op2.up_dif, md, nnd - md)
                if ia is None or ib is None:
                    continue
                c = 0.0
                for mm in range(-md, md + 1, SU):
                    q1, q2 = nnd - mm, mm - nd
                    ea = w3j(nnd, k1, md, -nnd, q1, mm)
                    eb = w3j(md, k2, nd, -mm, q2, nd) * _odd((md - mm) // 2)
                    cgk = w3j(k1, k2, K, q1, q2, -q) * _odd((-k1 + k2 + q) // 2) * np.sqrt(K + 1.0)
                    c += ea * eb * cgk
                if c != 0.0:
                    sub.mat += (coef * c / norm) * (op1.subs[ia].mat @ op2.subs[ib].mat)
    return Block(basis.len, up_dif, K, subs)


class BSub:
    __slots__ = ("spos", "sdim", "bl_num_up", "bl_num_down", "st_num_up", "st_num_down")

    def __init__(self, spos, sdim, bl_num_up, bl_num_down, st_num_up, st_num_down):
        self.spos = spos
        self.sdim = sdim
        self.bl_num_up = bl_num_up
        self.bl_num_down = bl_num_down
        self.st_num_up = st_num_up
        self.st_num_down = st_num_down


class BSector:
    __slots__ = ("new_num_up", "new_num_down", "dim", "subs", "_bl", "_full")

    def __init__(self, new_num_up, new_num_down):
        self.new_num_up = new_num_up
        self.new_num_down = new_num_down
        self.dim = 0
        self.subs = []
        self._bl = None
        self._full = None

    @property
    def num(self):
        return len(self.subs)

    def _build(self):
        self._bl, self._full = {}, {}
        for i, s in enumerate(self.subs):
            self._bl.setdefault((s.bl_num_up, s.bl_num_down), i)
            self._full.setdefault((s.bl_num_up, s.bl_num_down, s.st_num_up, s.st_num_down), i)

    def find_full(self, bu, bd, su, sd):
        if self._full is None:
            self._build()
        i = self._full.get((bu, bd, su, sd))
        return None if i is None else self.subs[i]

    def find_bl(self, bu, bd):
        if self._bl is None:
            self._build()
        i = self._bl.get((bu, bd))
        return None if i is None else self.subs[i]


class Basis:
    """Total_Basis (code/pubdata.f90:105-108)."""

    def __init__(self, len=0, sectors=None):
        self.len = len
        self.sectors = [] if sectors is None else sectors
        self._idx = None

    @property
    def num(self):
        return len(self.sectors)

    @property
    def dim(self):
        return sum(s.dim for s in self.sectors)

    def find(self, up, down):
        if self._idx is None:
            self._idx = {}
            for i, s in enumerate(self.sectors):
                self._idx.setdefault((s.new_num_up, s.new_num_down), i)
        i = self._idx.get((up, down))
        return None if i is None else self.sectors[i]

    def find_index(self, up, down):
        self.find(up, down)
        return self._idx.get((up, down))


def get_basis(block, site):
    """Get_basis (code/update.f90:11-112): enlarged-block sectors.

    ``block`` and ``site`` are the Hamiltonian-like blocks whose subs list the
    sectors (num_up, num_down, sdim).  Sectors are all (N_b+N_s, 2S) with
    |2S_b-2S_s| <= 2S <= 2S_b+2S_s, sorted by descending 2S then descending N
    (QuickSort_Integer, code/update.f90:240-273) and de-duplicated
    (Get_Unique_QN, code/update.f90:176-204).  Sub-blocks are ordered block-major
    then site, with offsets accumulated in that order.
    """
    pre = []
    for b in block.subs:
        for s in site.subs:
            lo = abs(b.num_down - s.num_down)
            hi = b.num_down + s.num_down
            for ss in range(lo, hi + 1, SU):
                pre.append((b.num_up + s.num_up, ss))
    uniq = sorted(set(pre), key=lambda q: (-q[1], -q[0]))
    basis = Basis(block.len + site.len)
    for (up, down) in uniq:
        sec = BSector(up, down)
        for b in block.subs:
            for s in site.subs:
                if b.num_up + s.num_up == up:
                    lo = abs(b.num_down - s.num_down)
                    hi = b.num_down + s.num_down
                    if lo <= down <= hi:
                        sdim = b.sdim * s.sdim
                        sec.subs.append(BSub(sec.dim, sdim, b.num_up, b.num_down,
                                             s.num_up, s.num_down))
                        sec.dim += sdim
        basis.sectors.append(sec)
    return basis


class SSector:
    __slots__ = ("sys_num_up", "sys_num_down", "env_num_up", "env_num_down",
                 "sys_dim", "env_dim")

    def __init__(self, su, sd, eu, ed, sdim, edim):
        self.sys_num_up = su
        self.sys_num_down = sd
        self.env_num_up = eu
        self.env_num_down = ed
        self.sys_dim = sdim
        self.env_dim = edim


class Super:
    def __init__(self, sys_len, env_len, subs):
        self.sys_len = sys_len
        self.env_len = env_len
        self.subs = subs

    @property
    def num(self):
        return len(self.subs)

    @property
    def dim(self):
        return sum(s.sys_dim * s.env_dim for s in self.subs)


def get_super_basis(sys_bs, env_bs, total_up, total_down):
    """Get_super_basis (code/update.f90:118-171): sys-major pairs of sectors."""
    subs = []
    for x in sys_bs.sectors:
        for y in env_bs.sectors:
            if y.new_num_up == total_up - x.new_num_up:
                lo = abs(y.new_num_down - x.new_num_down)
                hi = y.new_num_down + x.new_num_down
                if lo <= total_down <= hi:
                    subs.append(SSector(x.new_num_up, x.new_num_down, y.new_num_up,
                                        y.new_num_down, x.dim, y.dim))
    return Super(sys_bs.len, env_bs.len, subs)


class WSub:
    __slots__ = ("sys_num_up", "sys_num_down", "env_num_up", "env_num_down",
                 "sys_dim", "env_dim", "vec")

    def __init__(self, ss, vec=None):
        self.sys_num_up = ss.sys_num_up
        self.sys_num_down = ss.sys_num_down
        self.env_num_up = ss.env_num_up
        self.env_num_down = ss.env_num_down
        self.sys_dim = ss.sys_dim
        self.env_dim = ss.env_dim
        self.vec = (np.zeros((ss.sys_dim, ss.env_dim), dtype=np.complex128)
                    if vec is None else vec)


class Wave:
    """Wavefunction (code/pubdata.f90:126-136)."""

    def __init__(self, sys_len, env_len, subs):
        self.sys_len = sys_len
        self.env_len = env_len
        self.subs = subs
        self._idx = None

    @property
    def num(self):
        return len(self.subs)

    def find(self, su, sd, eu, ed):
        if self._idx is None:
            self._idx = {}
            for i, w in enumerate(self.subs):
                self._idx.setdefault((w.sys_num_up, w.sys_num_down, w.env_num_up,
                                      w.env_num_down), i)
        return self._idx.get((su, sd, eu, ed))

    def copy(self):
        return Wave(self.sys_len, self.env_len,
                    [WSub(w, w.vec.copy()) for w in self.subs])

    def zeros_like(self):
        return Wave(self.sys_len, self.env_len, [WSub(w) for w in self.subs])

    def flat(self):
        return np.concatenate([w.vec.ravel(order="F") for w in self.subs])

    def set_flat(self, v):
        o = 0
        for w in self.subs:
            n = w.sys_dim * w.env_dim
            w.vec = np.array(v[o:o + n].reshape((w.sys_dim, w.env_dim), order="F"))
            o += n


def allocate_wave(sup):
    """allocate_wave (code/space_info.f90:912-939)."""
    return Wave(sup.sys_len, sup.env_len, [WSub(s) for s in sup.subs])


# ---------------------------------------------------------------------------
# Wave vector operations (code/space_info.f90:1018-1214)
# ---------------------------------------------------------------------------
def wave_product(left, right):
    """Real part of <left|right> (code/space_info.f90:1018-1035)."""
    s = 0.0
    for a, b in zip(left.subs, right.subs):
        s += float(np.vdot(a.vec, b.vec).real)
    return s


def wave_norm(w):
    """code/space_info.f90:1038-1057."""
    s = 0.0
    for a in w.subs:
        s += float(np.vdot(a.vec, a.vec).real)
    return float(np.sqrt(s))


def wave_normalize(w):
    """code/space_info.f90:1060-1075."""
    n = wave_norm(w)
    for a in w.subs:
        a.vec = a.vec / n


def wave_initialize(w, rng, realcode=False):
    """Random start vector (code/space_info.f90:1079-1105), seeded here."""
    for a in w.subs:
        re = rng.random((a.sys_dim, a.env_dim))
        im = rng.random((a.sys_dim, a.env_dim))
        a.vec = re.astype(np.complex128) if realcode else (re + 1j * im)
    wave_normalize(w)


def gram_schmidt_process(prev, wnew):
    """Gram_Schmidt_process (code/space_info.f90:1176-1214).

    Projections use the real inner product (wave_product keeps Re<u,v>).
    """
    uv = [wave_product(p, wnew) for p in prev]
    uu = [wave_product(p, p) for p in prev]
    acc = [np.zeros_like(a.vec) for a in wnew.subs]
    for j, p in enumerate(prev):
        f = uv[j] / uu[j]
        for i, a in enumerate(p.subs):
            acc[i] = acc[i] + f * a.vec
    for i, a in enumerate(wnew.subs):
        a.vec = a.vec - acc[i]
    wave_normalize(wnew)


# ---------------------------------------------------------------------------
# Block enlargement helpers (code/update.f90:419-1381)
# ---------------------------------------------------------------------------
def update_block_dia(block, basis):
    """Embed a diagonal block operator in the enlarged basis (code/update.f90:419-472)."""
    nb = Block(basis.len, 0, 0)
    for sec in basis.sectors:
        nb.subs.append(Sub(sec.new_num_up, sec.new_num_down, 0, sec.dim, sec.dim))
    for k, sec in enumerate(basis.sectors):
        m = nb.subs[k].mat
        for x in sec.subs:
            i = block.find(x.bl_num_up, x.bl_num_down)
            if i is not None:
                c = np.sqrt((1.0 + sec.new_num_down) / (1.0 + block.subs[i].num_down))
                m[x.spos:x.spos + x.sdim, x.spos:x.spos + x.sdim] += \
                    block.subs[i].mat[:x.sdim, :x.sdim] * c
    return nb


def update_site_dia(site, basis):
    """Embed a diagonal site operator in the enlarged basis (code/update.f90:478-539)."""
    nb = Block(basis.len, 0, 0)
    for sec in basis.sectors:
        nb.subs.append(Sub(sec.new_num_up, sec.new_num_down, 0, sec.dim, sec.dim))
    for k, sec in enumerate(basis.sectors):
        m = nb.subs[k].mat
        for x in sec.subs:
            i = site.find(x.st_num_up, x.st_num_down)
            if i is not None:
                c = np.sqrt((1.0 + sec.new_num_down) / (1.0 + site.subs[i].num_down))
                m[x.spos:x.spos + x.sdim, x.spos:x.spos + x.sdim] += \
                    np.eye(x.sdim) * site.subs[i].mat[0, 0] * c
    return nb


def _ndia_layout(op, basis):
    """Sub layout shared by update_*_ndia_* (code/update.f90:572-633).

    For each rhs sector and each down_dif in -k..k, a sub exists when the lhs
    sector (rhs + (up_dif, down_dif)) is in the basis.
    """
    nb = Block(basis.len, op.up_dif, op.down_dif)
    k = op.down_dif
    for sec in basis.sectors:
        for dd in range(-k, k + 1, SU):
            lhs = basis.find(sec.new_num_up + op.up_dif, sec.new_num_down + dd)
            if lhs is not None:
                nb.subs.append(Sub(sec.new_num_up, sec.new_num_down, dd, lhs.dim, sec.dim))
    return nb


def _find_lhs_sub(sec, bl_up, bl_down, st_down=None, st_up=None, match_st=True):
    for y in sec.subs:
        if y.bl_num_up == bl_up and y.bl_num_down == bl_down:
            if st_down is None or y.st_num_down == st_down:
                return y
    return None


def update_block_ndia(block, basis, flag, side):
    """update_block_ndia_sys/env (code/update.f90:548-742, 750-958).

    Embeds a rank-k block operator; the env version multiplies by the fermion
    sign of the site (the site precedes the block in the env ordering).
    """
    nb = _ndia_layout(block, basis)
    k = block.down_dif
    for i, s in enumerate(nb.subs):
        rhs = basis.find(s.num_up, s.num_down)
        lhs = basis.find(s.num_up + block.up_dif, s.num_down + s.down_dif)
        if rhs is None or lhs is None:
            continue
        for x in rhs.subs:
            for sdd in range(-k, k + 1, SU):
                bid = block.find(x.bl_num_up, x.bl_num_down, sdd)
                if bid is None:
                    continue
                lu = x.bl_num_up + block.up_dif
                ld = x.bl_num_down + sdd
                y = None
                for yy in lhs.subs:
                    if yy.bl_num_up == lu and yy.bl_num_down == ld and yy.st_num_down == x.st_num_down:
                        y = yy
                        break
                if y is None:
                    continue
                sign = 1.0
                if side == "env" and flag == "F" and x.st_num_up % 2 == 1:
                    sign = -1.0
                j1, j2, j3, j4, j5, j6 = lhs.new_num_down, k, rhs.new_num_down, x.bl_num_down, x.st_num_down, ld
                c = w6j(j1, j2, j3, j4, j5, j6)
                c *= np.sqrt((1.0 + j1) * (1.0 + j3)) * parity_sign(j6 + j5 + j3 + j2)
                if c != 0.0:
                    s.mat[y.spos:y.spos + y.sdim, x.spos:x.spos + x.sdim] += \
                        sign * c * block.subs[bid].mat[:y.sdim, :x.sdim]
    nb.invalidate()
    return nb


def update_site_ndia(site, basis, flag, side):
    """update_site_ndia_sys/env (code/update.f90:969-1182, 1191-1381).

    The sys version carries the fermion sign of the block electron number (the
    site follows the block); the env version carries none.
    """
    nb = _ndia_layout(site, basis)
    k = site.down_dif
    for i, s in enumerate(nb.subs):
        rhs = basis.find(s.num_up, s.num_down)
        lhs = basis.find(s.num_up + site.up_dif, s.num_down + s.down_dif)
        if rhs is None or lhs is None:
            continue
        for x in rhs.subs:
            for sdd in range(-k, k + 1, SU):
                sid = site.find(x.st_num_up, x.st_num_down, sdd)
                if sid is None:
                    continue
                lu = x.st_num_up + site.up_dif
                ld = x.st_num_down + sdd
                y = None
                for yy in lhs.subs:
                    if yy.st_num_up == lu and yy.st_num_down == ld and yy.bl_num_down == x.bl_num_down:
                        y = yy
                        break
                if y is None:
                    continue
                sign = 1.0
                if side == "sys" and flag == "F" and x.bl_num_up % 2 == 1:
                    sign = -1.0
                j1, j2, j3, j4, j5, j6 = lhs.new_num_down, k, rhs.new_num_down, x.st_num_down, x.bl_num_down, ld
                c = w6j(j1, j2, j3, j4, j5, j6)
                c *= parity_sign(j5 + j4 + j1 + j2) * np.sqrt((1.0 + j1) * (1.0 + j3))
                if c != 0.0:
                    s.mat[y.spos:y.spos + x.sdim, x.spos:x.spos + x.sdim] += \
                        sign * c * np.eye(x.sdim) * site.subs[sid].mat[0, 0]
    nb.invalidate()
    return nb


# ---------------------------------------------------------------------------
# Truncation of operators (code/update.f90:1387-1605)
# ---------------------------------------------------------------------------
def update_trun_dia(ori, trun):
    """eff = T^H O T per kept sector (code/update.f90:1387-1449)."""
    eff = Block(ori.len, ori.up_dif, ori.down_dif)
    for t in trun.subs:
        e = Sub(t.num_up, t.num_down, 0, t.sdim, t.sdim)
        x = ori.find(t.num_up, t.num_down)
        if x is not None:
            mid = ori.subs[x].mat @ t.mat
            e.mat = np.conj(t.mat).T @ mid
        eff.subs.append(e)
    return eff


def update_trun_ndia(ori, trun):
    """eff = T_lhs^H O T_rhs per sector pair (code/update.f90:1457-1605)."""
    eff = Block(ori.len, ori.up_dif, ori.down_dif)
    k = ori.down_dif
    tidx = {(t.num_up, t.num_down): i for i, t in reversed(list(enumerate(trun.subs)))}
    for t in trun.subs:
        for dd in range(-k, k + 1, SU):
            li = tidx.get((t.num_up + ori.up_dif, t.num_down + dd))
            if li is not None:
                eff.subs.append(Sub(t.num_up, t.num_down, dd, trun.subs[li].sdim, t.sdim))
    for e in eff.subs:
        ri = tidx.get((e.num_up, e.num_down))
        li = tidx.get((e.num_up + ori.up_dif, e.num_down + e.down_dif))
        oi = ori.find(e.num_up, e.num_down, e.down_dif)
        if ri is not None and li is not None and oi is not None:
            mid = ori.subs[oi].mat @ trun.subs[ri].mat
            e.mat = np.conj(trun.subs[li].mat).T @ mid
    return eff
