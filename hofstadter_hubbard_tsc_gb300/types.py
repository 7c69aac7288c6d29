"""Host-side data model mirroring the reference's derived types (code/pubdata.f90:91-181).

These containers are what a caller hands to the library; they flatten to the
plain int/double arrays of the C ABI (include/hh_dmrg.h) with column-major
sub-blocks, the memory order of the Fortran arrays.
"""
import numpy as np

SU = 2  # spin steps in doubled units (code/pubdata.f90:11)


class SubBlock:
    """Sub_Block: operator block from ket sector (num_up, num_down) with 2S change down_dif."""
    __slots__ = ("num_up", "num_down", "down_dif", "mat")

    def __init__(self, num_up, num_down, down_dif, mat):
        self.num_up, self.num_down, self.down_dif = int(num_up), int(num_down), int(down_dif)
        self.mat = np.asarray(mat, dtype=np.complex128)

    @property
    def row_dim(self):
        return self.mat.shape[0]

    @property
    def sdim(self):
        return self.mat.shape[1]


class TotalBlock:
    """Total_Block: a block operator (code/pubdata.f90:146-149)."""

    def __init__(self, len=0, up_dif=0, down_dif=0, subs=None):
        self.len, self.up_dif, self.down_dif = int(len), int(up_dif), int(down_dif)
        self.subs = list(subs or [])

    @property
    def num(self):
        return len(self.subs)

    def qn_array(self):
        q = np.zeros((max(1, len(self.subs)), 5), dtype=np.int32)
        for i, s in enumerate(self.subs):
            q[i] = (s.num_up, s.num_down, s.down_dif, s.row_dim, s.sdim)
        return q

    def data(self):
        if not self.subs:
            return np.zeros(2, dtype=np.float64)
        parts = [np.asfortranarray(s.mat).ravel(order="F") for s in self.subs]
        return np.ascontiguousarray(np.concatenate(parts)).view(np.float64)

    def set_data(self, flat):
        z = np.asarray(flat, dtype=np.float64).view(np.complex128)
        o = 0
        for s in self.subs:
            n = s.row_dim * s.sdim
            s.mat = z[o:o + n].reshape((s.row_dim, s.sdim), order="F").copy()
            o += n


class SubBasisMap:
    __slots__ = ("spos", "sdim", "bl_num_up", "bl_num_down", "st_num_up", "st_num_down")

    def __init__(self, spos, sdim, bl_num_up, bl_num_down, st_num_up, st_num_down):
        self.spos, self.sdim = int(spos), int(sdim)
        self.bl_num_up, self.bl_num_down = int(bl_num_up), int(bl_num_down)
        self.st_num_up, self.st_num_down = int(st_num_up), int(st_num_down)


class BasisMap:
    __slots__ = ("new_num_up", "new_num_down", "dim", "subs")

    def __init__(self, new_num_up, new_num_down, subs=None):
        self.new_num_up, self.new_num_down = int(new_num_up), int(new_num_down)
        self.subs = list(subs or [])
        self.dim = sum(s.sdim for s in self.subs)


class TotalBasis:
    """Total_Basis: sectors of an enlarged block (code/pubdata.f90:105-108)."""

    def __init__(self, len=0, sectors=None):
        self.len = int(len)
        self.sectors = list(sectors or [])
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
            for s in reversed(self.sectors):
                self._idx[(s.new_num_up, s.new_num_down)] = s
        return self._idx.get((up, down))

    def arrays(self):
        sec = np.zeros((max(1, self.num), 3), dtype=np.int32)
        subs = []
        for i, s in enumerate(self.sectors):
            sec[i] = (s.new_num_up, s.new_num_down, len(s.subs))
            for u in s.subs:
                subs.append((u.spos, u.sdim, u.bl_num_up, u.bl_num_down, u.st_num_up, u.st_num_down))
        sub = np.array(subs if subs else [(0,) * 6], dtype=np.int32)
        return sec, sub


def get_basis(block, site):
    """Enlarged-block sectors of block (x) site, the rules of Get_basis (code/update.f90:11-112).

    ``block`` and ``site`` are Hamiltonian-like TotalBlocks listing the sectors
    (num_up, num_down) and their dimensions.  Sectors are sorted by descending
    2S, then descending N, de-duplicated; sub-blocks are block-major.
    """
    keys = set()
    for b in block.subs:
        for s in site.subs:
            for ss in range(abs(b.num_down - s.num_down), b.num_down + s.num_down + 1, SU):
                keys.add((b.num_up + s.num_up, ss))
    basis = TotalBasis(block.len + site.len)
    for (up, down) in sorted(keys, key=lambda q: (-q[1], -q[0])):
        subs = []
        pos = 0
        for b in block.subs:
            for s in site.subs:
                if b.num_up + s.num_up == up and abs(b.num_down - s.num_down) <= down <= b.num_down + s.num_down:
                    d = b.sdim * s.sdim
                    subs.append(SubBasisMap(pos, d, b.num_up, b.num_down, s.num_up, s.num_down))
                    pos += d
        basis.sectors.append(BasisMap(up, down, subs))
    return basis


class SuperSector:
    __slots__ = ("sys_num_up", "sys_num_down", "env_num_up", "env_num_down", "sys_dim", "env_dim")

    def __init__(self, su, sd, eu, ed, sdim, edim):
        self.sys_num_up, self.sys_num_down = su, sd
        self.env_num_up, self.env_num_down = eu, ed
        self.sys_dim, self.env_dim = sdim, edim


class SuperBasis:
    """Super_Basis: the (sys, env) sector pairs of the target state (code/pubdata.f90:114-123)."""

    def __init__(self, sys_len, env_len, subs):
        self.sys_len, self.env_len = sys_len, env_len
        self.subs = list(subs)

    @property
    def num(self):
        return len(self.subs)

    @property
    def dim(self):
        return sum(s.sys_dim * s.env_dim for s in self.subs)

    def array(self):
        a = np.zeros((max(1, self.num), 6), dtype=np.int32)
        for i, s in enumerate(self.subs):
            a[i] = (s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down, s.sys_dim, s.env_dim)
        return a


def get_super_basis(sys_bs, env_bs, total_up, total_down):
    """Sector pairs with N_s + N_e = total_up coupling to total 2S (code/update.f90:118-171)."""
    subs = []
    for x in sys_bs.sectors:
        for y in env_bs.sectors:
            if y.new_num_up == total_up - x.new_num_up:
                if abs(y.new_num_down - x.new_num_down) <= total_down <= y.new_num_down + x.new_num_down:
                    subs.append(SuperSector(x.new_num_up, x.new_num_down, y.new_num_up, y.new_num_down,
                                            x.dim, y.dim))
    return SuperBasis(sys_bs.len, env_bs.len, subs)


class SubWave:
    __slots__ = ("sys_num_up", "sys_num_down", "env_num_up", "env_num_down", "vec")

    def __init__(self, su, sd, eu, ed, vec):
        self.sys_num_up, self.sys_num_down = su, sd
        self.env_num_up, self.env_num_down = eu, ed
        self.vec = np.asarray(vec, dtype=np.complex128)

    @property
    def sys_dim(self):
        return self.vec.shape[0]

    @property
    def env_dim(self):
        return self.vec.shape[1]


class Wavefunction:
    """Wavefunction: one column-major matrix per super sector (code/pubdata.f90:126-136)."""

    def __init__(self, sys_len, env_len, subs):
        self.sys_len, self.env_len = sys_len, env_len
        self.subs = list(subs)

    @classmethod
    def zeros(cls, sup):
        return cls(sup.sys_len, sup.env_len,
                   [SubWave(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down,
                            np.zeros((s.sys_dim, s.env_dim), dtype=np.complex128)) for s in sup.subs])

    @classmethod
    def random(cls, sup, rng):
        w = cls.zeros(sup)
        for s in w.subs:
            s.vec = rng.random(s.vec.shape) + 1j * rng.random(s.vec.shape)
        n = np.sqrt(sum(float(np.vdot(s.vec, s.vec).real) for s in w.subs))
        for s in w.subs:
            s.vec /= n
        return w

    def layout(self):
        a = np.zeros((max(1, len(self.subs)), 6), dtype=np.int32)
        for i, s in enumerate(self.subs):
            a[i] = (s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down, s.sys_dim, s.env_dim)
        return a

    def flat(self):
        if not self.subs:
            return np.zeros(0, dtype=np.complex128)
        return np.concatenate([s.vec.ravel(order="F") for s in self.subs])

    def set_flat(self, z):
        o = 0
        for s in self.subs:
            n = s.vec.size
            s.vec = np.asarray(z[o:o + n]).reshape(s.vec.shape, order="F").copy()
            o += n
        return self


class TotalModel:
    """Total_Model: block Hamiltonian plus the boundary operators (code/pubdata.f90:175-181).

    ``sub`` maps the operator index of a boundary site to {name: TotalBlock}
    with names elec_up, elec_down (and spin_sd, num_sn for t-J).
    """

    def __init__(self, len, ham, sub=None):
        self.len = len
        self.ham = ham
        self.sub = dict(sub or {})
