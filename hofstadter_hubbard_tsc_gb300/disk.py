"""On-disk formats of the reference (code/space_info.f90:1406-1762), so that a
state written by one program can be read by the other, and a GPU sweep can be
checkpointed and resumed.

Unformatted files are Fortran sequential-access records: every record is a
4-byte little-endian length, the payload, and the length again; integers are
default INTEGER (int32) and operator/wave data complex*16 in column-major
order.  One record carries at most 2^31 - 1 bytes (the files here stay far
below; larger ones raise).  Record layouts:

  wave_to_disk     sys_len | env_len | num | dim | per sector: (empty) |
                   sys_num_up sys_num_down | env_num_up env_num_down |
                   sys_dim env_dim | vec
  block_to_disk    len | num | dim | up_dif | down_dif | per sub: (empty) |
                   num_up num_down down_dif | row_dim sdim | mat
  model_to_disk    len | block(ham) | for each boundary operator index:
                   block(elec_up) block(elec_down) [block(spin_sd) t-J]
                   [block(num_sn) v123]
  truns_to_disk    block(trun)

with dim = sum of the subs' sdim for a block and sum of sys_dim * env_dim for a
wave.  basis_to_disk is formatted text with the reference's edit descriptors
(A4,I6), (A11,I4), (A13,I4), (A10,I4,2X,A12,I4) and an empty line before each
sector.  The periodic-ring operators of model_to_disk (lring) belong to the
triangular-lattice builds only and are not written.
"""
import struct

import numpy as np

from .types import SubBlock, TotalBlock, SubBasisMap, BasisMap, TotalBasis, SubWave, Wavefunction, TotalModel

_MAXREC = 2 ** 31 - 1


class RecordWriter:
    def __init__(self, f):
        self.f = f

    def write(self, payload=b""):
        n = len(payload)
        if n > _MAXREC:
            raise ValueError(f"record of {n} bytes exceeds the 4-byte record marker")
        m = struct.pack("<i", n)
        self.f.write(m)
        self.f.write(payload)
        self.f.write(m)

    def ints(self, *v):
        self.write(struct.pack(f"<{len(v)}i", *[int(x) for x in v]))

    def cmat(self, a):
        self.write(np.asfortranarray(np.asarray(a, dtype=np.complex128)).tobytes(order="F"))


class RecordReader:
    def __init__(self, f):
        self.f = f

    def read(self):
        head = self.f.read(4)
        if len(head) < 4:
            raise EOFError("unexpected end of file")
        (n,) = struct.unpack("<i", head)
        if n < 0:
            raise ValueError("continued (sub)records are not supported")
        payload = self.f.read(n)
        (m,) = struct.unpack("<i", self.f.read(4))
        if m != n or len(payload) != n:
            raise ValueError("corrupt record markers")
        return payload

    def ints(self, count):
        p = self.read()
        if len(p) != 4 * count:
            raise ValueError(f"expected {count} integers, record has {len(p)} bytes")
        return struct.unpack(f"<{count}i", p)

    def cmat(self, rows, cols):
        p = self.read()
        if len(p) != 16 * rows * cols:
            raise ValueError("matrix record of the wrong size")
        return np.frombuffer(p, dtype=np.complex128).reshape((rows, cols), order="F").copy()


# ------------------------------------------------------------------ blocks
def block_to_disk(blk: TotalBlock, w: RecordWriter):
    w.ints(blk.len)
    w.ints(blk.num)
    w.ints(sum(s.sdim for s in blk.subs))
    w.ints(blk.up_dif)
    w.ints(blk.down_dif)
    for s in blk.subs:
        w.write()
        w.ints(s.num_up, s.num_down, s.down_dif)
        w.ints(s.row_dim, s.sdim)
        w.cmat(s.mat)


def block_from_disk(r: RecordReader) -> TotalBlock:
    (length,) = r.ints(1)
    (num,) = r.ints(1)
    r.ints(1)  # dim
    (up_dif,) = r.ints(1)
    (down_dif,) = r.ints(1)
    subs = []
    for _ in range(num):
        r.read()
        nu, nd, dd = r.ints(3)
        rows, cols = r.ints(2)
        subs.append(SubBlock(nu, nd, dd, r.cmat(rows, cols)))
    return TotalBlock(length, up_dif, down_dif, subs)


# ------------------------------------------------------------------- waves
def wave_to_disk(wave: Wavefunction, path):
    with open(path, "wb") as f:
        w = RecordWriter(f)
        w.ints(wave.sys_len)
        w.ints(wave.env_len)
        w.ints(len(wave.subs))
        w.ints(sum(s.sys_dim * s.env_dim for s in wave.subs))
        for s in wave.subs:
            w.write()
            w.ints(s.sys_num_up, s.sys_num_down)
            w.ints(s.env_num_up, s.env_num_down)
            w.ints(s.sys_dim, s.env_dim)
            w.cmat(s.vec)


def wave_from_disk(path) -> Wavefunction:
    with open(path, "rb") as f:
        r = RecordReader(f)
        (sys_len,) = r.ints(1)
        (env_len,) = r.ints(1)
        (num,) = r.ints(1)
        r.ints(1)  # dim
        subs = []
        for _ in range(num):
            r.read()
            su, sd = r.ints(2)
            eu, ed = r.ints(2)
            a, b = r.ints(2)
            subs.append(SubWave(su, sd, eu, ed, r.cmat(a, b)))
    return Wavefunction(sys_len, env_len, subs)


# ----------------------------------------------------------- models, truns
def model_to_disk(model: TotalModel, path, names):
    """names: the operators stored per boundary index, in the reference's order
    (elec_up, elec_down, then spin_sd for t-J and num_sn for v123)."""
    with open(path, "wb") as f:
        w = RecordWriter(f)
        w.ints(model.len)
        block_to_disk(model.ham, w)
        for ii in sorted(model.sub):
            for nm in names:
                block_to_disk(model.sub[ii][nm], w)


def model_from_disk(path, nleg, names) -> TotalModel:
    """nleg: boundary operator indices stored (nleg11(len) of the reference)."""
    with open(path, "rb") as f:
        r = RecordReader(f)
        (length,) = r.ints(1)
        ham = block_from_disk(r)
        sub = {}
        for ii in range(1, nleg + 1):
            sub[ii] = {nm: block_from_disk(r) for nm in names}
    return TotalModel(length, ham, sub)


def truns_to_disk(trun: TotalBlock, path):
    with open(path, "wb") as f:
        block_to_disk(trun, RecordWriter(f))


def truns_from_disk(path) -> TotalBlock:
    with open(path, "rb") as f:
        return block_from_disk(RecordReader(f))


# ------------------------------------------------------------------- bases
def basis_to_disk(basis: TotalBasis, path):
    lines = [f"len={basis.len:6d}", f"num={basis.num:6d}", f"dim={basis.dim:6d}"]
    for i, s in enumerate(basis.sectors, start=1):
        lines.append("")
        lines += [f"idx={i:6d}", f"num={len(s.subs):6d}", f"dim={s.dim:6d}",
                  f"new_num_up={s.new_num_up:4d}", f"new_num_down={s.new_num_down:4d}"]
        for u in s.subs:
            lines += [f"pos={u.spos:6d}", f"dim={u.sdim:6d}",
                      f"bl_num_up={u.bl_num_up:4d}  bl_num_down={u.bl_num_down:4d}",
                      f"st_num_up={u.st_num_up:4d}  st_num_down={u.st_num_down:4d}"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def basis_from_disk(path) -> TotalBasis:
    with open(path) as f:
        lines = f.read().split("\n")
    pos = 0

    def nxt():
        nonlocal pos
        line = lines[pos]
        pos += 1
        return line

    def fixed(width_label):
        line = nxt()
        return int(line[width_label:])

    length = fixed(4)
    num = fixed(4)
    fixed(4)  # dim
    sectors = []
    for _ in range(num):
        nxt()  # empty record line
        fixed(4)  # idx
        nsub = fixed(4)
        fixed(4)  # dim
        up = fixed(11)
        down = fixed(13)
        subs = []
        for _ in range(nsub):
            spos = fixed(4)
            sdim = fixed(4)
            a = nxt()
            b = nxt()
            subs.append(SubBasisMap(spos, sdim, int(a[10:14]), int(a[28:32]), int(b[10:14]), int(b[28:32])))
        sectors.append(BasisMap(up, down, subs))
    return TotalBasis(length, sectors)


def restart_to_disk(path, restart1, sys_len_start, restart2):
    """restart.dat (code/warm_up.f90:1580-1584, read at code/quantum.f90:43-46):
    two list-directed records, 'restart1 sys_len_start' and 'restart2'. The
    left-to-right sweep writes (1, label + 1) and 1 after each step so that a
    rerun resumes there. Integers are written in gfortran's layout (a leading
    blank, 12 columns each); the reader takes any whitespace."""
    with open(path, "w") as f:
        f.write(f" {int(restart1):11d} {int(sys_len_start):11d}\n {int(restart2):11d}\n")


def restart_from_disk(path):
    """(restart1, sys_len_start, restart2) of a restart.dat written by the
    reference or by restart_to_disk (list-directed: free format)."""
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n") if ln.strip()]
    first = lines[0].split()
    return int(first[0]), int(first[1]), int(lines[1].split()[0])
