"""The reference's on-disk formats (code/space_info.f90:1406-1762): record
layout, fixed-format basis text, and round trips."""
import struct

import numpy as np

from hofstadter_hubbard_tsc_gb300 import disk
from hofstadter_hubbard_tsc_gb300.types import (SubBlock, TotalBlock, SubWave, Wavefunction, TotalModel,
                                               get_basis)


def _rand_block(rng, shapes, length=3, up_dif=1, down_dif=1):
    subs = [SubBlock(nu, nd, dd, rng.normal(size=(r, c)) + 1j * rng.normal(size=(r, c)))
            for (nu, nd, dd, r, c) in shapes]
    return TotalBlock(length, up_dif, down_dif, subs)


def _records(path):
    out = []
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        (n,) = struct.unpack("<i", data[p:p + 4])
        payload = data[p + 4:p + 4 + n]
        (m,) = struct.unpack("<i", data[p + 4 + n:p + 8 + n])
        assert m == n
        out.append(payload)
        p += 8 + n
    return out


def test_wave_records(tmp_path):
    rng = np.random.default_rng(0)
    w = Wavefunction(5, 7, [SubWave(4, 0, 6, 0, rng.normal(size=(3, 2)) + 1j * rng.normal(size=(3, 2))),
                            SubWave(3, 1, 7, 1, rng.normal(size=(1, 4)) + 0j)])
    p = tmp_path / "wave.dat"
    disk.wave_to_disk(w, p)
    rec = _records(p)
    # header: sys_len, env_len, num, dim (= 6 + 4), then 5 records per sector
    assert [struct.unpack("<i", r)[0] for r in rec[:4]] == [5, 7, 2, 10]
    assert len(rec) == 4 + 5 * 2
    assert rec[4] == b"" and struct.unpack("<2i", rec[5]) == (4, 0) and struct.unpack("<2i", rec[7]) == (3, 2)
    np.testing.assert_array_equal(np.frombuffer(rec[8], np.complex128), w.subs[0].vec.ravel(order="F"))
    r = disk.wave_from_disk(p)
    assert (r.sys_len, r.env_len) == (5, 7)
    for a, b in zip(r.subs, w.subs):
        assert (a.sys_num_up, a.sys_num_down, a.env_num_up, a.env_num_down) == \
               (b.sys_num_up, b.sys_num_down, b.env_num_up, b.env_num_down)
        np.testing.assert_array_equal(a.vec, b.vec)


def test_block_model_truns_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    ham = _rand_block(rng, [(2, 0, 0, 3, 3), (1, 1, 0, 2, 2)], up_dif=0, down_dif=0)
    ops = {ii: {"elec_up": _rand_block(rng, [(1, 1, 1, 3, 2)]),
                "elec_down": _rand_block(rng, [(2, 0, -1, 2, 3), (1, 1, 1, 1, 2)])} for ii in (1, 2)}
    m = TotalModel(3, ham, ops)
    p = tmp_path / "model.dat"
    disk.model_to_disk(m, p, ["elec_up", "elec_down"])
    rec = _records(p)
    assert struct.unpack("<i", rec[0])[0] == 3
    # block header: len, num, dim = sum of sdim, up_dif, down_dif
    assert [struct.unpack("<i", x)[0] for x in rec[1:6]] == [3, 2, 5, 0, 0]
    r = disk.model_from_disk(p, 2, ["elec_up", "elec_down"])
    assert r.len == 3 and sorted(r.sub) == [1, 2]
    for ii in (1, 2):
        for nm in ("elec_up", "elec_down"):
            a, b = r.sub[ii][nm], ops[ii][nm]
            assert (a.len, a.up_dif, a.down_dif) == (b.len, b.up_dif, b.down_dif)
            for x, y in zip(a.subs, b.subs):
                assert (x.num_up, x.num_down, x.down_dif) == (y.num_up, y.num_down, y.down_dif)
                np.testing.assert_array_equal(x.mat, y.mat)
    t = _rand_block(rng, [(2, 0, 0, 5, 3)], up_dif=0, down_dif=0)
    disk.truns_to_disk(t, tmp_path / "trun.dat")
    np.testing.assert_array_equal(disk.truns_from_disk(tmp_path / "trun.dat").subs[0].mat, t.subs[0].mat)


def test_basis_fixed_format(tmp_path):
    blk = TotalBlock(2, 0, 0, [SubBlock(0, 0, 0, np.zeros((1, 1))), SubBlock(1, 1, 0, np.zeros((2, 2))),
                              SubBlock(2, 0, 0, np.zeros((1, 1)))])
    site = TotalBlock(1, 0, 0, [SubBlock(0, 0, 0, np.zeros((1, 1))), SubBlock(1, 1, 0, np.zeros((1, 1))),
                               SubBlock(2, 0, 0, np.zeros((1, 1)))])
    b = get_basis(blk, site)
    p = tmp_path / "basis.dat"
    disk.basis_to_disk(b, p)
    lines = open(p).read().split("\n")
    # (A4,I6), an empty line before each sector, (A11,I4), (A13,I4), (A10,I4,2X,A12,I4)
    assert lines[0] == "len=     3" and lines[3] == "" and lines[4] == "idx=     1"
    assert lines[7].startswith("new_num_up=") and len(lines[7]) == 15
    assert lines[8].startswith("new_num_down=") and len(lines[8]) == 17
    assert lines[11][:10] == "bl_num_up=" and lines[11][14:16] == "  " and lines[11][16:28] == "bl_num_down="
    r = disk.basis_from_disk(p)
    assert r.len == b.len and r.num == b.num and r.dim == b.dim
    for x, y in zip(r.sectors, b.sectors):
        assert (x.new_num_up, x.new_num_down, x.dim) == (y.new_num_up, y.new_num_down, y.dim)
        assert [(u.spos, u.sdim, u.bl_num_up, u.bl_num_down, u.st_num_up, u.st_num_down) for u in x.subs] == \
               [(u.spos, u.sdim, u.bl_num_up, u.bl_num_down, u.st_num_up, u.st_num_down) for u in y.subs]


def test_restart_flags_round_trip(tmp_path):
    """restart.dat: the reference's own file (restart1 = 0, sys_len_start = 0,
    restart2 = 0, free-format spacing) and what a left-to-right step writes."""
    from hofstadter_hubbard_tsc_gb300.disk import restart_from_disk, restart_to_disk
    ref = tmp_path / "restart_ref.dat"
    ref.write_text("         0 0  \n          0\n")
    assert restart_from_disk(ref) == (0, 0, 0)
    p = tmp_path / "restart.dat"
    restart_to_disk(p, 1, 17, 1)
    assert p.read_text() == "           1          17\n           1\n"
    assert restart_from_disk(p) == (1, 17, 1)
