"""Block enlargement ``Get_Hamiltonian_Sys/Env`` (code/get_ham.f90:4-659).

A block of length l plus one site becomes the enlarged block; its Hamiltonian
gets the bonds between the new site and the block
(``Get_hamiltonian_ndia``, code/get_ham.f90:954-1152, and
``Get_hamiltonian_dia``, code/get_ham.f90:852-941) and the on-site U; the
boundary operators are embedded (code/update.f90) and then everything is
truncated with T (``update_trun_*``).  The model is updated in place, as the
reference updates ``pre``.
"""
import numpy as np

from .blocks import (SU, block_transfer_trans, block_add_block_two, update_block_dia,
                     update_site_dia, update_block_ndia, update_site_ndia,
                     update_trun_dia, update_trun_ndia)
from .su2 import w6j, parity_sign


class Model:
    """Total_Model (code/pubdata.f90:175-181): Hamiltonian plus boundary operators."""

    def __init__(self, length, ham):
        self.len = length
        self.ham = ham
        self.sub = {}      # op index (inb1) -> {name: Block}
        self.snc = [None, None]
        self.sub_s = {}


def get_hamiltonian_ndia(block, site, basis, coef, ham, flag_sign, flags):
    """Add coef * [O_block . O_site]^0 (+ h.c.) to ham (code/get_ham.f90:954-1152)."""
    up_dif, k = block.up_dif, block.down_dif
    for hs in ham.subs:
        rhs = basis.find(hs.num_up, hs.num_down)
        lhs = basis.find(hs.num_up, hs.num_down + hs.down_dif)
        if rhs is None or lhs is None:
            continue
        for x in rhs.subs:
            for sdd in range(-k, k + 1, SU):
                bid = block.find(x.bl_num_up, x.bl_num_down, sdd)
                if bid is None:
                    continue
                lsu, lsd = x.bl_num_up + up_dif, x.bl_num_down + sdd
                for nsd in range(abs(x.st_num_down - site.down_dif), x.st_num_down + site.down_dif + 1, SU):
                    st_dd = x.st_num_down - nsd
                    nsu = x.st_num_up - site.up_dif
                    sid = site.find(nsu, nsd, st_dd)
                    y = None
                    for yy in lhs.subs:
                        if yy.bl_num_up == lsu and yy.bl_num_down == lsd and yy.st_num_down == nsd:
                            y = yy
                            break
                    if y is None or sid is None:
                        continue
                    j1, j2, j3, j4, j5, j6 = lsd, x.bl_num_down, k, x.st_num_down, nsd, rhs.new_num_down
                    c = w6j(j1, j2, j3, j4, j5, j6)
                    c *= np.sqrt((1.0 + j6) / (1.0 + j3)) * parity_sign(j2 + j5 + j3 + j6) * site.subs[sid].mat[0, 0]
                    if flags == "S":
                        sign = -1.0 if (flag_sign == "F" and x.bl_num_up % 2 == 1) else 1.0
                    else:
                        sign = -1.0 if (flag_sign == "F" and x.st_num_up % 2 == 0) else 1.0
                    if c != 0.0:
                        c1 = c * coef * sign
                        bm = block.subs[bid].mat[:y.sdim, :x.sdim]
                        hs.mat[y.spos:y.spos + y.sdim, x.spos:x.spos + x.sdim] += c1 * bm
                        if site.up_dif != 0:
                            hs.mat[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim] += np.conj(c1) * np.conj(bm).T


def get_hamiltonian_dia(op1, op2, coef, ham):
    """ham += coef/sqrt(2S+1) * O1 O2 per sector (code/get_ham.f90:852-941)."""
    for hs in ham.subs:
        a = op1.find(hs.num_up, hs.num_down)
        b = op2.find(hs.num_up, hs.num_down)
        if a is not None and b is not None:
            c1 = coef / np.sqrt(1.0 + hs.num_down)
            hs.mat += c1 * (op1.subs[a].mat @ op2.subs[b].mat)


def _ij_list(geo):
    """Operator classes handled per model (code/get_ham.f90:36-52)."""
    if geo.tjmodel:
        return [1, 3] + ([5] if geo.v123 else [])
    return [1, 6] + ([5] if geo.v123 else [])


def get_hamiltonian(pre, basis, trun, geo, st, side, mshift=0):
    """Get_Hamiltonian_Sys (side='sys') / Get_Hamiltonian_Env (side='env')."""
    lat = geo.lat
    next_ham = update_block_dia(pre.ham, basis)
    next_sub = {}
    L = pre.len
    if side == "sys":
        jdm = L + 1
        jlat = jdm
    else:
        jdm = L + 1 + mshift
        jlat = geo.nposi_lat[jdm]

    def block_neighbours():
        out = []
        for kdir, I in geo.bonds(jlat):
            II = I if side == "sys" else geo.nposi_dm.get(I, 0) - mshift
            if 0 < II <= L:
                i1 = lat.inb1.get((II, L), 10000)
                if 0 < i1 <= lat.nleg11.get(L, 0):
                    out.append((kdir, I, i1))
        return out

    for ij in _ij_list(geo):
        names = {1: ["elec_up", "elec_down"], 3: ["spin_sd"], 5: ["num_sn"], 6: []}[ij]
        # bond terms that use the block operators before they are embedded
        for kdir, I, i1 in block_neighbours():
            if side == "sys":
                coefx = np.conj(geo.jt(kdir, jlat) * geo.pint(jlat, I))
            else:
                coefx = np.conj(geo.jt(kdir, jlat) * geo.pint(jlat, I))
            coefsd = geo.jd(kdir, jlat)
            if ij == 1 and coefx != 0:
                if side == "sys":
                    get_hamiltonian_ndia(pre.sub[i1]["elec_up"], block_transfer_trans(st.elec_down),
                                         basis, coefx, next_ham, "F", "S")
                else:
                    get_hamiltonian_ndia(pre.sub[i1]["elec_down"], block_transfer_trans(st.elec_up),
                                         basis, coefx, next_ham, "F", "E")
            if ij == 3 and coefsd != 0:
                get_hamiltonian_ndia(pre.sub[i1]["spin_sd"], st.sd, basis, coefsd, next_ham,
                                     "B", "S" if side == "sys" else "E")
        # embed the block operators of the boundary sites
        for y in range(1, L + 1):
            i1 = lat.inb1.get((y, L), 10000)
            if i1 <= lat.nleg11.get(L, 0):
                d = next_sub.setdefault(i1, {})
                for nm in names:
                    if ij == 5:
                        d[nm] = update_block_dia(pre.sub[i1][nm], basis)
                    else:
                        d[nm] = update_block_ndia(pre.sub[i1][nm], basis,
                                                  "F" if ij == 1 else "B", side)
        # the new site's operators in the enlarged basis
        tmp = {}
        if ij == 1:
            tmp["elec_up"] = update_site_ndia(st.elec_up, basis, "F", side)
            tmp["elec_down"] = update_site_ndia(st.elec_down, basis, "F", side)
        elif ij == 3:
            tmp["spin_sd"] = update_site_ndia(st.sd, basis, "B", side)
        elif ij == 5:
            tmp["num_sn"] = update_site_dia(st.num_elec, basis)
        elif ij == 6:
            dbl = update_site_dia(st.double, basis)
        if ij == 5:
            for kdir, I, i1 in block_neighbours():
                cn = geo.jn(kdir, jlat)
                if cn != 0:
                    get_hamiltonian_dia(next_sub[i1]["num_sn"], tmp["num_sn"], cn, next_ham)
        if ij == 6:
            u = geo.hubbard(jlat)
            if u != 0.0:
                block_add_block_two(dbl, u + 0j, next_ham)
        # compact the operator indices for the enlarged block (code/get_ham.f90:227-264)
        nleg1 = lat.nleg11.get(L + 1, 0)
        for I in range(1, L + 1):
            I1 = lat.inb1.get((I, L), 10000)
            J = lat.inb1.get((I, L + 1), 10000)
            if J <= nleg1 and J != I1:
                for nm in names:
                    next_sub.setdefault(J, {})[nm] = next_sub[I1][nm].copy()
        j = lat.inb1.get((L + 1, L + 1), 10000)
        for nm in names:
            if j <= nleg1:
                next_sub.setdefault(j, {})[nm] = tmp[nm]
        for jj in range(nleg1 + 1, lat.nleg11.get(L, 0) + 1):
            if jj in next_sub:
                for nm in names:
                    next_sub[jj].pop(nm, None)
        # truncate the boundary operators (code/get_ham.f90:301-327)
        for ii in range(1, lat.nleg11.get(L + 1, 0) + 1):
            dst = pre.sub.setdefault(ii, {})
            for nm in names:
                if ij == 5:
                    dst[nm] = update_trun_dia(next_sub[ii][nm], trun)
                else:
                    dst[nm] = update_trun_ndia(next_sub[ii][nm], trun)
    for ii in list(pre.sub.keys()):
        if ii > lat.nleg11.get(L + 1, 0):
            del pre.sub[ii]
    pre.ham = update_trun_dia(next_ham, trun)
    pre.len = L + 1
    return pre
