"""Superblock matvec ``model_wave`` and its term kernels (code/mat_vec.f90).

Every function restates the loop nest of the Fortran routine named in its
docstring: the same sector matching, the same 6j recoupling coefficients,
phases and fermion signs, and the same pair of GEMMs per sub-block (numpy
``@`` in place of ZGEMM).  ``coef`` arguments are complex.
"""
import numpy as np

from .blocks import SU, block_transfer_trans, block_add_block_two
from .su2 import w6j, parity_sign


def _fsign(flag, n):
    if flag == "B":
        return 1.0
    return 1.0 if n % 2 == 0 else -1.0


# ---------------------------------------------------------------------------
# diagonal (rank-0) terms
# ---------------------------------------------------------------------------
def block_vec_dia(sys_bl, sys_bs, invec, outvec, coef):
    """(O_sys x 1) psi (code/mat_vec.f90:165-215)."""
    for i, w in enumerate(invec.subs):
        sec = sys_bs.find(w.sys_num_up, w.sys_num_down)
        if sec is None:
            continue
        for y in sec.subs:
            c1 = coef / np.sqrt(1.0 + y.bl_num_down)
            k = sys_bl.find(y.bl_num_up, y.bl_num_down)
            if k is not None:
                o = outvec.subs[i].vec
                o[y.spos:y.spos + y.sdim, :] += c1 * (sys_bl.subs[k].mat @ w.vec[y.spos:y.spos + y.sdim, :])


def vec_block_dia(env_bl, env_bs, invec, outvec, coef):
    """(1 x O_env) psi = psi O_env^H (code/mat_vec.f90:218-267)."""
    for i, w in enumerate(invec.subs):
        sec = env_bs.find(w.env_num_up, w.env_num_down)
        if sec is None:
            continue
        for y in sec.subs:
            c1 = coef / np.sqrt(1.0 + y.bl_num_down)
            k = env_bl.find(y.bl_num_up, y.bl_num_down)
            if k is not None:
                o = outvec.subs[i].vec
                o[:, y.spos:y.spos + y.sdim] += c1 * (w.vec[:, y.spos:y.spos + y.sdim]
                                                      @ np.conj(env_bl.subs[k].mat).T)


def block_site_vec_dia(sys_bl, sys_st, sys_bs, invec, outvec, coef):
    """(O_sysblock n_syssite) psi (code/mat_vec.f90:388-460)."""
    for i, w in enumerate(invec.subs):
        sec = sys_bs.find(w.sys_num_up, w.sys_num_down)
        if sec is None:
            continue
        for y in sec.subs:
            b = sys_bl.find(y.bl_num_up, y.bl_num_down)
            s = sys_st.find(y.st_num_up, y.st_num_down)
            if b is not None and s is not None:
                c = coef * sys_st.subs[s].mat[0, 0] / np.sqrt((1.0 + y.bl_num_down) * (1.0 + y.st_num_down))
                o = outvec.subs[i].vec
                o[y.spos:y.spos + y.sdim, :] += c * (sys_bl.subs[b].mat @ w.vec[y.spos:y.spos + y.sdim, :])


def vec_block_site_dia(env_bl, env_st, env_bs, invec, outvec, coef):
    """(O_envblock n_envsite) psi (code/mat_vec.f90:463-537)."""
    for i, w in enumerate(invec.subs):
        sec = env_bs.find(w.env_num_up, w.env_num_down)
        if sec is None:
            continue
        for y in sec.subs:
            b = env_bl.find(y.bl_num_up, y.bl_num_down)
            s = env_st.find(y.st_num_up, y.st_num_down)
            if b is not None and s is not None:
                c = coef * env_st.subs[s].mat[0, 0] / np.sqrt((1.0 + y.bl_num_down) * (1.0 + y.st_num_down))
                o = outvec.subs[i].vec
                o[:, y.spos:y.spos + y.sdim] += c * (w.vec[:, y.spos:y.spos + y.sdim]
                                                     @ np.conj(env_bl.subs[b].mat).T)


def site_vec_site_dia(sys_st, env_st, sys_bs, env_bs, invec, outvec, coef):
    """(n_syssite x n_envsite) psi as scaled sub-block copies (code/mat_vec.f90:540-636)."""
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        o = outvec.subs[i].vec
        for x in ss.subs:
            a = sys_st.find(x.st_num_up, x.st_num_down)
            for y in es.subs:
                b = env_st.find(y.st_num_up, y.st_num_down)
                if a is not None and b is not None:
                    c = coef * sys_st.subs[a].mat[0, 0] * env_st.subs[b].mat[0, 0]
                    c = c / np.sqrt((1.0 + x.st_num_down) * (1.0 + y.st_num_down))
                    o[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim] += \
                        c * w.vec[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim]


def block_vec_site_dia(sys_bl, env_st, sys_bs, env_bs, invec, outvec, coef):
    """(O_sysblock n_envsite) psi (code/mat_vec.f90:640-740)."""
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        o = outvec.subs[i].vec
        for x in ss.subs:
            a = sys_bl.find(x.bl_num_up, x.bl_num_down)
            for y in es.subs:
                b = env_st.find(y.st_num_up, y.st_num_down)
                if a is not None and b is not None:
                    c = coef * env_st.subs[b].mat[0, 0] / np.sqrt((1.0 + y.st_num_down) * (1.0 + x.bl_num_down))
                    o[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim] += \
                        c * (sys_bl.subs[a].mat @ w.vec[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim])


def site_vec_block_dia(sys_st, env_bl, sys_bs, env_bs, invec, outvec, coef):
    """(n_syssite O_envblock) psi (code/mat_vec.f90:743-843)."""
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        o = outvec.subs[i].vec
        for x in ss.subs:
            a = sys_st.find(x.st_num_up, x.st_num_down)
            for y in es.subs:
                b = env_bl.find(y.bl_num_up, y.bl_num_down)
                if a is not None and b is not None:
                    c = coef * sys_st.subs[a].mat[0, 0] / np.sqrt((1.0 + y.bl_num_down) * (1.0 + x.st_num_down))
                    o[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim] += \
                        c * (w.vec[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim]
                             @ np.conj(env_bl.subs[b].mat).T)


def block_vec_block_dia(sys_bl, env_bl, sys_bs, env_bs, invec, outvec, coef):
    """(O_sysblock x O_envblock) psi, rank 0 (code/mat_vec.f90:846-951)."""
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        o = outvec.subs[i].vec
        for x in ss.subs:
            a = sys_bl.find(x.bl_num_up, x.bl_num_down)
            for y in es.subs:
                b = env_bl.find(y.bl_num_up, y.bl_num_down)
                if a is not None and b is not None:
                    c = coef / np.sqrt((1.0 + y.bl_num_down) * (1.0 + x.bl_num_down))
                    mat = sys_bl.subs[a].mat @ w.vec[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim]
                    o[x.spos:x.spos + x.sdim, y.spos:y.spos + y.sdim] += c * (mat @ np.conj(env_bl.subs[b].mat).T)


# ---------------------------------------------------------------------------
# non-diagonal (rank-k) terms
# ---------------------------------------------------------------------------
def block_site_vec_ndia(sys_bl, flag_bl, sys_st, flag_st, sys_bs, invec, outvec, coef):
    """(O_sysblock . O_syssite)^0 psi + h.c. (code/mat_vec.f90:960-1216).

    Loops over sys sub-blocks x and the two component shifts; the output stays
    in the same superblock sector.  6j: {new_bl, bl, k; st, new_st, J}.
    """
    up_dif, k = sys_bl.up_dif, sys_bl.down_dif
    assert up_dif == sys_st.up_dif and k == sys_st.down_dif
    for i, w in enumerate(invec.subs):
        sec = sys_bs.find(w.sys_num_up, w.sys_num_down)
        if sec is None:
            continue
        o = outvec.subs[i].vec
        for x in sec.subs:
            for dd in range(-k, k + 1, SU):
                for sdd in range(-k, k + 1, SU):
                    bl_id = sys_bl.find(x.bl_num_up, x.bl_num_down, dd)
                    nsu, nsd = x.st_num_up - up_dif, x.st_num_down - sdd
                    st_id = sys_st.find(nsu, nsd, sdd)
                    nbu, nbd = x.bl_num_up + up_dif, x.bl_num_down + dd
                    if bl_id is None or st_id is None:
                        continue
                    y = sec.find_full(nbu, nbd, nsu, nsd)
                    if y is None:
                        continue
                    sgn = _fsign(flag_st, x.bl_num_up)
                    j1, j2, j3, j4, j5, j6 = nbd, x.bl_num_down, k, x.st_num_down, nsd, w.sys_num_down
                    c1 = w6j(j1, j2, j3, j4, j5, j6)
                    if c1 == 0.0:
                        continue
                    c1 = c1 * parity_sign(j2 + j5 + j3 + j6) / np.sqrt(1.0 + k)
                    c = sgn * c1 * coef * sys_st.subs[st_id].mat[0, 0]
                    A = sys_bl.subs[bl_id].mat
                    o[y.spos:y.spos + y.sdim, :] += c * (A @ w.vec[x.spos:x.spos + x.sdim, :])
                    if up_dif != 0:
                        o[x.spos:x.spos + x.sdim, :] += np.conj(c) * (np.conj(A).T @ w.vec[y.spos:y.spos + y.sdim, :])


def vec_block_site_ndia(env_bl, flag_bl, env_st, flag_st, env_bs, invec, outvec, coef):
    """(O_envblock . O_envsite)^0 psi + h.c. (code/mat_vec.f90:1219-1503)."""
    up_dif, k = env_bl.up_dif, env_bl.down_dif
    assert up_dif == env_st.up_dif and k == env_st.down_dif
    for i, w in enumerate(invec.subs):
        sec = env_bs.find(w.env_num_up, w.env_num_down)
        if sec is None:
            continue
        o = outvec.subs[i].vec
        for x in sec.subs:
            for bdd in range(-k, k + 1, SU):
                bl_id = env_bl.find(x.bl_num_up, x.bl_num_down, bdd)
                for sdd in range(-k, k + 1, SU):
                    nsu, nsd = x.st_num_up - up_dif, x.st_num_down - sdd
                    st_id = env_st.find(nsu, nsd, sdd)
                    nbu, nbd = x.bl_num_up + up_dif, x.bl_num_down + bdd
                    if st_id is None or bl_id is None:
                        continue
                    y = sec.find_full(nbu, nbd, nsu, nsd)
                    if y is None:
                        continue
                    sbl = _fsign(flag_bl, w.sys_num_up + nsu)
                    sst = _fsign(flag_st, w.sys_num_up)
                    j1, j2, j3, j4, j5, j6 = nbd, x.bl_num_down, k, x.st_num_down, nsd, w.env_num_down
                    c1 = w6j(j1, j2, j3, j4, j5, j6)
                    if c1 == 0.0:
                        continue
                    c1 = c1 * parity_sign(j2 + j5 + j3 + j6) / np.sqrt(1.0 + k)
                    c = sbl * sst * c1 * coef * env_st.subs[st_id].mat[0, 0]
                    B = env_bl.subs[bl_id].mat
                    o[:, y.spos:y.spos + y.sdim] += c * (w.vec[:, x.spos:x.spos + x.sdim] @ np.conj(B).T)
                    if up_dif != 0:
                        o[:, x.spos:x.spos + x.sdim] += np.conj(c) * (w.vec[:, y.spos:y.spos + y.sdim] @ B)


def block_vec_block_ndia(sys_bl, flag_sl, env_bl, flag_el, sys_bs, env_bs, invec, outvec, coef):
    """(O_sysblock . O_envblock)^0 psi + h.c., the dominant term (code/mat_vec.f90:1505-1928).

    For each in-sector i, sys sub m, env sub n, the two component shifts and
    each admissible new total 2S': out_k[new sys sub, new env sub] +=
    c * A psi_i[m, n] B and, when up_dif != 0, the h.c. pair.  Coefficient
    (code/mat_vec.f90:1693-1731): 6j{J', k, J; j_bl, s, j_bl'} * 6j on the env
    side * sqrt((2S'_e+1)(2S_e+1)/(k+1)) * phase * fermion sign.
    """
    up_dif, k = sys_bl.up_dif, sys_bl.down_dif
    assert up_dif == env_bl.up_dif and k == env_bl.down_dif
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        for m in ss.subs:
            for n in es.subs:
                for dd in range(-k, k + 1, SU):
                    sb_id = sys_bl.find(m.bl_num_up, m.bl_num_down, dd)
                    nsbu, nsbd = m.bl_num_up + up_dif, m.bl_num_down + dd
                    for edd in range(-k, k + 1, SU):
                        nebu, nebd = n.bl_num_up - up_dif, n.bl_num_down - edd
                        eb_id = env_bl.find(nebu, nebd, edd)
                        if sb_id is None or eb_id is None:
                            continue
                        for nsd in range(abs(w.sys_num_down - k), w.sys_num_down + k + 1, SU):
                            nsu = w.sys_num_up + up_dif
                            neu = w.env_num_up - up_dif
                            ned = nsd
                            tsec = sys_bs.find(nsu, nsd)
                            ms = tsec.find_full(nsbu, nsbd, m.st_num_up, m.st_num_down) if tsec else None
                            tsec2 = env_bs.find(neu, ned)
                            me = tsec2.find_full(nebu, nebd, n.st_num_up, n.st_num_down) if tsec2 else None
                            if ms is None or me is None:
                                continue
                            kk = outvec.find(nsu, nsd, neu, ned)
                            if kk is None:
                                continue
                            sel = _fsign(flag_el, w.sys_num_up + n.st_num_up)
                            j1, j2, j3, j4, j5, j6 = nsd, k, w.sys_num_down, m.bl_num_down, m.st_num_down, nsbd
                            j11, j22, j33, j44, j55, j66 = ned, k, w.env_num_down, n.bl_num_down, n.st_num_down, nebd
                            c1 = w6j(j1, j2, j3, j4, j5, j6)
                            if c1 == 0.0:
                                continue
                            c11 = w6j(j11, j22, j33, j44, j55, j66)
                            if c11 == 0.0:
                                continue
                            c1 = c1 * c11 * np.sqrt((1.0 + j11) * (1.0 + j33) / (1.0 + k))
                            if ((j6 + j5 + j3 + j2) // 2 + (j66 + j55 + j33 + j22) // 2) % 2 == 1:
                                c1 = -c1
                            c = sel * coef * c1
                            A = sys_bl.subs[sb_id].mat
                            B = env_bl.subs[eb_id].mat
                            x_in = w.vec[m.spos:m.spos + m.sdim, n.spos:n.spos + n.sdim]
                            o = outvec.subs[kk].vec
                            mat = A @ x_in
                            o[ms.spos:ms.spos + ms.sdim, me.spos:me.spos + me.sdim] += c * (mat @ B)
                            if up_dif != 0:
                                x2 = invec.subs[kk].vec[ms.spos:ms.spos + ms.sdim, me.spos:me.spos + me.sdim]
                                mat2 = np.conj(A).T @ x2
                                outvec.subs[i].vec[m.spos:m.spos + m.sdim, n.spos:n.spos + n.sdim] += \
                                    np.conj(c) * (mat2 @ np.conj(B).T)


def block_vec_site_ndia(sys_bl, flag_sl, env_st, flag_et, sys_bs, env_bs, invec, outvec, coef):
    """(O_sysblock . O_envsite)^0 psi + h.c. (code/mat_vec.f90:2324-2690)."""
    up_dif, k = sys_bl.up_dif, sys_bl.down_dif
    assert up_dif == env_st.up_dif and k == env_st.down_dif
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        for m in ss.subs:
            for n in es.subs:
                for bdd in range(-k, k + 1, SU):
                    nsbu, nsbd = m.bl_num_up + up_dif, m.bl_num_down + bdd
                    sb_id = sys_bl.find(m.bl_num_up, m.bl_num_down, bdd)
                    for sdd in range(-k, k + 1, SU):
                        nesu, nesd = n.st_num_up - up_dif, n.st_num_down - sdd
                        st_id = env_st.find(nesu, nesd, sdd)
                        nsu = w.sys_num_up + up_dif
                        neu = w.env_num_up - up_dif
                        if sb_id is None or st_id is None:
                            continue
                        for nsd in range(abs(w.sys_num_down - k), w.sys_num_down + k + 1, SU):
                            ned = nsd
                            tsec = sys_bs.find(nsu, nsd)
                            ms = None
                            if tsec is not None:
                                for l in tsec.subs:
                                    if l.bl_num_up == nsbu and l.bl_num_down == nsbd and l.st_num_down == m.st_num_down:
                                        ms = l
                                        break
                            tsec2 = env_bs.find(neu, ned)
                            me = None
                            if tsec2 is not None:
                                for l in tsec2.subs:
                                    if l.st_num_up == nesu and l.st_num_down == nesd and l.bl_num_down == n.bl_num_down:
                                        me = l
                                        break
                            if ms is None or me is None:
                                continue
                            kk = outvec.find(nsu, nsd, neu, ned)
                            if kk is None:
                                continue
                            set_ = _fsign(flag_et, w.sys_num_up)
                            j1, j2, j3, j4, j5, j6 = nsd, k, w.sys_num_down, m.bl_num_down, m.st_num_down, nsbd
                            j11, j22, j33, j44, j55, j66 = ned, k, w.env_num_down, n.st_num_down, n.bl_num_down, nesd
                            c1 = w6j(j1, j2, j3, j4, j5, j6)
                            if c1 == 0.0:
                                continue
                            c11 = w6j(j11, j22, j33, j44, j55, j66)
                            if c11 == 0.0:
                                continue
                            c1 = c1 * c11 * np.sqrt((1.0 + j11) * (1.0 + j33) / (1.0 + k))
                            if ((j6 + j5 + j3 + j2) // 2 + (j55 + j44 + j11 + j22) // 2) % 2 != 0:
                                c1 = -c1
                            c = set_ * c1 * coef * env_st.subs[st_id].mat[0, 0]
                            A = sys_bl.subs[sb_id].mat
                            edim = n.sdim
                            x_in = w.vec[m.spos:m.spos + m.sdim, n.spos:n.spos + edim]
                            o = outvec.subs[kk].vec
                            o[ms.spos:ms.spos + ms.sdim, me.spos:me.spos + edim] += c * (A @ x_in)
                            if up_dif != 0:
                                x2 = invec.subs[kk].vec[ms.spos:ms.spos + ms.sdim, me.spos:me.spos + edim]
                                outvec.subs[i].vec[m.spos:m.spos + m.sdim, n.spos:n.spos + edim] += \
                                    np.conj(c) * (np.conj(A).T @ x2)


def site_vec_block_ndia(sys_st, flag_st, env_bl, flag_el, sys_bs, env_bs, invec, outvec, coef):
    """(O_syssite . O_envblock)^0 psi + h.c. (code/mat_vec.f90:2695-3098)."""
    up_dif, k = sys_st.up_dif, sys_st.down_dif
    assert up_dif == env_bl.up_dif and k == env_bl.down_dif
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        for m in ss.subs:
            for n in es.subs:
                for sdd in range(-k, k + 1, SU):
                    nssu, nssd = m.st_num_up + up_dif, m.st_num_down + sdd
                    ss_id = sys_st.find(m.st_num_up, m.st_num_down, sdd)
                    for bdd in range(-k, k + 1, SU):
                        nebu, nebd = n.bl_num_up - up_dif, n.bl_num_down - bdd
                        eb_id = env_bl.find(nebu, nebd, bdd)
                        nsu = w.sys_num_up + up_dif
                        neu = w.env_num_up - up_dif
                        if ss_id is None or eb_id is None:
                            continue
                        for nsd in range(abs(w.sys_num_down - k), w.sys_num_down + k + 1, SU):
                            ned = nsd
                            tsec = sys_bs.find(nsu, nsd)
                            ms = tsec.find_full(m.bl_num_up, m.bl_num_down, nssu, nssd) if tsec else None
                            tsec2 = env_bs.find(neu, ned)
                            me = tsec2.find_full(nebu, nebd, n.st_num_up, n.st_num_down) if tsec2 else None
                            if ms is None or me is None:
                                continue
                            kk = outvec.find(nsu, nsd, neu, ned)
                            if kk is None:
                                continue
                            j1, j2, j3, j4, j5, j6 = nsd, k, w.sys_num_down, m.st_num_down, m.bl_num_down, nssd
                            j11, j22, j33, j44, j55, j66 = ned, k, w.env_num_down, n.bl_num_down, n.st_num_down, nebd
                            c1 = w6j(j1, j2, j3, j4, j5, j6)
                            if c1 == 0.0:
                                continue
                            c11 = w6j(j11, j22, j33, j44, j55, j66)
                            if c11 == 0.0:
                                continue
                            c1 = c1 * c11 * np.sqrt((1.0 + j11) * (j33 + 1.0) / (1.0 + k))
                            if ((j66 + j55 + j33 + j22) // 2 + (j5 + j4 + j1 + j2) // 2) % 2 != 0:
                                c1 = -c1
                            sst = _fsign(flag_st, m.bl_num_up)
                            sel = _fsign(flag_el, w.sys_num_up + n.st_num_up)
                            c = sst * sel * c1 * coef * sys_st.subs[ss_id].mat[0, 0]
                            B = env_bl.subs[eb_id].mat
                            sdim = m.sdim
                            x_in = w.vec[m.spos:m.spos + sdim, n.spos:n.spos + n.sdim]
                            o = outvec.subs[kk].vec
                            o[ms.spos:ms.spos + sdim, me.spos:me.spos + me.sdim] += c * (x_in @ B)
                            if up_dif != 0:
                                x2 = invec.subs[kk].vec[ms.spos:ms.spos + sdim, me.spos:me.spos + me.sdim]
                                outvec.subs[i].vec[m.spos:m.spos + sdim, n.spos:n.spos + n.sdim] += \
                                    np.conj(c) * (x2 @ np.conj(B).T)


def site_vec_site_ndia(sys_st, flag_st, env_st, flag_et, sys_bs, env_bs, invec, outvec, coef):
    """(O_syssite . O_envsite)^0 psi + h.c. as scaled copies (code/mat_vec.f90:3101-3470)."""
    up_dif, k = sys_st.up_dif, sys_st.down_dif
    assert up_dif == env_st.up_dif and k == env_st.down_dif
    for i, w in enumerate(invec.subs):
        ss = sys_bs.find(w.sys_num_up, w.sys_num_down)
        es = env_bs.find(w.env_num_up, w.env_num_down)
        if ss is None or es is None:
            continue
        for m in ss.subs:
            for n in es.subs:
                for sdd1 in range(-k, k + 1, SU):
                    s_id = sys_st.find(m.st_num_up, m.st_num_down, sdd1)
                    nssu, nssd = m.st_num_up + up_dif, m.st_num_down + sdd1
                    for sdd2 in range(-k, k + 1, SU):
                        nesu, nesd = n.st_num_up - up_dif, n.st_num_down - sdd2
                        e_id = env_st.find(nesu, nesd, sdd2)
                        nsu = w.sys_num_up + up_dif
                        neu = w.env_num_up - up_dif
                        if s_id is None or e_id is None:
                            continue
                        for nsd in range(abs(w.sys_num_down - k), w.sys_num_down + k + 1, SU):
                            ned = nsd
                            tsec = sys_bs.find(nsu, nsd)
                            ms = None
                            if tsec is not None:
                                for l in tsec.subs:
                                    if l.st_num_up == nssu and l.st_num_down == nssd and l.bl_num_down == m.bl_num_down:
                                        ms = l
                                        break
                            tsec2 = env_bs.find(neu, ned)
                            me = None
                            if tsec2 is not None:
                                for l in tsec2.subs:
                                    if l.st_num_up == nesu and l.st_num_down == nesd and l.bl_num_down == n.bl_num_down:
                                        me = l
                                        break
                            if ms is None or me is None:
                                continue
                            kk = outvec.find(nsu, nsd, neu, ned)
                            if kk is None:
                                continue
                            sst = _fsign(flag_st, m.bl_num_up)
                            set_ = _fsign(flag_et, w.sys_num_up)
                            ctmp = sst * set_ * coef
                            j1, j2, j3, j4, j5, j6 = nsd, k, w.sys_num_down, m.st_num_down, m.bl_num_down, nssd
                            j11, j22, j33, j44, j55, j66 = ned, k, w.env_num_down, n.st_num_down, n.bl_num_down, nesd
                            c1 = w6j(j1, j2, j3, j4, j5, j6)
                            if c1 == 0.0:
                                continue
                            c11 = w6j(j11, j22, j33, j44, j55, j66)
                            if c11 == 0.0:
                                continue
                            c1 = c1 * c11 * np.sqrt((1.0 + j11) * (1.0 + j33) / (1.0 + k))
                            if ((j55 + j44 + j11 + j22) // 2 + (j5 + j4 + j1 + j2) // 2) % 2 != 0:
                                c1 = -c1
                            c = ctmp * c1 * sys_st.subs[s_id].mat[0, 0] * env_st.subs[e_id].mat[0, 0]
                            sdim, edim = m.sdim, n.sdim
                            outvec.subs[kk].vec[ms.spos:ms.spos + sdim, me.spos:me.spos + edim] += \
                                c * w.vec[m.spos:m.spos + sdim, n.spos:n.spos + edim]
                            if up_dif != 0:
                                outvec.subs[i].vec[m.spos:m.spos + sdim, n.spos:n.spos + edim] += \
                                    np.conj(c) * invec.subs[kk].vec[ms.spos:ms.spos + sdim, me.spos:me.spos + edim]


# ---------------------------------------------------------------------------
# hmerge and model_wave
# ---------------------------------------------------------------------------
def hmerge(sys, env, geo):
    """Merge boundary couplings into snc/sub_s operators (code/mat_vec.f90:3623-3852).

    ``geo`` holds the lattice tables of the current superblock (see
    ``oracle.lattice``).  Sets geo.coup_bs, geo.coup_bb and geo.inb.
    """
    sl, el = sys.len, env.len
    syssite = sl + 1
    dmsite = sl + el + 2
    coup_bs = [[0, 0], [0, 0]]
    for j in geo.neighbours(syssite):
        p = geo.region(j)
        if p == 3:
            coup_bs[1][0] = 1
        if p == 1:
            coup_bs[0][0] = 1
    for j in geo.neighbours(geo.nposi_lat[dmsite]):
        p = geo.region(j)
        if p == 3:
            coup_bs[1][1] = 1
        if p == 1:
            coup_bs[0][1] = 1
    geo.coup_bs = coup_bs
    names = geo.op_names()
    for ia in range(2):
        if coup_bs[0][ia]:
            sys.snc[ia] = {nm: sys.sub[1][nm].zeros_like() for nm in names if nm != "elec_down"}
        if coup_bs[1][ia]:
            env.snc[ia] = {nm: env.sub[1][nm].zeros_like() for nm in names}
    for ia in range(2):
        j = sl + 1 + (el + 1) * ia
        lj = geo.nposi_lat[j]
        for kdir, ib in geo.bonds(lj):
            p = geo.region(ib)
            if p == 3 and coup_bs[1][ia]:
                ib1 = geo.inb1[(geo.nposi_dm[ib] - sl - 1, el)]
                jt1 = geo.jt(kdir, lj) * geo.pint(lj, ib)
                jd1 = geo.jd(kdir, lj)
                jn1 = geo.jn(kdir, lj)
                if jt1 != 0:
                    block_add_block_two(env.sub[ib1]["elec_up"], jt1, env.snc[ia]["elec_up"])
                    block_add_block_two(env.sub[ib1]["elec_down"], np.conj(jt1), env.snc[ia]["elec_down"])
                if geo.tjmodel and jd1 != 0:
                    block_add_block_two(env.sub[ib1]["spin_sd"], jd1, env.snc[ia]["spin_sd"])
                if jn1 != 0 and "num_sn" in env.snc[ia]:
                    block_add_block_two(env.sub[ib1]["num_sn"], jn1, env.snc[ia]["num_sn"])
            if p == 1 and coup_bs[0][ia]:
                ib1 = geo.inb1[(geo.nposi_dm[ib], sl)]
                jt1 = geo.jt(kdir, lj) * geo.pint(lj, ib)
                jd1 = geo.jd(kdir, lj)
                jn1 = geo.jn(kdir, lj)
                if jt1 != 0:
                    block_add_block_two(sys.sub[ib1]["elec_up"], np.conj(jt1), sys.snc[ia]["elec_up"])
                if geo.tjmodel and jd1 != 0:
                    block_add_block_two(sys.sub[ib1]["spin_sd"], jd1, sys.snc[ia]["spin_sd"])
                if jn1 != 0 and "num_sn" in sys.snc[ia]:
                    block_add_block_two(sys.sub[ib1]["num_sn"], jn1, sys.snc[ia]["num_sn"])

    # block-block bookkeeping (code/mat_vec.f90:3745-3782)
    inb = {}
    k11 = 0
    for i in range(1, sl + 1):
        k1 = sum(1 for j in geo.neighbours(i) if geo.region(j) == 3)
        inb[i] = k1
        if geo.nleg11.get(el, 0) < geo.nleg11.get(sl, 0):
            inb[i] = 0
        if inb[i] != 0:
            k11 += 1
    cbb1 = k11
    inb[sl + 1] = 0
    inb[sl + 1 + el + 1] = 0
    for i in range(1, el + 1):
        k1 = 0
        inb[i + sl + 1] = 0
        for j in geo.neighbours(geo.nposi_lat[i + sl + 1]):
            if geo.region(j) == 1 and inb.get(j, 0) == 0:
                k1 += 1
        inb[i + sl + 1] = k1
        if k1 != 0:
            k11 += 1
    geo.coup_bb = [cbb1, k11 - cbb1]
    geo.inb = inb
    env.sub_s = {i: {nm: env.sub[1][nm].zeros_like() for nm in names} for i in range(1, cbb1 + 1)}
    sys.sub_s = {i: {nm: sys.sub[1][nm].zeros_like() for nm in names if nm != "elec_down"}
                 for i in range(1, geo.coup_bb[1] + 1)}
    jc = 0
    for i in range(1, sl + el + 2):
        if inb.get(i, 0) == 0:
            continue
        ia = geo.nposi_lat[i]
        jc += 1
        for kdir, ib in geo.bonds(ia):
            p = geo.region(ib)
            if p == 3 and i <= sl:
                ib1 = geo.inb1[(geo.nposi_dm[ib] - sl - 1, el)]
                jt1 = geo.jt(kdir, ia) * geo.pint(ia, ib)
                jd1 = geo.jd(kdir, ia)
                jn1 = geo.jn(kdir, ia)
                if jt1 != 0:
                    block_add_block_two(env.sub[ib1]["elec_up"], jt1, env.sub_s[jc]["elec_up"])
                    block_add_block_two(env.sub[ib1]["elec_down"], np.conj(jt1), env.sub_s[jc]["elec_down"])
                if geo.tjmodel and jd1 != 0:
                    block_add_block_two(env.sub[ib1]["spin_sd"], jd1, env.sub_s[jc]["spin_sd"])
                if jn1 != 0 and "num_sn" in env.sub_s[jc]:
                    block_add_block_two(env.sub[ib1]["num_sn"], jn1, env.sub_s[jc]["num_sn"])
            if p == 1 and i > sl + 1:
                if inb.get(geo.nposi_dm[ib], 0) == 0:
                    ib1 = geo.inb1[(ib, sl)]
                    jc1 = jc - cbb1
                    jt1 = geo.jt(kdir, ia) * geo.pint(ia, ib)
                    jd1 = geo.jd(kdir, ia)
                    jn1 = geo.jn(kdir, ia)
                    if jt1 != 0:
                        block_add_block_two(sys.sub[ib1]["elec_up"], np.conj(jt1), sys.sub_s[jc1]["elec_up"])
                    if geo.tjmodel and jd1 != 0:
                        block_add_block_two(sys.sub[ib1]["spin_sd"], jd1, sys.sub_s[jc1]["spin_sd"])
                    if jn1 != 0 and "num_sn" in sys.sub_s[jc1]:
                        block_add_block_two(sys.sub[ib1]["num_sn"], jn1, sys.sub_s[jc1]["num_sn"])


def model_wave(sys, env, sys_bs, env_bs, invec, outvec, geo, st):
    """H psi for the superblock [sys_bl - sys_site - env_site - env_bl]
    (code/mat_vec.f90:3476-3620).  ``st`` holds the site operators."""
    one = 1.0 + 0.0j
    for w in outvec.subs:
        w.vec[...] = 0.0
    block_vec_dia(sys.ham, sys_bs, invec, outvec, one)
    vec_block_dia(env.ham, env_bs, invec, outvec, one)
    is_ = geo.nposi_lat[sys.len + 1]
    js = geo.nposi_lat[sys.len + env.len + 2]
    if geo.hubbard(is_) != 0.0:
        site_vec_site_dia(st.double, st.si, sys_bs, env_bs, invec, outvec, geo.hubbard(is_) + 0j)
    if geo.hubbard(js) != 0.0:
        site_vec_site_dia(st.si, st.double, sys_bs, env_bs, invec, outvec, geo.hubbard(js) + 0j)
    ii = geo.neiba(is_, js)
    if ii != 0:
        jd1 = geo.jd(ii, is_)
        jn1 = geo.jn(ii, is_)
        coefx = geo.jt(ii, is_) * geo.pint(is_, js)
        if coefx != 0:
            site_vec_site_ndia(st.elec_up, "F", block_transfer_trans(st.elec_down), "F",
                               sys_bs, env_bs, invec, outvec, coefx)
        if jd1 != 0:
            site_vec_site_ndia(st.sd, "B", st.sd, "B", sys_bs, env_bs, invec, outvec, jd1)
        if jn1 != 0:
            site_vec_site_dia(st.num_elec, st.num_elec, sys_bs, env_bs, invec, outvec, jn1)
    cb = geo.coup_bs
    if cb[0][0] == 1:
        block_site_vec_ndia(sys.snc[0]["elec_up"], "F", block_transfer_trans(st.elec_down), "F",
                            sys_bs, invec, outvec, one)
        if geo.tjmodel:
            block_site_vec_ndia(sys.snc[0]["spin_sd"], "B", st.sd, "B", sys_bs, invec, outvec, one)
        if geo.v123:
            block_site_vec_dia(sys.snc[0]["num_sn"], st.num_elec, sys_bs, invec, outvec, one)
    if cb[0][1] == 1:
        block_vec_site_ndia(sys.snc[1]["elec_up"], "F", block_transfer_trans(st.elec_down), "F",
                            sys_bs, env_bs, invec, outvec, one)
        if geo.tjmodel:
            block_vec_site_ndia(sys.snc[1]["spin_sd"], "B", st.sd, "B", sys_bs, env_bs, invec, outvec, one)
        if geo.v123:
            block_vec_site_dia(sys.snc[1]["num_sn"], st.num_elec, sys_bs, env_bs, invec, outvec, one)
    if cb[1][0] == 1:
        site_vec_block_ndia(st.elec_up, "F", block_transfer_trans(env.snc[0]["elec_down"]), "F",
                            sys_bs, env_bs, invec, outvec, one)
        if geo.tjmodel:
            site_vec_block_ndia(st.sd, "B", block_transfer_trans(env.snc[0]["spin_sd"]), "B",
                                sys_bs, env_bs, invec, outvec, one)
        if geo.v123:
            site_vec_block_dia(st.num_elec, env.snc[0]["num_sn"], sys_bs, env_bs, invec, outvec, one)
    if cb[1][1] == 1:
        vec_block_site_ndia(env.snc[1]["elec_up"], "F", block_transfer_trans(st.elec_down), "F",
                            env_bs, invec, outvec, one)
        if geo.tjmodel:
            vec_block_site_ndia(env.snc[1]["spin_sd"], "B", st.sd, "B", env_bs, invec, outvec, one)
        if geo.v123:
            vec_block_site_dia(env.snc[1]["num_sn"], st.num_elec, env_bs, invec, outvec, one)
    jc = 0
    for i in range(1, sys.len + 1 + env.len + 1):
        if geo.inb.get(i, 0) == 0:
            continue
        jc += 1
        if i <= sys.len:
            i1 = geo.inb1[(i, sys.len)]
            block_vec_block_ndia(sys.sub[i1]["elec_up"], "F",
                                 block_transfer_trans(env.sub_s[jc]["elec_down"]), "F",
                                 sys_bs, env_bs, invec, outvec, one)
            if geo.tjmodel:
                block_vec_block_ndia(sys.sub[i1]["spin_sd"], "B",
                                     block_transfer_trans(env.sub_s[jc]["spin_sd"]), "B",
                                     sys_bs, env_bs, invec, outvec, one)
            if geo.v123:
                block_vec_block_dia(sys.sub[i1]["num_sn"], env.sub_s[jc]["num_sn"],
                                    sys_bs, env_bs, invec, outvec, one)
        else:
            i1 = geo.inb1[(i - sys.len - 1, env.len)]
            jc1 = jc - geo.coup_bb[0]
            block_vec_block_ndia(sys.sub_s[jc1]["elec_up"], "F",
                                 block_transfer_trans(env.sub[i1]["elec_down"]), "F",
                                 sys_bs, env_bs, invec, outvec, one)
            if geo.tjmodel:
                block_vec_block_ndia(sys.sub_s[jc1]["spin_sd"], "B",
                                     block_transfer_trans(env.sub[i1]["spin_sd"]), "B",
                                     sys_bs, env_bs, invec, outvec, one)
            if geo.v123:
                block_vec_block_dia(sys.sub_s[jc1]["num_sn"], env.sub[i1]["num_sn"],
                                    sys_bs, env_bs, invec, outvec, one)
