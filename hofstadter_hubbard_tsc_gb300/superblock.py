"""The superblock step behind the reference's subroutine names.

``Superblock`` holds one DMRG step's superblock [sys - site - site - env] on
the GPU: the block operators (resident), the merged boundary operators of
``hmerge`` (code/mat_vec.f90:3623-3852), the model_wave task plan and the
Lanczos workspace.  ``model_wave`` (code/mat_vec.f90:3476) and
``lanczos_memo_new`` (code/lanczos.f90:4) are its methods; the host work done
here is bookkeeping (which term kernels run with which operators and
coefficients); every arithmetic operation on blocks and waves runs in
libhh_dmrg.so.
"""
import ctypes as C

import numpy as np

from . import _lib
from .device import Device, DBlock, DBasis, DWave
from .sites import SiteOperators
from .types import Wavefunction, TotalBlock

F, B = ord("F"), ord("B")


class Term:
    __slots__ = ("kind", "op0", "op1", "flag0", "flag1", "trans0", "trans1", "coef")

    def __init__(self, kind, op0, op1=None, flag0=B, flag1=B, trans0=0, trans1=0, coef=1.0):
        self.kind, self.op0, self.op1 = kind, op0, op1
        self.flag0, self.flag1, self.trans0, self.trans1 = flag0, flag1, trans0, trans1
        self.coef = complex(coef)


def _dev_block(dev, b, cache):
    if isinstance(b, DBlock):
        return b
    key = id(b)
    if key not in cache:
        cache[key] = (b, DBlock.upload(dev, b))
    return cache[key][1]


class Superblock:
    """One superblock of the sweep (the arguments of lanczos_memo_new)."""

    def __init__(self, dev: Device, sys, env, sys_bs, env_bs, sup, geo, site_ops=None, precision=0):
        self.dev = dev
        self.sys, self.env = sys, env
        self.sys_bs, self.env_bs, self.sup, self.geo = sys_bs, env_bs, sup, geo
        self.st = site_ops or SiteOperators("tj" if geo.tjmodel else "hubbard")
        self._cache = {}
        self.precision = precision
        up = lambda b: _dev_block(dev, b, self._cache)
        self.d_sys_ham, self.d_env_ham = up(sys.ham), up(env.ham)
        self.d_sys = {i: {n: up(b) for n, b in d.items()} for i, d in sys.sub.items()}
        self.d_env = {i: {n: up(b) for n, b in d.items()} for i, d in env.sub.items()}
        st = self.st
        self.d_st = {n: up(getattr(st, n)) for n in ("elec_up", "elec_down", "num_elec", "double", "sd", "si")}
        self.hmerge()
        self.terms = self.model_wave_terms()
        self.d_sys_bs, self.d_env_bs = DBasis(dev, sys_bs), DBasis(dev, env_bs)
        self.layout = sup.array()
        self.w_in = DWave(dev, self.layout, sup.sys_len, sup.env_len)
        self.w_out = DWave(dev, self.layout, sup.sys_len, sup.env_len)
        self.plan = self._make_plan(self.terms)

    # ------------------------------------------------------------ hmerge
    def hmerge(self):
        """Merge the couplings of each boundary partner (code/mat_vec.f90:3623-3852)."""
        geo, sl, el = self.geo, self.sys.len, self.env.len
        names = geo.op_names()
        cb = [[0, 0], [0, 0]]
        for j in geo.neighbours(sl + 1):
            r = geo.region(j)
            if r == 3:
                cb[1][0] = 1
            if r == 1:
                cb[0][0] = 1
        for j in geo.neighbours(geo.nposi_lat[sl + el + 2]):
            r = geo.region(j)
            if r == 3:
                cb[1][1] = 1
            if r == 1:
                cb[0][1] = 1
        self.coup_bs = cb
        self.sys_snc, self.env_snc = [None, None], [None, None]
        for ia in range(2):
            if cb[0][ia]:
                self.sys_snc[ia] = {n: DBlock.zeros_like(self.d_sys[1][n]) for n in names if n != "elec_down"}
            if cb[1][ia]:
                self.env_snc[ia] = {n: DBlock.zeros_like(self.d_env[1][n]) for n in names}
        for ia in range(2):
            j = sl + 1 + (el + 1) * ia
            lj = geo.nposi_lat[j]
            for k, ib in geo.bonds(lj):
                r = geo.region(ib)
                jt1 = geo.jt(k, lj) * geo.pint(lj, ib)
                jd1, jn1 = geo.jd(k, lj), geo.jn(k, lj)
                if r == 3 and cb[1][ia]:
                    i1 = geo.inb1[(geo.nposi_dm[ib] - sl - 1, el)]
                    src, dst = self.d_env[i1], self.env_snc[ia]
                    if jt1 != 0:
                        dst["elec_up"].add(jt1, src["elec_up"])
                        dst["elec_down"].add(np.conj(jt1), src["elec_down"])
                    if geo.tjmodel and jd1 != 0:
                        dst["spin_sd"].add(jd1, src["spin_sd"])
                    if jn1 != 0 and "num_sn" in dst:
                        dst["num_sn"].add(jn1, src["num_sn"])
                if r == 1 and cb[0][ia]:
                    i1 = geo.inb1[(geo.nposi_dm[ib], sl)]
                    src, dst = self.d_sys[i1], self.sys_snc[ia]
                    if jt1 != 0:
                        dst["elec_up"].add(np.conj(jt1), src["elec_up"])
                    if geo.tjmodel and jd1 != 0:
                        dst["spin_sd"].add(jd1, src["spin_sd"])
                    if jn1 != 0 and "num_sn" in dst:
                        dst["num_sn"].add(jn1, src["num_sn"])
        # block-block partners (code/mat_vec.f90:3745-3849)
        inb = {}
        k11 = 0
        for i in range(1, sl + 1):
            inb[i] = sum(1 for j in geo.neighbours(i) if geo.region(j) == 3)
            if geo.nleg11.get(el, 0) < geo.nleg11.get(sl, 0):
                inb[i] = 0
            if inb[i]:
                k11 += 1
        cbb1 = k11
        inb[sl + 1] = 0
        inb[sl + el + 2] = 0
        for i in range(1, el + 1):
            k1 = sum(1 for j in geo.neighbours(geo.nposi_lat[i + sl + 1])
                     if geo.region(j) == 1 and inb.get(j, 0) == 0)
            inb[i + sl + 1] = k1
            if k1:
                k11 += 1
        self.coup_bb = [cbb1, k11 - cbb1]
        self.inb = inb
        self.env_sub_s = {i: {n: DBlock.zeros_like(self.d_env[1][n]) for n in names} for i in range(1, cbb1 + 1)}
        self.sys_sub_s = {i: {n: DBlock.zeros_like(self.d_sys[1][n]) for n in names if n != "elec_down"}
                          for i in range(1, self.coup_bb[1] + 1)}
        jc = 0
        for i in range(1, sl + el + 2):
            if inb.get(i, 0) == 0:
                continue
            ia = geo.nposi_lat[i]
            jc += 1
            for k, ib in geo.bonds(ia):
                r = geo.region(ib)
                jt1 = geo.jt(k, ia) * geo.pint(ia, ib)
                jd1, jn1 = geo.jd(k, ia), geo.jn(k, ia)
                if r == 3 and i <= sl:
                    i1 = geo.inb1[(geo.nposi_dm[ib] - sl - 1, el)]
                    src, dst = self.d_env[i1], self.env_sub_s[jc]
                    if jt1 != 0:
                        dst["elec_up"].add(jt1, src["elec_up"])
                        dst["elec_down"].add(np.conj(jt1), src["elec_down"])
                    if geo.tjmodel and jd1 != 0:
                        dst["spin_sd"].add(jd1, src["spin_sd"])
                    if jn1 != 0 and "num_sn" in dst:
                        dst["num_sn"].add(jn1, src["num_sn"])
                if r == 1 and i > sl + 1 and inb.get(geo.nposi_dm[ib], 0) == 0:
                    i1 = geo.inb1[(ib, sl)]
                    src, dst = self.d_sys[i1], self.sys_sub_s[jc - cbb1]
                    if jt1 != 0:
                        dst["elec_up"].add(np.conj(jt1), src["elec_up"])
                    if geo.tjmodel and jd1 != 0:
                        dst["spin_sd"].add(jd1, src["spin_sd"])
                    if jn1 != 0 and "num_sn" in dst:
                        dst["num_sn"].add(jn1, src["num_sn"])

    # ------------------------------------------------------- model_wave
    def model_wave_terms(self):
        """The term kernels model_wave calls, in its order (code/mat_vec.f90:3502-3615)."""
        geo, st, sl, el = self.geo, self.d_st, self.sys.len, self.env.len
        T = []
        T.append(Term(_lib.BLOCK_VEC_DIA, self.d_sys_ham))
        T.append(Term(_lib.VEC_BLOCK_DIA, self.d_env_ham))
        is_, js = geo.nposi_lat[sl + 1], geo.nposi_lat[sl + el + 2]
        if geo.hubbard(is_) != 0.0:
            T.append(Term(_lib.SITE_VEC_SITE_DIA, st["double"], st["si"], coef=geo.hubbard(is_)))
        if geo.hubbard(js) != 0.0:
            T.append(Term(_lib.SITE_VEC_SITE_DIA, st["si"], st["double"], coef=geo.hubbard(js)))
        ii = geo.neiba(is_, js)
        if ii:
            coefx = geo.jt(ii, is_) * geo.pint(is_, js)
            jd1, jn1 = geo.jd(ii, is_), geo.jn(ii, is_)
            if coefx != 0:
                T.append(Term(_lib.SITE_VEC_SITE_NDIA, st["elec_up"], st["elec_down"], F, F, 0, 1, coefx))
            if jd1 != 0:
                T.append(Term(_lib.SITE_VEC_SITE_NDIA, st["sd"], st["sd"], B, B, 0, 0, jd1))
            if jn1 != 0:
                T.append(Term(_lib.SITE_VEC_SITE_DIA, st["num_elec"], st["num_elec"], coef=jn1))
        cb = self.coup_bs
        if cb[0][0]:
            s = self.sys_snc[0]
            T.append(Term(_lib.BLOCK_SITE_VEC_NDIA, s["elec_up"], st["elec_down"], F, F, 0, 1))
            if geo.tjmodel:
                T.append(Term(_lib.BLOCK_SITE_VEC_NDIA, s["spin_sd"], st["sd"], B, B))
            if geo.v123:
                T.append(Term(_lib.BLOCK_SITE_VEC_DIA, s["num_sn"], st["num_elec"]))
        if cb[0][1]:
            s = self.sys_snc[1]
            T.append(Term(_lib.BLOCK_VEC_SITE_NDIA, s["elec_up"], st["elec_down"], F, F, 0, 1))
            if geo.tjmodel:
                T.append(Term(_lib.BLOCK_VEC_SITE_NDIA, s["spin_sd"], st["sd"], B, B))
            if geo.v123:
                T.append(Term(_lib.BLOCK_VEC_SITE_DIA, s["num_sn"], st["num_elec"]))
        if cb[1][0]:
            e = self.env_snc[0]
            T.append(Term(_lib.SITE_VEC_BLOCK_NDIA, st["elec_up"], e["elec_down"], F, F, 0, 1))
            if geo.tjmodel:
                T.append(Term(_lib.SITE_VEC_BLOCK_NDIA, st["sd"], e["spin_sd"], B, B, 0, 1))
            if geo.v123:
                T.append(Term(_lib.SITE_VEC_BLOCK_DIA, st["num_elec"], e["num_sn"]))
        if cb[1][1]:
            e = self.env_snc[1]
            T.append(Term(_lib.VEC_BLOCK_SITE_NDIA, e["elec_up"], st["elec_down"], F, F, 0, 1))
            if geo.tjmodel:
                T.append(Term(_lib.VEC_BLOCK_SITE_NDIA, e["spin_sd"], st["sd"], B, B))
            if geo.v123:
                T.append(Term(_lib.VEC_BLOCK_SITE_DIA, e["num_sn"], st["num_elec"]))
        jc = 0
        for i in range(1, sl + el + 2):
            if self.inb.get(i, 0) == 0:
                continue
            jc += 1
            if i <= sl:
                a = self.d_sys[geo.inb1[(i, sl)]]
                b = self.env_sub_s[jc]
            else:
                a = self.sys_sub_s[jc - self.coup_bb[0]]
                b = self.d_env[geo.inb1[(i - sl - 1, el)]]
            T.append(Term(_lib.BLOCK_VEC_BLOCK_NDIA, a["elec_up"], b["elec_down"], F, F, 0, 1))
            if geo.tjmodel:
                T.append(Term(_lib.BLOCK_VEC_BLOCK_NDIA, a["spin_sd"], b["spin_sd"], B, B, 0, 1))
            if geo.v123:
                T.append(Term(_lib.BLOCK_VEC_BLOCK_DIA, a["num_sn"], b["num_sn"]))
        return T

    def _make_plan(self, terms):
        arr = (_lib.HHTerm * max(1, len(terms)))()
        for k, t in enumerate(terms):
            arr[k] = _lib.HHTerm(t.kind, t.flag0, t.flag1, t.trans0, t.trans1, t.op0.h,
                                 t.op1.h if t.op1 is not None else None, t.coef.real, t.coef.imag)
        h = C.c_void_p()
        self.dev.check(self.dev.lib.hh_plan_create(self.dev.h, self.d_sys_bs.h, self.d_env_bs.h, self.w_in.h,
                                                   len(terms), arr, C.byref(h)))
        return h

    def stats(self):
        c = np.zeros(_lib.HH_PLAN_STATS)
        self.dev.check(self.dev.lib.hh_plan_stats(self.plan, c.ctypes.data_as(C.POINTER(C.c_double))))
        keys = ["ref_flops", "exec_flops", "tiles", "segments", "stage1", "scratch_bytes", "op_bytes",
                "wave_bytes", "exec_flops_s1", "exec_flops_s2", "ref_flops_first", "ref_flops_rest",
                "tc_flops_s1", "tc_flops_s2", "tc_image_bytes", "tc_ready", "fp64_launches", "tc_launches",
                "fp64_work_tiles", "tc_stage1_persistent"]
        return dict(zip(keys, c.tolist()))

    def matvec(self, w_in: DWave, w_out: DWave, precision=None):
        p = self.precision if precision is None else precision
        self.dev.check(self.dev.lib.hh_matvec(self.plan, w_in.h, w_out.h, int(p)))

    def model_wave(self, invec: Wavefunction, precision=None) -> Wavefunction:
        """outvec = H invec (model_wave, code/mat_vec.f90:3476) through host buffers."""
        z = invec.flat()
        out = np.zeros_like(z)
        p = self.precision if precision is None else precision
        zin = np.ascontiguousarray(z)
        self.dev.check(self.dev.lib.hh_matvec_host(self.plan, zin.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                                   out.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)), int(p)))
        w = Wavefunction(invec.sys_len, invec.env_len,
                         [type(s)(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down, s.vec.copy())
                          for s in invec.subs])
        return w.set_flat(out)

    def lanczos_memo_new(self, eigvec: Wavefunction, lanzero, maxit=100, precision=None):
        """Ground state (lanczos_memo_new, code/lanczos.f90:4): returns (E0, iterations, eigvec)."""
        p = self.precision if precision is None else precision
        self.w_in.upload(eigvec.flat())
        e = C.c_double()
        it = C.c_int()
        self.dev.check(self.dev.lib.hh_lanczos(self.plan, self.w_in.h, float(lanzero), int(maxit), int(p),
                                               C.byref(e), C.byref(it)))
        eigvec.set_flat(self.w_in.download())
        return e.value, it.value, eigvec

    def lanczos_device(self, psi, lanzero, maxit=100, precision=None):
        """lanczos_memo_new on a device-resident wave (DWave), in place: returns (E0, iterations)."""
        p = self.precision if precision is None else precision
        e = C.c_double()
        it = C.c_int()
        self.dev.check(self.dev.lib.hh_lanczos(self.plan, psi.h, float(lanzero), int(maxit), int(p),
                                               C.byref(e), C.byref(it)))
        return e.value, it.value

    def free(self):
        if getattr(self, "plan", None) is not None and self.dev.h is not None:
            self.dev.lib.hh_plan_free(self.plan)
        self.plan = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
