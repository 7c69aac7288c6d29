"""Finite two-block DMRG with every block operation on the GPU.

The host side mirrors the reference's driver (warm_up_point, left_to_right,
right_to_left, Get_Ground_State; code/warm_up.f90:1284-1849, code/quantum.f90:
179-288) and its enlargement routine (Get_Hamiltonian_Sys/Env, code/get_ham.f90:
4-659): it decides which operator goes where; libhh_dmrg.so does the work.
Models, truncations and waves stay in device memory between steps, where the
reference writes them to disk per length.
"""
import ctypes as C
import json
import os
import time
from collections import defaultdict
from contextlib import contextmanager

import numpy as np

from . import _lib
from .device import DBlock, DBasis, DWave
from .sites import SiteOperators
from .step import density_truncate, update_trun, wave_trans, SYS, ENV
from .superblock import Superblock
from .types import TotalBlock, SubBlock, TotalModel, SuperBasis, SuperSector, Wavefunction, get_basis, get_super_basis
from . import disk

F, B = ord("F"), ord("B")


class GModel:
    """Total_Model on the device: Hamiltonian and the boundary operators."""

    def __init__(self, length, ham, sub=None):
        self.len = length
        self.ham = ham
        self.sub = dict(sub or {})

    def copy(self):
        return GModel(self.len, self.ham, {i: dict(d) for i, d in self.sub.items()})


def _sector_block(dblk):
    """A host TotalBlock listing only the sectors of a device block (for Get_basis)."""
    return TotalBlock(dblk.len, 0, 0, [SubBlock(int(q[0]), int(q[1]), int(q[2]), np.zeros((int(q[3]), int(q[4]))))
                                       for q in dblk.qn])


class GPUDMRG:
    def __init__(self, dev, lattice, n_elec, kept_min, kept_max, trun_err=1e-18, lanzero=1e-10,
                 precision=_lib.HH_PREC_FP64, seed=20261203, maxit=100, guess_hook=None, verbose=False):
        self.dev, self.lat = dev, lattice
        self.n_elec = n_elec
        self.kept_min, self.kept_max = kept_min, kept_max
        self.trun_err, self.lanzero, self.precision, self.maxit = trun_err, lanzero, precision, maxit
        self.seed = seed
        self.st = SiteOperators("tj" if lattice.tjmodel else "hubbard")
        self.d_st = {n: DBlock.upload(dev, getattr(self.st, n))
                     for n in ("elec_up", "elec_down", "num_elec", "double", "sd", "si")}
        self.sz_host = self.st.sz
        self.sys_models, self.env_models = {}, {}
        self.sys_truns, self.env_truns = {}, {}
        self.sys_bases, self.env_bases = {}, {}
        self.wave = None          # (DWave, sys_len, env_len)
        self.energies = []        # (sys_len, env_len, E0, iterations, seconds)
        self.guess_hook = guess_hook
        self.verbose = verbose
        self._nrand = 0
        self.guess_kind = "random"     # how the next Lanczos start vector was made
        self.phase_s = defaultdict(float)   # host wall seconds per phase of a step

    @property
    def _block_precision(self):
        """Arithmetic of the block renormalisations T^H O T: FP64 in an FP64
        run (the reference's), double-float (FP64-class, on the FP32 pipe) in
        a split-precision run."""
        return _lib.HH_PREC_FP64 if self.precision == _lib.HH_PREC_FP64 else _lib.HH_PREC_FP32X2

    @contextmanager
    def _phase(self, name):
        """Host wall time of a phase, its device work included: the phase's
        queued kernels are waited for at its end, so that work queued without a
        wait (enlargement, renormalisation) is not billed to the next phase."""
        t0 = time.perf_counter()
        try:
            yield
        finally:
            self.dev.sync()
            self.phase_s[name] += time.perf_counter() - t0

    # ------------------------------------------------------------------ setup
    def _site_model(self, geo, lat_idx):
        u = geo.hubbard(lat_idx)
        h = DBlock.upload(self.dev, self.st.site_ham(u) if hasattr(self.st, "site_ham") else self._site_ham(u))
        d = {"elec_up": self.d_st["elec_up"], "elec_down": self.d_st["elec_down"]}
        if geo.tjmodel:
            d["spin_sd"] = self.d_st["sd"]
        if geo.v123:
            d["num_sn"] = self.d_st["num_elec"]
        return GModel(1, h, {1: d})

    def _site_ham(self, u):
        return TotalBlock(1, 0, 0, [SubBlock(s.num_up, s.num_down, 0, u * s.mat) for s in self.st.double.subs])

    def _basis(self, model):
        with self._phase("basis"):
            b = get_basis(_sector_block(model.ham), self.sz_host)
            return b, DBasis(self.dev, b)

    def _super(self, sys_bs, env_bs, tot_up, tot_down):
        with self._phase("basis"):
            return get_super_basis(sys_bs, env_bs, tot_up, tot_down)

    def _new_wave(self, sup):
        return DWave(self.dev, sup.array(), sup.sys_len, sup.env_len)

    def _random_wave(self, sup):
        w = self._new_wave(sup)
        self._nrand += 1
        self.dev.check(self.dev.lib.hh_wave_random(w.h, C.c_ulonglong(self.seed * 1000003 + self._nrand)))
        return w

    # --------------------------------------------------------- enlargement
    def _enlarge(self, pre, basis, dbasis, trun, geo, side, mshift):
        """Get_Hamiltonian_Sys (side 'sys') / Get_Hamiltonian_Env ('env') on the device."""
        with self._phase("enlarge"):
            return self._enlarge_impl(pre, basis, dbasis, trun, geo, side, mshift)

    def _enlarge_impl(self, pre, basis, dbasis, trun, geo, side, mshift):
        dev, lat, st = self.dev, self.lat, self.d_st
        sd = 0 if side == "sys" else 1

        def embed(mode, op, flag=B):
            h = C.c_void_p()
            dev.check(dev.lib.hh_enlarge_operator(dev.h, mode, op.h, dbasis.h, flag, sd, C.byref(h)))
            return DBlock.from_handle(dev, h)

        def add_bond(ham, blk, site, trans, coef, flag, flags):
            c = np.array([complex(coef).real, complex(coef).imag])
            dev.check(dev.lib.hh_ham_add_bond(dev.h, ham.h, blk.h, site.h, trans, dbasis.h,
                                              c.ctypes.data_as(C.POINTER(C.c_double)), flag, flags))

        next_ham = embed(0, pre.ham)
        L = pre.len
        jlat = L + 1 if side == "sys" else geo.nposi_lat[L + 1 + mshift]
        bonds = []
        for kdir, I in geo.bonds(jlat):
            II = I if side == "sys" else geo.nposi_dm.get(I, 0) - mshift
            if 0 < II <= L:
                i1 = lat.inb1.get((II, L), 10000)
                if 0 < i1 <= lat.nleg11.get(L, 0):
                    bonds.append((kdir, I, i1))
        ijs = ([1, 3] + ([5] if geo.v123 else [])) if geo.tjmodel else ([1, 6] + ([5] if geo.v123 else []))
        next_sub = {}
        for ij in ijs:
            names = {1: ["elec_up", "elec_down"], 3: ["spin_sd"], 5: ["num_sn"], 6: []}[ij]
            for kdir, I, i1 in bonds:
                coefx = np.conj(geo.jt(kdir, jlat) * geo.pint(jlat, I))
                coefsd = geo.jd(kdir, jlat)
                if ij == 1 and coefx != 0:
                    if side == "sys":
                        add_bond(next_ham, pre.sub[i1]["elec_up"], st["elec_down"], 1, coefx, F, ord("S"))
                    else:
                        add_bond(next_ham, pre.sub[i1]["elec_down"], st["elec_up"], 1, coefx, F, ord("E"))
                if ij == 3 and coefsd != 0:
                    add_bond(next_ham, pre.sub[i1]["spin_sd"], st["sd"], 0, coefsd, B,
                             ord("S") if side == "sys" else ord("E"))
            for y in range(1, L + 1):
                i1 = lat.inb1.get((y, L), 10000)
                if i1 <= lat.nleg11.get(L, 0):
                    d = next_sub.setdefault(i1, {})
                    for nm in names:
                        d[nm] = embed(0, pre.sub[i1][nm]) if ij == 5 else embed(2, pre.sub[i1][nm], F if ij == 1 else B)
            tmp = {}
            if ij == 1:
                tmp["elec_up"] = embed(3, st["elec_up"], F)
                tmp["elec_down"] = embed(3, st["elec_down"], F)
            elif ij == 3:
                tmp["spin_sd"] = embed(3, st["sd"], B)
            elif ij == 5:
                tmp["num_sn"] = embed(1, st["num_elec"])
            elif ij == 6:
                dbl = embed(1, st["double"])
            if ij == 5:
                for kdir, I, i1 in bonds:
                    cn = geo.jn(kdir, jlat)
                    if cn != 0:
                        c = np.array([complex(cn).real, complex(cn).imag])
                        dev.check(dev.lib.hh_ham_add_product(dev.h, next_ham.h, next_sub[i1]["num_sn"].h,
                                                             tmp["num_sn"].h, c.ctypes.data_as(C.POINTER(C.c_double))))
            if ij == 6:
                u = geo.hubbard(jlat)
                if u != 0.0:
                    next_ham.add(u, dbl)
            nleg1 = lat.nleg11.get(L + 1, 0)
            for I in range(1, L + 1):
                I1 = lat.inb1.get((I, L), 10000)
                J = lat.inb1.get((I, L + 1), 10000)
                if J <= nleg1 and J != I1:
                    for nm in names:
                        next_sub.setdefault(J, {})[nm] = next_sub[I1][nm]
            j = lat.inb1.get((L + 1, L + 1), 10000)
            for nm in names:
                if j <= nleg1:
                    next_sub.setdefault(j, {})[nm] = tmp[nm]
            for ii in range(1, nleg1 + 1):
                dst = pre.sub.setdefault(ii, {})
                for nm in names:
                    dst[nm] = update_trun(dev, next_sub[ii][nm], trun, dia=(ij == 5), precision=self._block_precision)
        for ii in list(pre.sub.keys()):
            if ii > lat.nleg11.get(L + 1, 0):
                del pre.sub[ii]
        pre.ham = update_trun(dev, next_ham, trun, dia=True, precision=self._block_precision)
        pre.len = L + 1
        return pre

    # ---------------------------------------------------------------- solve
    def _solve(self, sys, env, sys_bs, env_bs, geo, sup, psi):
        t0 = time.perf_counter()
        with self._phase("plan"):
            sb = Superblock(self.dev, sys, env, sys_bs, env_bs, sup, geo, self.st, precision=self.precision)
        if self.guess_hook is not None:
            with self._phase("guess"):
                self.guess_hook(self, sb, psi, "before")
        with self._phase("lanczos"):
            e0, it = sb.lanczos_device(psi, self.lanzero, self.maxit)
        if self.guess_hook is not None:
            with self._phase("guess"):
                self.guess_hook(self, sb, psi, "after")
        with self._phase("plan"):
            sb.free()
        dt = time.perf_counter() - t0
        self.energies.append((sys.len, env.len, e0, it, dt))
        if self.verbose:
            print(f"  sys={sys.len} env={env.len} dim={sup.dim} E0={e0:.12f} it={it} {dt:.3f}s")
        return e0

    def _trun(self, wave, side, basis, dbasis, force_truncate=False):
        if not force_truncate and basis.dim <= self.kept_max:
            # identity truncation (code/warm_up.f90:1432-1439)
            subs = [SubBlock(s.new_num_up, s.new_num_down, 0, np.eye(s.dim)) for s in basis.sectors]
            return DBlock.upload(self.dev, TotalBlock(basis.len, 0, 0, subs))
        with self._phase("truncate"):
            trun, ns, err, ent, _ = density_truncate(self.dev, wave, side, self.kept_min, self.kept_max,
                                                     self.trun_err)
        self.last_trunc = (ns, err, ent)
        return trun

    def _wave_trans(self, direction, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave):
        """wave_trans_LR / wave_trans_RL: in a split-precision run the
        transformed guess (it only starts Lanczos) is formed with FP32
        arithmetic, in an FP64 run with FP64 as in the reference."""
        wave_trans(self.dev, direction, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave,
                   _lib.HH_PREC_FP64 if self.precision == _lib.HH_PREC_FP64 else _lib.HH_PREC_FP32)

    # ---------------------------------------------------------------- sweeps
    def warm_up(self):
        """warm_up_point(1, N/2) (code/warm_up.f90:1284-1491)."""
        N = self.lat.N
        geo = self.lat.geometry(1, 1)
        sys = self._site_model(geo, 1)
        env = self._site_model(geo, geo.nposi_lat[3])
        self.sys_models[1], self.env_models[1] = sys.copy(), env.copy()
        label = 1
        while label + 1 <= N // 2:
            sys_bs, dsys_bs = self._basis(sys)
            env_bs, denv_bs = self._basis(env)
            geo = self.lat.geometry(sys.len, env.len)
            tot_up = int(1.0 * (sys_bs.len + env_bs.len) / N * self.n_elec + 0.001)
            tot_up -= tot_up % 2
            tot_up = min(tot_up, self.n_elec)
            sup = self._super(sys_bs, env_bs, tot_up, 0)
            wv = self._random_wave(sup)
            self.guess_kind = "random"
            self._solve(sys, env, sys_bs, env_bs, geo, sup, wv)
            strun = self._trun(wv, SYS, sys_bs, dsys_bs)
            etrun = self._trun(wv, ENV, env_bs, denv_bs)
            self._enlarge(sys, sys_bs, dsys_bs, strun, geo, "sys", 0)
            self._enlarge(env, env_bs, denv_bs, etrun, geo, "env", sys.len)
            self.sys_models[label + 1], self.env_models[label + 1] = sys.copy(), env.copy()
            self.sys_truns[label + 1], self.env_truns[label + 1] = strun, etrun
            self.sys_bases[label + 1] = (sys_bs, dsys_bs)
            self.env_bases[label + 1] = (env_bs, denv_bs)
            self.wave = (wv, sup)
            label += 1

    def left_to_right(self, bg_id, end_id):
        """left_to_right (code/warm_up.f90:1495-1671)."""
        N = self.lat.N
        label = bg_id
        sys = self.sys_models[label].copy()
        env = self.env_models[N - label - 2].copy()
        geo = self.lat.geometry(sys.len, env.len)
        sys_bs, dsys_bs = self._basis(sys)
        env_bs, denv_bs = self._basis(env)
        sup = self._super(sys_bs, env_bs, self.n_elec, 0)
        if self.wave is not None and self.wave[1].sys_len == sys_bs.len and self.wave[1].env_len == env_bs.len:
            wv = self.wave[0]
            self.guess_kind = "previous"
        elif self.wave is not None:
            wv = self._new_wave(sup)
            self._wave_trans("LR", dsys_bs, self.env_bases[N - label][1], self.sys_truns[label],
                       self.env_truns[N - label - 1], self.wave[0], wv)
            self.guess_kind = "transformed"
        else:
            wv = self._random_wave(sup)
            self.guess_kind = "random"
        self._solve(sys, env, sys_bs, env_bs, geo, sup, wv)
        strun = self._trun(wv, SYS, sys_bs, dsys_bs, force_truncate=True)
        self._enlarge(sys, sys_bs, dsys_bs, strun, geo, "sys", 0)
        self.sys_models[label + 1], self.sys_truns[label + 1] = sys.copy(), strun
        self.sys_bases[label + 1] = (sys_bs, dsys_bs)
        self.wave = (wv, sup)
        label += 1
        while label + 1 <= end_id:
            sys_bs, dsys_bs = self._basis(sys)
            env_bs, denv_bs = self.env_bases[N - label - 1]
            env = self.env_models[N - label - 2].copy()
            geo = self.lat.geometry(sys.len, env.len)
            sup = self._super(sys_bs, env_bs, self.n_elec, 0)
            wv = self._new_wave(sup)
            with self._phase("transform"):
                self._wave_trans("LR", dsys_bs, self.env_bases[N - label][1], strun,
                           self.env_truns[N - label - 1], self.wave[0], wv)
            self.guess_kind = "transformed"
            self._solve(sys, env, sys_bs, env_bs, geo, sup, wv)
            strun = self._trun(wv, SYS, sys_bs, dsys_bs, force_truncate=True)
            self._enlarge(sys, sys_bs, dsys_bs, strun, geo, "sys", 0)
            self.sys_models[label + 1], self.sys_truns[label + 1] = sys.copy(), strun
            self.sys_bases[label + 1] = (sys_bs, dsys_bs)
            self.wave = (wv, sup)
            label += 1

    def right_to_left(self, bg_id, end_id):
        """right_to_left (code/warm_up.f90:1675-1849)."""
        N = self.lat.N
        label = bg_id
        sys = self.sys_models[label - 1].copy()
        env = self.env_models[N - label - 1].copy()
        geo = self.lat.geometry(sys.len, env.len)
        sys_bs, dsys_bs = self._basis(sys)
        env_bs, denv_bs = self._basis(env)
        sup = self._super(sys_bs, env_bs, self.n_elec, 0)
        if self.wave is not None and self.wave[1].sys_len == sys_bs.len and self.wave[1].env_len == env_bs.len:
            wv = self.wave[0]
            self.guess_kind = "previous"
        elif self.wave is not None:
            wv = self._new_wave(sup)
            self._wave_trans("RL", self.sys_bases[label + 1][1], denv_bs, self.sys_truns[label],
                       self.env_truns[N - label - 1], self.wave[0], wv)
            self.guess_kind = "transformed"
        else:
            wv = self._random_wave(sup)
            self.guess_kind = "random"
        self._solve(sys, env, sys_bs, env_bs, geo, sup, wv)
        etrun = self._trun(wv, ENV, env_bs, denv_bs, force_truncate=True)
        self._enlarge(env, env_bs, denv_bs, etrun, geo, "env", sys.len + 1)
        self.env_models[N - label], self.env_truns[N - label] = env.copy(), etrun
        self.env_bases[N - label] = (env_bs, denv_bs)
        self.wave = (wv, sup)
        label -= 1
        while label - 1 >= end_id:
            sys_bs, dsys_bs = self.sys_bases[label]
            env_bs, denv_bs = self._basis(env)
            sup = self._super(sys_bs, env_bs, self.n_elec, 0)
            sys = self.sys_models[label - 1].copy()
            geo = self.lat.geometry(sys.len, env.len)
            wv = self._new_wave(sup)
            with self._phase("transform"):
                self._wave_trans("RL", self.sys_bases[label + 1][1], denv_bs, self.sys_truns[label], etrun,
                           self.wave[0], wv)
            self.guess_kind = "transformed"
            self._solve(sys, env, sys_bs, env_bs, geo, sup, wv)
            etrun = self._trun(wv, ENV, env_bs, denv_bs, force_truncate=True)
            self._enlarge(env, env_bs, denv_bs, etrun, geo, "env", sys.len + 1)
            self.env_models[N - label], self.env_truns[N - label] = env.copy(), etrun
            self.env_bases[N - label] = (env_bs, denv_bs)
            self.wave = (wv, sup)
            label -= 1

    def sweep(self):
        """One finite sweep: left_to_right then right_to_left (code/quantum.f90:255-256)."""
        N = self.lat.N
        self.left_to_right(1, N - 2)
        self.right_to_left(N - 2, 1)

    def _end_sweep(self):
        """Lets a guess hook with an ``end_sweep`` method (the learned corrector
        trains there) see the finished sweep; runs outside the sweep timer."""
        if self.guess_hook is not None and hasattr(self.guess_hook, "end_sweep"):
            self.guess_hook.end_sweep(self)

    # ------------------------------------------------------------ checkpoints
    def _op_names(self):
        names = ["elec_up", "elec_down"]
        if self.lat.tjmodel:
            names.append("spin_sd")
        if self.lat.v123:
            names.append("num_sn")
        return names

    def save(self, path):
        """Writes the sweep state in the reference's on-disk formats
        (model_to_disk, truns_to_disk, basis_to_disk, wave_to_disk;
        code/space_info.f90:1406-1762), one file per block length and side,
        plus state.json with the driver's bookkeeping."""
        os.makedirs(path, exist_ok=True)
        names = self._op_names()
        state = {"n_elec": self.n_elec, "nrand": self._nrand, "guess_kind": self.guess_kind,
                 "energies": [list(e) for e in self.energies], "models": {}, "truns": {}, "bases": {}}
        for side, models, truns, bases in (("sys", self.sys_models, self.sys_truns, self.sys_bases),
                                           ("env", self.env_models, self.env_truns, self.env_bases)):
            state["models"][side] = {}
            for L, m in models.items():
                tm = TotalModel(m.len, m.ham.download(), {ii: {nm: d[nm].download() for nm in names}
                                                          for ii, d in m.sub.items()})
                disk.model_to_disk(tm, os.path.join(path, f"{side}_model_{L}.dat"), names)
                state["models"][side][str(L)] = len(m.sub)
            for L, t in truns.items():
                disk.truns_to_disk(t.download(), os.path.join(path, f"{side}_trun_{L}.dat"))
            for L, (b, _) in bases.items():
                disk.basis_to_disk(b, os.path.join(path, f"{side}_basis_{L}.dat"))
            state["truns"][side] = sorted(truns)
            state["bases"][side] = sorted(bases)
        if self.wave is not None:
            wv, sup = self.wave
            disk.wave_to_disk(Wavefunction.zeros(sup).set_flat(wv.download()), os.path.join(path, "wave.dat"))
        with open(os.path.join(path, "state.json"), "w") as f:
            json.dump(state, f)

    def load(self, path):
        """Restores a state written by ``save`` (same lattice and parameters)."""
        with open(os.path.join(path, "state.json")) as f:
            state = json.load(f)
        dev, names = self.dev, self._op_names()
        self.energies = [tuple(e) for e in state["energies"]]
        self._nrand, self.guess_kind = state["nrand"], state["guess_kind"]
        for side, models, truns, bases in (("sys", self.sys_models, self.sys_truns, self.sys_bases),
                                           ("env", self.env_models, self.env_truns, self.env_bases)):
            models.clear()
            truns.clear()
            bases.clear()
            for L, nleg in state["models"][side].items():
                tm = disk.model_from_disk(os.path.join(path, f"{side}_model_{L}.dat"), nleg, names)
                models[int(L)] = GModel(tm.len, DBlock.upload(dev, tm.ham),
                                        {ii: {nm: DBlock.upload(dev, b) for nm, b in d.items()}
                                         for ii, d in tm.sub.items()})
            for L in state["truns"][side]:
                truns[L] = DBlock.upload(dev, disk.truns_from_disk(os.path.join(path, f"{side}_trun_{L}.dat")))
            for L in state["bases"][side]:
                b = disk.basis_from_disk(os.path.join(path, f"{side}_basis_{L}.dat"))
                bases[L] = (b, DBasis(dev, b))
        self.wave = None
        wpath = os.path.join(path, "wave.dat")
        if os.path.exists(wpath):
            w = disk.wave_from_disk(wpath)
            sup = SuperBasis(w.sys_len, w.env_len, [SuperSector(s.sys_num_up, s.sys_num_down, s.env_num_up,
                                                                s.env_num_down, s.sys_dim, s.env_dim)
                                                    for s in w.subs])
            dw = self._new_wave(sup)
            dw.upload(w.flat())
            self.wave = (dw, sup)

    def run(self, sweeps=2):
        """Get_Ground_State with trun_idx = 1 (code/quantum.f90:179-288)."""
        N = self.lat.N
        self.warm_up()
        self.left_to_right(N // 2 - 1, N - 2)
        self.right_to_left(N - 2, 1)
        self._end_sweep()
        times = []
        for _ in range(sweeps):
            self.phase_s.clear()
            t0 = time.perf_counter()
            self.sweep()
            times.append(time.perf_counter() - t0)
            self._end_sweep()
        self.sweep_times = times
        return self.energies[-1][2]
