"""Two-block finite DMRG driver (code/warm_up.f90:1284-2170, code/quantum.f90:179-288).

Restates ``warm_up_point``, ``left_to_right``, ``right_to_left`` and the
wavefunction transformations ``wave_trans_LR/RL``.  Models, truncations and
bases that the reference writes to disk per length are kept in dictionaries.
Random start vectors come from a seeded generator (the reference's
``random_number`` is unseeded).
"""
import numpy as np

from .blocks import (get_basis, get_super_basis, allocate_wave, wave_initialize,
                     wave_normalize, SU)
from .density import (get_density_matrix_sys, get_density_matrix_env,
                      get_truncation_operator, identity_truncation)
from .enlarge import Model, get_hamiltonian
from .lanczos import lanczos_memo_new
from .matvec import hmerge, model_wave
from .sites import SiteOps


def wave_trans_lr(sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave):
    """Guess for the next L->R step (code/warm_up.f90:1855-2012).

    ``env_bs`` is the basis in which the previous env block (length l_e) was
    built, ``env_trun`` its truncation; ``sys_trun`` truncates the current sys
    enlarged block.  new = coef * T_sys^H psi_sub T_env^H re-blocked.
    """
    for ow in old_wave.subs:
        st_id = sys_trun.find(ow.sys_num_up, ow.sys_num_down)
        if st_id is None:
            continue
        esec = env_bs.find(ow.env_num_up, ow.env_num_down)
        if esec is None:
            continue
        for x in esec.subs:
            su, sd = x.st_num_up, x.st_num_down
            neu, ned = x.bl_num_up, x.bl_num_down
            old_pos, old_sub_dim = x.spos, x.sdim
            et_id = env_trun.find(neu, ned)
            for nsd in range(abs(ow.sys_num_down - sd), ow.sys_num_down + sd + 1, SU):
                nsu = ow.sys_num_up + su
                ssec = sys_bs.find(nsu, nsd)
                y = ssec.find_full(ow.sys_num_up, ow.sys_num_down, su, sd) if ssec else None
                nw = new_wave.find(nsu, nsd, neu, ned)
                if et_id is None or y is None or nw is None:
                    continue
                j12, j3, j4, j123, j34 = ow.sys_num_down, sd, ned, nsd, ow.env_num_down
                c = (-1.0) ** ((j12 + j3 + j123) // 2) / np.sqrt((1.0 + j12) * (1.0 + j123))
                if c != 0.0:
                    c *= np.sqrt((1.0 + j123) * (j34 + 1.0))
                    if ((j12 + j3 + j4) // 2) % 2 != 0:
                        c = -c
                    if ((j3 + j4 - j34) // 2) % 2 != 0:
                        c = -c
                    T = sys_trun.subs[st_id].mat
                    E = env_trun.subs[et_id].mat
                    sub = c * (np.conj(T).T @ ow.vec[:, old_pos:old_pos + old_sub_dim])
                    nv = new_wave.subs[nw].vec
                    nv[y.spos:y.spos + y.sdim, :] += sub @ np.conj(E).T
    wave_normalize(new_wave)


def wave_trans_rl(sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave):
    """Guess for the next R->L step (code/warm_up.f90:2016-2170)."""
    for ow in old_wave.subs:
        et_id = env_trun.find(ow.env_num_up, ow.env_num_down)
        if et_id is None:
            continue
        ssec = sys_bs.find(ow.sys_num_up, ow.sys_num_down)
        if ssec is None:
            continue
        for x in ssec.subs:
            sd, su = x.st_num_down, x.st_num_up
            nsu, nsd = x.bl_num_up, x.bl_num_down
            for ned in range(abs(ow.env_num_down - sd), ow.env_num_down + sd + 1, SU):
                neu = ow.env_num_up + su
                old_pos, old_sub_dim = x.spos, x.sdim
                st_id = sys_trun.find(nsu, nsd)
                esec = env_bs.find(neu, ned)
                y = esec.find_full(ow.env_num_up, ow.env_num_down, su, sd) if esec else None
                nw = new_wave.find(nsu, nsd, neu, ned)
                if st_id is None or y is None or nw is None:
                    continue
                j12, j3, j4, j123, j34 = ow.env_num_down, sd, nsd, ned, ow.sys_num_down
                c = (-1.0) ** ((j34 + j4 + j3) // 2) / np.sqrt((1.0 + j12) * (1.0 + j4))
                if c != 0.0:
                    c *= np.sqrt((1.0 + j123) * (j34 + 1.0))
                    if ((j4 + j3 + j12) // 2) % 2 != 0:
                        c = -c
                    if ((j12 + j3 - j123) // 2) % 2 != 0:
                        c = -c
                    T = sys_trun.subs[st_id].mat
                    E = env_trun.subs[et_id].mat
                    sub = c * (T @ ow.vec[old_pos:old_pos + old_sub_dim, :])
                    nv = new_wave.subs[nw].vec
                    nv[:, y.spos:y.spos + y.sdim] += sub @ E
    wave_normalize(new_wave)


class DMRG:
    """Finite two-block DMRG of one lattice with the reference's schedule."""

    def __init__(self, lattice, n_elec, kept_min, kept_max, trun_err=1e-18,
                 lanzero=1e-10, seed=20261203, verbose=False):
        self.lat = lattice
        self.st = SiteOps("tj" if lattice.tjmodel else "hubbard")
        self.n_elec = n_elec
        self.kept_min, self.kept_max = kept_min, kept_max
        self.trun_err = trun_err
        self.lanzero = lanzero
        self.rng = np.random.default_rng(seed)
        self.sys_models, self.env_models = {}, {}
        self.sys_truns, self.env_truns = {}, {}
        self.sys_bases, self.env_bases = {}, {}
        self.wave = None
        self.energies = []
        self.verbose = verbose
        self.last_step = None   # (sys, env, sys_bs, env_bs, geo, wave) of the last solve
        self.record = None      # optional list: (sys, env, sys_bs, env_bs, geo, sup, start wave) per solve

    # ---------------------------------------------------------------------
    def _site_model(self, geo, lat_idx):
        ham = self.st.site_ham(geo.hubbard(lat_idx))
        m = Model(1, ham)
        d = {"elec_up": self.st.elec_up.copy(), "elec_down": self.st.elec_down.copy()}
        if geo.tjmodel:
            d["spin_sd"] = self.st.sd.copy()
        if geo.v123:
            d["num_sn"] = self.st.num_elec.copy()
        m.sub[1] = d
        return m

    def _copy_model(self, m):
        c = Model(m.len, m.ham.copy())
        c.sub = {k: {n: b.copy() for n, b in v.items()} for k, v in m.sub.items()}
        return c

    def solve(self, sys, env, sys_bs, env_bs, geo, sup, guess):
        if self.record is not None:
            self.record.append((self._copy_model(sys), self._copy_model(env), sys_bs, env_bs,
                                self.lat.geometry(sys.len, env.len), sup, guess.copy()))
        hmerge(sys, env, geo)

        def apply_h(v, out):
            model_wave(sys, env, sys_bs, env_bs, v, out, geo, self.st)

        e0, it = lanczos_memo_new(apply_h, guess, self.lanzero)
        self.energies.append((sys.len, env.len, e0, it))
        self.last_step = (sys, env, sys_bs, env_bs, geo, guess)
        if self.verbose:
            print(f"  sys={sys.len} env={env.len} dim={sup.dim} E0={e0:.12f} it={it}")
        return e0

    # ---------------------------------------------------------------------
    def warm_up(self):
        """warm_up_point(1, N/2) (code/warm_up.f90:1284-1491)."""
        N = self.lat.N
        geo = self.lat.geometry(1, 1)
        sys = self._site_model(geo, 1)
        env = self._site_model(geo, geo.nposi_lat[3])
        self.sys_models[1] = self._copy_model(sys)
        self.env_models[1] = self._copy_model(env)
        label = 1
        while label + 1 <= N // 2:
            sys_bs = get_basis(sys.ham, self.st.sz)
            env_bs = get_basis(env.ham, self.st.sz)
            geo = self.lat.geometry(sys.len, env.len)
            tot_up = int(1.0 * (sys_bs.len + env_bs.len) / N * self.n_elec + 0.001)
            tot_up -= tot_up % 2
            tot_up = min(tot_up, self.n_elec)
            sup = get_super_basis(sys_bs, env_bs, tot_up, 0)
            wv = allocate_wave(sup)
            wave_initialize(wv, self.rng)
            self.solve(sys, env, sys_bs, env_bs, geo, sup, wv)
            sys_den = get_density_matrix_sys(wv)
            env_den = get_density_matrix_env(wv)
            if sys_bs.dim <= self.kept_max:
                strun = identity_truncation(sys_bs)
            else:
                strun = get_truncation_operator(sys_den, self.kept_min, self.kept_max, self.trun_err)[0]
            get_hamiltonian(sys, sys_bs, strun, geo, self.st, "sys", 0)
            if env_bs.dim <= self.kept_max:
                etrun = identity_truncation(env_bs)
            else:
                etrun = get_truncation_operator(env_den, self.kept_min, self.kept_max, self.trun_err)[0]
            get_hamiltonian(env, env_bs, etrun, geo, self.st, "env", sys.len)
            self.sys_models[label + 1] = self._copy_model(sys)
            self.env_models[label + 1] = self._copy_model(env)
            self.sys_truns[label + 1], self.env_truns[label + 1] = strun, etrun
            self.sys_bases[label + 1], self.env_bases[label + 1] = sys_bs, env_bs
            self.wave = wv
            label += 1

    def left_to_right(self, bg_id, end_id, restart_wave=True):
        """left_to_right (code/warm_up.f90:1495-1671)."""
        N = self.lat.N
        label = bg_id
        sys = self._copy_model(self.sys_models[label])
        env = self._copy_model(self.env_models[N - label - 2])
        geo = self.lat.geometry(sys.len, env.len)
        sys_bs = get_basis(sys.ham, self.st.sz)
        env_bs = get_basis(env.ham, self.st.sz)
        sup = get_super_basis(sys_bs, env_bs, self.n_elec, 0)
        wv = allocate_wave(sup)
        if (not restart_wave or self.wave is None or self.wave.sys_len != sys_bs.len
                or self.wave.env_len != env_bs.len):
            if self.wave is not None and restart_wave and self.wave.sys_len != sys_bs.len:
                wave_trans_lr(sys_bs, self.env_bases[N - label], self.sys_truns[label],
                              self.env_truns[N - label - 1], self.wave, wv)
            else:
                wave_initialize(wv, self.rng)
        else:
            wv = self.wave
        self.solve(sys, env, sys_bs, env_bs, geo, sup, wv)
        sys_den = get_density_matrix_sys(wv)
        strun, ns, err, ent, _ = get_truncation_operator(sys_den, self.kept_min, self.kept_max, self.trun_err)
        get_hamiltonian(sys, sys_bs, strun, geo, self.st, "sys", 0)
        self.sys_models[label + 1] = self._copy_model(sys)
        self.sys_truns[label + 1] = strun
        self.sys_bases[label + 1] = sys_bs
        self.wave = wv
        label += 1
        while label + 1 <= end_id:
            sys_bs = get_basis(sys.ham, self.st.sz)
            env_bs = self.env_bases[N - label - 1]
            env_basis = self.env_bases[N - label]
            env = self._copy_model(self.env_models[N - label - 2])
            geo = self.lat.geometry(sys.len, env.len)
            sup = get_super_basis(sys_bs, env_bs, self.n_elec, 0)
            etrun = self.env_truns[N - label - 1]
            wv = allocate_wave(sup)
            wave_trans_lr(sys_bs, env_basis, strun, etrun, self.wave, wv)
            self.solve(sys, env, sys_bs, env_bs, geo, sup, wv)
            sys_den = get_density_matrix_sys(wv)
            strun, ns, err, ent, _ = get_truncation_operator(sys_den, self.kept_min, self.kept_max, self.trun_err)
            get_hamiltonian(sys, sys_bs, strun, geo, self.st, "sys", 0)
            self.sys_models[label + 1] = self._copy_model(sys)
            self.sys_truns[label + 1] = strun
            self.sys_bases[label + 1] = sys_bs
            self.wave = wv
            label += 1

    def right_to_left(self, bg_id, end_id):
        """right_to_left (code/warm_up.f90:1675-1849)."""
        N = self.lat.N
        label = bg_id
        sys = self._copy_model(self.sys_models[label - 1])
        env = self._copy_model(self.env_models[N - label - 1])
        geo = self.lat.geometry(sys.len, env.len)
        sys_bs = get_basis(sys.ham, self.st.sz)
        env_bs = get_basis(env.ham, self.st.sz)
        sup = get_super_basis(sys_bs, env_bs, self.n_elec, 0)
        wv = allocate_wave(sup)
        if self.wave is not None and self.wave.sys_len != sys_bs.len:
            wave_trans_rl(self.sys_bases[label + 1], env_bs, self.sys_truns[label],
                          self.env_truns[N - label - 1], self.wave, wv)
        elif self.wave is not None and self.wave.sys_len == sys_bs.len:
            wv = self.wave
        else:
            wave_initialize(wv, self.rng)
        self.solve(sys, env, sys_bs, env_bs, geo, sup, wv)
        env_den = get_density_matrix_env(wv)
        etrun, ns, err, ent, _ = get_truncation_operator(env_den, self.kept_min, self.kept_max, self.trun_err)
        get_hamiltonian(env, env_bs, etrun, geo, self.st, "env", sys.len + 1)
        self.env_models[N - label] = self._copy_model(env)
        self.env_truns[N - label] = etrun
        self.env_bases[N - label] = env_bs
        self.wave = wv
        label -= 1
        while label - 1 >= end_id:
            sys_bs = self.sys_bases[label]
            sys_basis = self.sys_bases[label + 1]
            env_bs = get_basis(env.ham, self.st.sz)
            sup = get_super_basis(sys_bs, env_bs, self.n_elec, 0)
            sys = self._copy_model(self.sys_models[label - 1])
            geo = self.lat.geometry(sys.len, env.len)
            strun = self.sys_truns[label]
            wv = allocate_wave(sup)
            wave_trans_rl(sys_basis, env_bs, strun, etrun, self.wave, wv)
            self.solve(sys, env, sys_bs, env_bs, geo, sup, wv)
            env_den = get_density_matrix_env(wv)
            etrun, ns, err, ent, _ = get_truncation_operator(env_den, self.kept_min, self.kept_max, self.trun_err)
            get_hamiltonian(env, env_bs, etrun, geo, self.st, "env", sys.len + 1)
            self.env_models[N - label] = self._copy_model(env)
            self.env_truns[N - label] = etrun
            self.env_bases[N - label] = env_bs
            self.wave = wv
            label -= 1

    def run(self, sweeps=2):
        """Get_Ground_State schedule (code/quantum.f90:179-288) with trun_idx=1."""
        N = self.lat.N
        self.warm_up()
        idx1 = 1
        self.left_to_right(N // 2 - 1, N - idx1 - 1)
        self.right_to_left(N - idx1 - 1, idx1)
        for _ in range(sweeps):
            self.left_to_right(idx1, N - idx1 - 1)
            self.right_to_left(N - idx1 - 1, idx1)
        return self.energies[-1][2]
