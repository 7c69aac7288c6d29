"""Test helpers: run the oracle DMRG and convert its objects to the product's types."""
import numpy as np

from oracle.lattice import Lattice
from oracle.dmrg import DMRG
from oracle.matvec import hmerge, model_wave
from oracle.sites import SiteOps

from hofstadter_hubbard_tsc_gb300 import types as T
from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice


def block(ob):
    return T.TotalBlock(ob.len, ob.up_dif, ob.down_dif,
                        [T.SubBlock(s.num_up, s.num_down, s.down_dif, s.mat.copy()) for s in ob.subs])


def basis(obs):
    b = T.TotalBasis(obs.len)
    for sec in obs.sectors:
        b.sectors.append(T.BasisMap(sec.new_num_up, sec.new_num_down,
                                    [T.SubBasisMap(x.spos, x.sdim, x.bl_num_up, x.bl_num_down,
                                                   x.st_num_up, x.st_num_down) for x in sec.subs]))
    return b


def model(om):
    return T.TotalModel(om.len, block(om.ham), {i: {n: block(b) for n, b in d.items()}
                                               for i, d in om.sub.items()})


def superbasis(osup):
    return T.SuperBasis(osup.sys_len, osup.env_len,
                        [T.SuperSector(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down,
                                       s.sys_dim, s.env_dim) for s in osup.subs])


def wave(ow):
    return T.Wavefunction(ow.sys_len, ow.env_len,
                          [T.SubWave(w.sys_num_up, w.sys_num_down, w.env_num_up, w.env_num_down, w.vec.copy())
                           for w in ow.subs])


def product_lattice(olat):
    return SquareLattice(olat.W, olat.L, model=olat.model, t=olat.t, U=olat.U, J=olat.J, phi=olat.phi)


def record_superblocks(W, L, n_elec, m, U=8.0, phi=0.25, model="hubbard", J=0.0, sweeps=1, seed=7):
    """Run the oracle DMRG and keep every superblock it solved."""
    lat = Lattice(W, L, model=model, U=U, phi=phi, J=J, t=1.0)
    d = DMRG(lat, n_elec, kept_min=m, kept_max=m, trun_err=1e-14, lanzero=1e-11, seed=seed)
    d.record = []
    d.run(sweeps=sweeps)
    return lat, d


def oracle_hpsi(rec, st, psi):
    """model_wave of the oracle on one recorded superblock."""
    sys, env, sys_bs, env_bs, geo, sup, _ = rec
    # hmerge mutates the models: work on copies
    s2, e2 = copy_model(sys), copy_model(env)
    hmerge(s2, e2, geo)
    out = psi.zeros_like()
    model_wave(s2, e2, sys_bs, env_bs, psi, out, geo, st)
    return out


def copy_model(m):
    from oracle.enlarge import Model
    c = Model(m.len, m.ham.copy())
    c.sub = {k: {n: b.copy() for n, b in v.items()} for k, v in m.sub.items()}
    return c


def random_wave(sup_oracle, seed):
    from oracle.blocks import allocate_wave, wave_initialize
    w = allocate_wave(sup_oracle)
    wave_initialize(w, np.random.default_rng(seed))
    return w
