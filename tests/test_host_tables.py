"""Host-side tables of the product agree with the oracle's restatement."""
import numpy as np

from oracle.lattice import Lattice
from oracle.blocks import get_basis as o_get_basis, get_super_basis as o_gsb
from oracle.sites import SiteOps

from hofstadter_hubbard_tsc_gb300 import types as T
from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice
from hofstadter_hubbard_tsc_gb300.sites import SiteOperators
from tests.helpers import block, basis


def test_lattice_tables_match():
    for W, L in [(2, 6), (4, 5), (6, 4)]:
        o = Lattice(W, L, phi=0.25)
        p = SquareLattice(W, L, phi=0.25)
        assert {k: v for k, v in o.inb1.items() if k[1] < o.N - 1} == \
               {k: v for k, v in p.inb1.items() if k[1] < p.N - 1}
        for ns in range(1, o.N - 1):
            assert o.nleg11[ns] == p.nleg11[ns]
        for ns in range(1, o.N - 3):
            go, gp = o.geometry(ns, o.N - ns - 2), p.geometry(ns, p.N - ns - 2)
            assert go.nposi == gp.nposi and go.nposi_lat == gp.nposi_lat and go.nposi_dm == gp.nposi_dm
            for i in range(1, o.N + 1):
                assert go.bonds(i) == gp.bonds(i)
                for _, j in go.bonds(i):
                    assert go.pint(i, j) == gp.pint(i, j)


def test_site_operators_match():
    o, p = SiteOps("hubbard"), SiteOperators("hubbard")
    for n in ("elec_up", "elec_down", "num_elec", "double", "sd", "si"):
        ob, pb = getattr(o, n), getattr(p, n)
        assert (ob.up_dif, ob.down_dif) == (pb.up_dif, pb.down_dif)
        for a, b in zip(ob.subs, pb.subs):
            assert (a.num_up, a.num_down, a.down_dif) == (b.num_up, b.num_down, b.down_dif)
            np.testing.assert_array_equal(a.mat, b.mat)


def test_get_basis_matches():
    st = SiteOps("hubbard")
    rng = np.random.default_rng(1)
    from oracle.blocks import Block, Sub
    ob = Block(5, 0, 0)
    for (n, s) in [(4, 0), (4, 2), (5, 1), (3, 1), (6, 0), (5, 3)]:
        d = int(rng.integers(1, 6))
        ob.subs.append(Sub(n, s, 0, d, d))
    obs = o_get_basis(ob, st.sz)
    pbs = T.get_basis(block(ob), block(st.sz))
    ref = basis(obs)
    assert [(s.new_num_up, s.new_num_down, s.dim) for s in ref.sectors] == \
           [(s.new_num_up, s.new_num_down, s.dim) for s in pbs.sectors]
    for a, b in zip(ref.sectors, pbs.sectors):
        assert [(x.spos, x.sdim, x.bl_num_up, x.bl_num_down, x.st_num_up, x.st_num_down) for x in a.subs] == \
               [(x.spos, x.sdim, x.bl_num_up, x.bl_num_down, x.st_num_up, x.st_num_down) for x in b.subs]
    osup = o_gsb(obs, obs, 10, 0)
    psup = T.get_super_basis(pbs, pbs, 10, 0)
    assert [(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down, s.sys_dim, s.env_dim) for s in osup.subs] == \
           [tuple(r) for r in psup.array()[:psup.num]]
