"""Algebraic identities of the SU(2) operator product (block_mul_block_ndia,
code/space_info.f90:373-631) in the reference's reduced conventions: on one
site, [c+ x c]^0 = n / sqrt(2) and [c+ x c]^1 = sqrt(2) sd, whether the site
is the enlarged basis's new site or its block."""
import numpy as np
import pytest

from oracle.blocks import (block_mul_block_ndia, update_block_dia, update_block_ndia, update_site_dia,
                           update_site_ndia)
from oracle.dmrg import DMRG
from oracle.lattice import Lattice


@pytest.fixture(scope="module")
def basis2():
    d = DMRG(Lattice(2, 4, U=8.0, phi=0.25), 6, kept_min=256, kept_max=256, trun_err=1e-14, lanzero=1e-11, seed=3)
    d.run(sweeps=1)
    return d.sys_bases[2], d.st


def _ratio(prod, ref, with_dd):
    """The single constant c with prod = c ref (sub-block by sub-block)."""
    vals = []
    for s in prod.subs:
        k = ref.find(s.num_up, s.num_down, s.down_dif) if with_dd else ref.find(s.num_up, s.num_down)
        if k is None:
            np.testing.assert_allclose(s.mat, 0, atol=1e-12)
            continue
        m = ref.subs[k].mat
        mask = np.abs(m) > 1e-12
        np.testing.assert_allclose(s.mat[~mask], 0, atol=1e-12)
        vals.extend((s.mat[mask] / m[mask]).ravel())
    vals = np.array(vals)
    assert len(vals) > 0
    np.testing.assert_allclose(vals, vals[0], atol=1e-12)
    return vals[0]


@pytest.mark.parametrize("where", ["site", "block"])
def test_rank0_product_is_number_operator(basis2, where):
    B, st = basis2
    if where == "site":
        up, dn = update_site_ndia(st.elec_up, B, "F", "sys"), update_site_ndia(st.elec_down, B, "F", "sys")
        n = update_site_dia(st.num_elec, B)
    else:
        up, dn = update_block_ndia(st.elec_up, B, "F", "sys"), update_block_ndia(st.elec_down, B, "F", "sys")
        n = update_block_dia(st.num_elec, B)
    assert _ratio(block_mul_block_ndia(up, dn, 0, B), n, False) == pytest.approx(1 / np.sqrt(2), abs=1e-12)


def test_rank1_product_is_spin_operator(basis2):
    B, st = basis2
    up, dn = update_site_ndia(st.elec_up, B, "F", "sys"), update_site_ndia(st.elec_down, B, "F", "sys")
    sd = update_site_ndia(st.sd, B, "B", "sys")
    assert _ratio(block_mul_block_ndia(up, dn, 2, B), sd, True) == pytest.approx(np.sqrt(2), abs=1e-12)
