"""lanczos_memo_new on the GPU against the oracle restatement (same start vector)."""
import numpy as np
import pytest

from oracle.sites import SiteOps
from oracle.lanczos import lanczos_memo_new as o_lanczos
from oracle.matvec import hmerge, model_wave
from hofstadter_hubbard_tsc_gb300.superblock import Superblock
from tests import helpers as H

pytestmark = pytest.mark.gpu


def test_lanczos_energy_matches_oracle(device):
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    st = SiteOps("hubbard")
    for rec in d.record[-4:]:
        sys, env, sys_bs, env_bs, geo, sup, guess = rec
        s2, e2 = H.copy_model(sys), H.copy_model(env)
        hmerge(s2, e2, geo)
        start = H.random_wave(sup, 5)
        o_psi = start.copy()
        e_ref, it_ref = o_lanczos(lambda v, o: model_wave(s2, e2, sys_bs, env_bs, v, o, geo, st), o_psi, 1e-10)
        sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                        H.superbasis(sup), plat.geometry(sys.len, env.len))
        e_gpu, it_gpu, psi = sb.lanczos_memo_new(H.wave(start), 1e-10)
        assert e_gpu == pytest.approx(e_ref, abs=1e-9)
        assert abs(it_gpu - it_ref) <= 2
        # ground state vectors agree up to a global phase
        a, b = psi.flat(), H.wave(o_psi).flat()
        ov = abs(np.vdot(a, b))
        assert ov == pytest.approx(1.0, abs=1e-7)
        sb.free()
