"""model_wave on the GPU (FP64 path) against the oracle on superblocks that the
oracle DMRG actually solved: flux ladders and cylinders, every step of a sweep."""
import numpy as np
import pytest

from oracle.sites import SiteOps
from hofstadter_hubbard_tsc_gb300.superblock import Superblock
from tests import helpers as H

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # relative to ||H psi||; complex FP64 on both sides


def _check_case(device, W, L, ne, m, U=8.0, phi=0.25, stride=1, model="hubbard", J=0.0):
    lat, d = H.record_superblocks(W, L, ne, m, U=U, phi=phi, model=model, J=J)
    plat = H.product_lattice(lat)
    st = SiteOps(model)
    worst = 0.0
    for idx, rec in enumerate(d.record[::stride]):
        sys, env, sys_bs, env_bs, geo, sup, guess = rec
        psi = H.random_wave(sup, seed=idx)
        ref = H.oracle_hpsi(rec, st, psi)
        sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                        H.superbasis(sup), plat.geometry(sys.len, env.len))
        out = sb.model_wave(H.wave(psi))
        a, b = out.flat(), ref.flat()
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
        worst = max(worst, err)
        assert err < RTOL, (idx, sys.len, env.len, err)
        sb.free()
    return worst


def test_matvec_ladder_2x6(device):
    _check_case(device, 2, 6, 10, 32)


def test_matvec_cylinder_4x3(device):
    _check_case(device, 4, 3, 10, 24, U=4.0, stride=2)


def test_matvec_tj_ladder_2x6(device):
    """t-J terms (S.S and n n couplings, the v123 branch of model_wave)."""
    _check_case(device, 2, 6, 10, 32, U=0.0, phi=1.0 / 6.0, model="tj", J=0.4)


def test_matvec_hermitian(device):
    lat, d = H.record_superblocks(2, 6, 10, 32)
    plat = H.product_lattice(lat)
    rec = d.record[-3]
    sys, env, sys_bs, env_bs, geo, sup, _ = rec
    sb = Superblock(device, H.model(sys), H.model(env), H.basis(sys_bs), H.basis(env_bs),
                    H.superbasis(sup), plat.geometry(sys.len, env.len))
    x = H.wave(H.random_wave(sup, 11))
    y = H.wave(H.random_wave(sup, 12))
    hx, hy = sb.model_wave(x).flat(), sb.model_wave(y).flat()
    lhs = np.vdot(x.flat(), hy)
    rhs = np.conj(np.vdot(y.flat(), hx))
    assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))
