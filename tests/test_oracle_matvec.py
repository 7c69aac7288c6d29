"""Known answers for the oracle's model_wave on superblocks of an oracle DMRG
run: Hermiticity <x, H y> = conj <y, H x> and linearity, Hubbard and t-J."""
import numpy as np
import pytest

from tests import helpers as H


@pytest.mark.parametrize("kw", [dict(W=2, L=6, n_elec=10, m=32, U=8.0, phi=0.25),
                                dict(W=2, L=6, n_elec=10, m=32, U=0.0, phi=1.0 / 6.0, model="tj", J=0.4)])
def test_oracle_matvec_hermitian_and_linear(kw):
    lat, d = H.record_superblocks(**kw)
    for rec in (d.record[len(d.record) // 2], d.record[-3]):
        sup = rec[5]
        x, y = H.random_wave(sup, 11), H.random_wave(sup, 12)
        hx, hy = H.oracle_hpsi(rec, d.st, x).flat(), H.oracle_hpsi(rec, d.st, y).flat()
        lhs = np.vdot(x.flat(), hy)
        rhs = np.conj(np.vdot(y.flat(), hx))
        assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))
        a, b = 0.3 - 1.1j, -0.7 + 0.2j
        z = x.zeros_like()
        z.set_flat(a * x.flat() + b * y.flat())
        hz = H.oracle_hpsi(rec, d.st, z).flat()
        np.testing.assert_allclose(hz, a * hx + b * hy, atol=1e-12 * np.abs(hz).max())
