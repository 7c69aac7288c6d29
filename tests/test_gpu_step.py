"""Density matrix + truncation, operator renormalisation and wavefunction
transformation on the GPU against the oracle, on states and operators of real
oracle DMRG runs."""
import numpy as np
import pytest

import oracle.dmrg as odmrg
from oracle.density import get_density_matrix_sys, get_density_matrix_env, get_truncation_operator
from oracle.blocks import update_trun_ndia, update_trun_dia
from oracle.lattice import Lattice
from hofstadter_hubbard_tsc_gb300.device import DBlock, DBasis, DWave
from hofstadter_hubbard_tsc_gb300 import _lib, step
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _dwave(device, ow):
    w = H.wave(ow)
    dw = DWave(device, w.layout(), w.sys_len, w.env_len)
    dw.upload(w.flat())
    return dw


def _projectors(blk):
    return {(s.num_up, s.num_down): s.mat @ s.mat.conj().T for s in blk.subs}


@pytest.mark.parametrize("side", [0, 1])
def test_density_truncate(device, side):
    lat, d = H.record_superblocks(2, 6, 10, 24)
    for rec in d.record[-4:]:
        sup = rec[5]
        psi = H.random_wave(sup, 3)
        den = get_density_matrix_sys(psi) if side == 0 else get_density_matrix_env(psi)
        kmin, kmax = 12, 20
        o_trun, o_ns, o_err, o_ent, o_spec = get_truncation_operator(den, kmin, kmax, 1e-6)
        trun, ns, err, ent, spec = step.density_truncate(device, _dwave(device, psi), side, kmin, kmax, 1e-6)
        assert ns == o_ns
        assert err == pytest.approx(o_err, abs=1e-12)
        assert ent == pytest.approx(o_ent, abs=1e-12)
        np.testing.assert_allclose(spec, o_spec, atol=1e-13)
        # the kept subspace is unique when the cut falls in a gap of the spectrum
        if ns < len(spec) and (spec[ns - 1] < 1e-10 or spec[ns - 1] - spec[ns] < 1e-10):
            continue
        g = trun.download()
        assert [(s.num_up, s.num_down, s.row_dim, s.sdim) for s in g.subs] == \
               [(s.num_up, s.num_down, s.row_dim, s.sdim) for s in o_trun.subs]
        po, pg = _projectors(o_trun), _projectors(g)
        for k in po:
            np.testing.assert_allclose(pg[k], po[k], atol=1e-10)


@pytest.mark.parametrize("side", [0, 1])
def test_density_truncate_sector_sizes(device, side):
    """Sector sizes on both sides of each switch of the eigensolver: its
    Jacobi kernel (up to 16 states), the cluster reduction with the sector in
    shared memory (up to about 600) and with the sector in place in global
    memory (700 here), with a spectrum decaying over many decades like a DMRG
    density matrix."""
    from oracle.blocks import SSector, Super, WSub, Wave
    dims = [(1, 2), (7, 9), (31, 12), (32, 40), (33, 50), (64, 60), (112, 120), (150, 160), (300, 280),
            (512, 400), (700, 300)]
    rng = np.random.default_rng(21)
    subs = []
    for k, (a, b) in enumerate(dims):
        ss = SSector(2 * k, k % 3, 40 - 2 * k, k % 3, a, b)
        decay = np.exp(-np.arange(max(a, b)) / 6.0)
        v = rng.normal(size=(a, b)) + 1j * rng.normal(size=(a, b))
        v *= (decay[:a, None] if side == 0 else decay[None, :b]) * np.exp(-k / 2.0)
        subs.append(WSub(ss, v))
    psi = Wave(3, 3, subs)
    nrm = np.sqrt(sum(np.vdot(w.vec, w.vec).real for w in subs))
    for w in subs:
        w.vec /= nrm
    den = get_density_matrix_sys(psi) if side == 0 else get_density_matrix_env(psi)
    kmin, kmax = 150, 260
    o_trun, o_ns, o_err, o_ent, o_spec = get_truncation_operator(den, kmin, kmax, 1e-10)
    trun, ns, err, ent, spec = step.density_truncate(device, _dwave(device, psi), side, kmin, kmax, 1e-10)
    assert ns == o_ns
    assert err == pytest.approx(o_err, abs=1e-12)
    assert ent == pytest.approx(o_ent, abs=1e-12)
    np.testing.assert_allclose(spec, o_spec, atol=5e-14)
    g = trun.download()
    assert [(s.num_up, s.num_down, s.row_dim, s.sdim) for s in g.subs] == \
           [(s.num_up, s.num_down, s.row_dim, s.sdim) for s in o_trun.subs]
    rho = {(s.num_up, s.num_down): s.mat for s in den.subs}
    for sg in g.subs:
        # every kept column is an eigenvector of its sector, the columns are
        # orthonormal and each carries the canonical phase
        v = sg.mat
        r = rho[(sg.num_up, sg.num_down)]
        lam = np.einsum("ij,ik,kj->j", v.conj(), r, v).real
        np.testing.assert_allclose(r @ v - v * lam, 0.0, atol=5e-14)
        np.testing.assert_allclose(v.conj().T @ v, np.eye(sg.sdim), atol=1e-12)
        top = v[np.argmax(np.abs(v), axis=0), np.arange(sg.sdim)]
        np.testing.assert_allclose(top.imag, 0.0, atol=1e-15)
        assert np.all(top.real > 0)


def test_renormalize(device):
    lat, d = H.record_superblocks(2, 6, 10, 24)
    st = odmrg.SiteOps("hubbard")
    for rec in d.record[-3:]:
        sys_, env, sys_bs, env_bs, geo, sup, _ = rec
        from oracle.blocks import update_block_dia, update_block_ndia
        psi = H.random_wave(sup, 4)
        o_trun, *_ = get_truncation_operator(get_density_matrix_sys(psi), 10, 16, 1e-8)
        d_trun = DBlock.upload(device, H.block(o_trun))
        # an enlarged diagonal operator (the Hamiltonian) and a rank-1/2 boundary operator
        ham = update_block_dia(sys_.ham, sys_bs)
        op = update_block_ndia(sys_.sub[1]["elec_up"], sys_bs, "F", "sys")
        for blk, dia in ((ham, True), (op, False)):
            ref = update_trun_dia(blk, o_trun) if dia else update_trun_ndia(blk, o_trun)
            got = step.update_trun(device, DBlock.upload(device, H.block(blk)), d_trun, dia).download()
            assert [(s.num_up, s.num_down, s.down_dif, s.row_dim, s.sdim) for s in ref.subs] == \
                   [(s.num_up, s.num_down, s.down_dif, s.row_dim, s.sdim) for s in got.subs]
            for a, b in zip(ref.subs, got.subs):
                np.testing.assert_allclose(b.mat, a.mat, atol=1e-11)
            # double-float products (the block operators of split-precision
            # sweeps): FP64-class, then the context back at FP64
            gdf = step.update_trun(device, DBlock.upload(device, H.block(blk)), d_trun, dia,
                                   precision=_lib.HH_PREC_FP32X2).download()
            for a, b in zip(ref.subs, gdf.subs):
                np.testing.assert_allclose(b.mat, a.mat, atol=1e-11)
            again = step.update_trun(device, DBlock.upload(device, H.block(blk)), d_trun, dia).download()
            for a, b in zip(got.subs, again.subs):
                np.testing.assert_array_equal(a.mat, b.mat)
    assert device.lib.hh_ctx_set_renormalize_precision(device.h, _lib.HH_PREC_BF16X3) == -1


def test_wave_transform(device, monkeypatch):
    calls = []
    for name in ("wave_trans_lr", "wave_trans_rl"):
        orig = getattr(odmrg, name)

        def wrap(sys_bs, env_bs, sys_trun, env_trun, old, new, _o=orig, _n=name):
            before = old.copy()
            _o(sys_bs, env_bs, sys_trun, env_trun, old, new)
            calls.append((_n, sys_bs, env_bs, sys_trun, env_trun, before, new.copy()))
        monkeypatch.setattr(odmrg, name, wrap)
    lat = Lattice(2, 6, U=8.0, phi=0.25)
    d = odmrg.DMRG(lat, 10, kept_min=16, kept_max=16, trun_err=1e-12, lanzero=1e-9, seed=5)
    d.run(sweeps=1)
    assert len(calls) > 4
    for (name, sbs, ebs, strun, etrun, old, new) in calls:
        direction = "LR" if name.endswith("lr") else "RL"
        dold = _dwave(device, old)
        dnew = DWave(device, H.wave(new).layout(), new.sys_len, new.env_len)
        args = (DBasis(device, H.basis(sbs)), DBasis(device, H.basis(ebs)), DBlock.upload(device, H.block(strun)),
                DBlock.upload(device, H.block(etrun)), dold, dnew)
        step.wave_trans(device, direction, *args)
        np.testing.assert_allclose(dnew.download(), H.wave(new).flat(), atol=1e-12)
        # the FP32-arithmetic transform of split-precision runs (a Lanczos start
        # vector): within FP32 rounding of the FP64 result, then back to FP64
        step.wave_trans(device, direction, *args, precision=_lib.HH_PREC_FP32)
        ref = H.wave(new).flat()
        assert np.linalg.norm(dnew.download() - ref) <= 1e-6 * np.linalg.norm(ref)
    assert device.lib.hh_ctx_set_transform_precision(device.h, _lib.HH_PREC_BF16X3) == -1
