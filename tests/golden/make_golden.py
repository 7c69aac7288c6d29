"""Writes the golden fixtures of tests/test_golden.py (run from the repository
root: python tests/golden/make_golden.py).

The reference (Fortran + MKL) cannot be built or run here, so the fixtures
are known answers of this project's own independent code paths:

* ed_known_answers.json: Fock-basis exact diagonalisation (oracle/ed.py,
  which shares nothing with the SU(2) code) of a Hubbard flux ladder and a
  t-J ladder: singlet ground energies, and for the Hubbard ladder the density,
  spin and electron (sum_s <c+_i c_j>, complex) correlation matrices and
  singlet-pair correlations <D+_x D_y> of bonds on either side of the middle
  (for the t-J ladder: spin, electron and pair correlations of its singlet);
* matvec_tj_2x6.npz and matvec_hubbard_4x4.npz: a seeded input vector and the
  oracle's model_wave of it on small synthetic mid-chain superblocks
  (hofstadter_hubbard_tsc_gb300/synth.py).
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ed  # noqa: E402
from oracle.lattice import Lattice  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

PAIR_BONDS = [[1, 2], [8, 7], [7, 6], [6, 5], [8, 6], [7, 5], [8, 5]]

MATVEC_CASES = {
    "matvec_tj_2x6": dict(W=2, L=6, n_elec=10, m=24, model="tj", J=0.4, phi=1.0 / 6.0),
    "matvec_hubbard_4x4": dict(W=4, L=4, n_elec=14, m=30, phi=0.25),
}


def ed_fixtures():
    hub = Lattice(2, 4, U=8.0, phi=0.25)
    e_h, _ = ed.singlet_ground_energy(hub, 6)
    _, dens, corr = ed.hubbard_density_correlations(hub, 3, 3)
    _, ss, _ = ed.hubbard_spin_correlations(hub, 3, 3)
    _, G = ed.hubbard_green(hub, 3, 3)
    _, P = ed.hubbard_pair_correlations(hub, 3, 3, PAIR_BONDS)
    tj = Lattice(2, 4, model="tj", J=0.4, U=0.0, phi=1.0 / 6.0)
    e_t = ed.tj_singlet_ground_energy(tj, 6)
    _, Gt, Pt = ed.tj_singlet_correlations(tj, 6, [tuple(b) for b in PAIR_BONDS])
    _, sst = ed.tj_singlet_spin_correlations(tj, 6)
    return {
        "hubbard_2x4_U8_phi0.25_Ne6": {"energy": float(e_h), "density": dens.tolist(), "nn": corr.tolist(),
                                       "ss": ss.tolist(), "green_re": G.real.tolist(), "green_im": G.imag.tolist(),
                                       "pair_bonds": PAIR_BONDS, "pair_re": P.real.tolist(),
                                       "pair_im": P.imag.tolist()},
        "tj_2x4_J0.4_phi1/6_Ne6": {"energy": float(e_t), "ss": sst.tolist(), "green_re": Gt.real.tolist(),
                                   "green_im": Gt.imag.tolist(), "pair_bonds": PAIR_BONDS,
                                   "pair_re": Pt.real.tolist(), "pair_im": Pt.imag.tolist()},
    }


def matvec_fixture(kw, seed=42):
    import bench
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    wl = Workload(**kw)
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    _, hpsi = bench.cpu_matvec_timer(wl, psi, 1)
    return psi, hpsi


if __name__ == "__main__":
    with open(os.path.join(HERE, "ed_known_answers.json"), "w") as f:
        json.dump(ed_fixtures(), f, indent=1)
    for name, kw in MATVEC_CASES.items():
        psi, hpsi = matvec_fixture(kw)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), psi=psi, hpsi=hpsi)
        print(name, psi.size)
