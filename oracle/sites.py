"""SU(2)-reduced single-site operators (code/warm_up.f90:818-991, 1248-1279).

Reduced matrix elements carry the sqrt(2j+1) factor of the reference: the
identity on the spin-1/2 multiplet is sqrt(2) and n on the doublon is 2.
Hubbard sites have the multiplets (N, 2S) = (0,0), (1,1), (2,0); t-J sites drop
the doublon.
"""
import numpy as np

from .blocks import Block, Sub


def _one(num_up, num_down, dd, val):
    return Sub(num_up, num_down, dd, 1, 1, np.array([[val]], dtype=np.complex128))


class SiteOps:
    def __init__(self, model="hubbard"):
        hub = model == "hubbard"
        self.model = model
        self.n_max = 3 if hub else 2
        r2 = np.sqrt(2.0)
        # c^+ (code/warm_up.f90:850-872): <(1,1)||c+||(0,0)> = -sqrt2, <(2,0)||c+||(1,1)> = sqrt2
        self.elec_up = Block(1, 1, 1, [_one(0, 0, 1, -r2)] + ([_one(1, 1, -1, r2)] if hub else []))
        # c (code/warm_up.f90:875-888): copies c+ then relabels the kets
        self.elec_down = Block(1, -1, 1, [_one(1, 1, -1, -r2)] + ([_one(2, 0, 1, -r2)] if hub else []))
        subs_n = [_one(0, 0, 0, 0.0), _one(1, 1, 0, r2)] + ([_one(2, 0, 0, 2.0)] if hub else [])
        self.num_elec = Block(1, 0, 0, subs_n)
        self.double = Block(1, 0, 0, [_one(0, 0, 0, 0.0), _one(1, 1, 0, 0.0)]
                            + ([_one(2, 0, 0, 1.0)] if hub else []))
        # S (rank 1, down_dif=su) (code/warm_up.f90:935-948)
        self.sd = Block(1, 0, 2, [_one(1, 1, 0, np.sqrt(1.5))])
        self.sz = Block(1, 0, 0, [_one(0, 0, 0, 0.0), _one(1, 1, 0, 0.5)]
                        + ([_one(2, 0, 0, 0.0)] if hub else []))
        # identity with reduced elements sqrt(2j+1) (code/warm_up.f90:985-988)
        self.si = Block(1, 0, 0, [_one(0, 0, 0, 1.0), _one(1, 1, 0, r2)]
                        + ([_one(2, 0, 0, 1.0)] if hub else []))

    def site_ham(self, u=0.0):
        """Single-site Hamiltonian block (code/warm_up.f90:1208-1244, 1318-1323)."""
        h = self.num_elec.copy()
        for s, d in zip(h.subs, self.double.subs):
            s.mat = u * d.mat.copy()
        return h
