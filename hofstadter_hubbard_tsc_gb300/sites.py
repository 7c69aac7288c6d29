"""SU(2)-reduced single-site operators (values of code/warm_up.f90:818-991).

Hubbard sites have the multiplets (N, 2S) = (0,0), (1,1), (2,0); t-J sites
drop the doublon.  Reduced elements carry sqrt(2j+1): <(1,1)||c+||(0,0)> =
-sqrt2, <(2,0)||c+||(1,1)> = sqrt2, the identity on the doublet is sqrt2.
"""
import numpy as np

from .types import SubBlock, TotalBlock


def _s(up, down, dd, v):
    return SubBlock(up, down, dd, np.array([[v]], dtype=np.complex128))


class SiteOperators:
    def __init__(self, model="hubbard"):
        hub = model == "hubbard"
        r2 = np.sqrt(2.0)
        self.elec_up = TotalBlock(1, 1, 1, [_s(0, 0, 1, -r2)] + ([_s(1, 1, -1, r2)] if hub else []))
        self.elec_down = TotalBlock(1, -1, 1, [_s(1, 1, -1, -r2)] + ([_s(2, 0, 1, -r2)] if hub else []))
        self.num_elec = TotalBlock(1, 0, 0, [_s(0, 0, 0, 0.0), _s(1, 1, 0, r2)] + ([_s(2, 0, 0, 2.0)] if hub else []))
        self.double = TotalBlock(1, 0, 0, [_s(0, 0, 0, 0.0), _s(1, 1, 0, 0.0)] + ([_s(2, 0, 0, 1.0)] if hub else []))
        self.sd = TotalBlock(1, 0, 2, [_s(1, 1, 0, np.sqrt(1.5))])
        self.sz = TotalBlock(1, 0, 0, [_s(0, 0, 0, 0.0), _s(1, 1, 0, 0.5)] + ([_s(2, 0, 0, 0.0)] if hub else []))
        self.si = TotalBlock(1, 0, 0, [_s(0, 0, 0, 1.0), _s(1, 1, 0, r2)] + ([_s(2, 0, 0, 1.0)] if hub else []))

    @staticmethod
    def trans_of(b):
        """block_transfer_trans of a site operator (code/space_info.f90:32-63)."""
        return TotalBlock(b.len, -b.up_dif, b.down_dif,
                          [SubBlock(s.num_up + b.up_dif, s.num_down + s.down_dif, -s.down_dif,
                                    np.conj(s.mat.T)) for s in b.subs])
