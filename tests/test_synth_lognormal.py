"""The synthetic block-sparse configuration (lognormal sector dimensions,
the 12-term superblock of a 6-wide cylinder, 8 uneven wavefunctions): its
generator and, at small scale, the oracle's matvec on it."""
import numpy as np

import bench
from hofstadter_hubbard_tsc_gb300.synth import Workload, lognormal_sectors, uneven_batch

FULL = dict(n_sectors=150, median=96, max_dim=2048)
SMALL = dict(W=6, L=8, n_elec=42, U=8.0, phi=1.0 / 3.0, lognormal=(24, 8, 32))


def test_lognormal_sectors_full_size():
    """150 sectors per block of the 6x24 mid-chain (71 sites, 1/12 doping):
    valid SU(2) labels, one connected graph under the rank-1/2 moves
    (N +- 1, 2S +- 1), dims within [8, 2048] with the largest 2048 and the
    median near 96."""
    rng = np.random.default_rng(20261203)
    sec = lognormal_sectors(71, 132 / 144 * 71, FULL["n_sectors"], FULL["median"], FULL["max_dim"], rng)
    assert len(sec) == 150 and len({(N, S2) for N, S2, _ in sec}) == 150
    assert all(S2 % 2 == N % 2 and 0 <= S2 <= min(N, 142 - N) for N, S2, _ in sec)
    dims = np.array([d for *_, d in sec])
    assert dims.min() >= 8 and dims.max() == 2048
    assert 70 <= np.median(dims) <= 130
    labels = {(N, S2) for N, S2, _ in sec}
    start = next(iter(labels))
    seen, todo = {start}, [start]
    while todo:
        N, S2 = todo.pop()
        for dn in (-1, 1):
            for ds in (-1, 1):
                q = (N + dn, S2 + ds)
                if q in labels and q not in seen:
                    seen.add(q)
                    todo.append(q)
    assert seen == labels


def test_small_scale_workload_and_oracle():
    """The small-scale configuration has the 12-term superblock; the oracle's
    H psi on it is Hermitian; the uneven batch spans eight decades of norm."""
    wl = Workload(**SMALL)
    assert wl.describe()["block_sectors"] == [24, 24]
    rng = np.random.default_rng(4)
    sizes = [s.sys_dim * s.env_dim for s in wl.sup.subs]
    psi = uneven_batch(sizes, 8, rng)
    norms = np.linalg.norm(psi, axis=1)
    assert norms[-1] / norms[0] > 1e6
    x, y = psi[3], psi[4]
    _, hx = bench.cpu_matvec_timer(wl, x, 1)
    _, hy = bench.cpu_matvec_timer(wl, y, 1)
    lhs, rhs = np.vdot(x, hy), np.conj(np.vdot(y, hx))
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)
