"""Seeded synthetic superblocks with the sector structure of a real DMRG step.

Used by bench.py when a workload is too large to grow with a full sweep (the
4x32 Hubbard cylinder at m = 2000, the 4x48 t-J cylinder at m = 4000, the 6x24
Hubbard cylinder at m = 6000): a
mid-chain superblock of a W x L cylinder keeps m multiplets per block, spread
over (N, 2S) block sectors with a Gaussian profile in N around the filling and
a profile (2S+1) exp(-S(S+1)/(2 s^2)) in S.  The profile was read off a real
finite-size run (4x6 cylinder, N_e=20, U=8, phi=1/4, m=120, 12-site blocks:
13 sectors, sigma_N = 1.2, s = 1.0, largest sector 17% of the states) and
widened for m=2000 and 63-site blocks to sigma_N = 2.5, s = 1.5 (65 sectors,
largest 123 multiplets).  Operator entries are N(0,1) complex (re, im ~ N(0, 1/2)); block
Hamiltonians are Hermitian.  The term list and every quantum-number rule come
from the real geometry (hmerge / model_wave), so the task structure and FLOP
count of the matvec are those of the physical superblock; only the numbers in
the blocks are random.  t-J blocks have no doubly occupied sites (N <= sites)
and carry, besides the hopping operators, the rank-1 spin operator spin_sd
and the rank-0 density num_sn of their boundary sites.
"""
import numpy as np

from .types import SubBlock, TotalBlock, TotalModel, get_basis, get_super_basis
from .sites import SiteOperators
from .lattice import SquareLattice


def block_sectors(n_sites, n_fill, m, rng, sigma_n=2.5, s_scale=1.5, max_dim=None, tj=False):
    """(N, 2S, dim) of a block that keeps m multiplets (tj: at most one
    electron per site)."""
    lo = max(0, int(n_fill - 4 * sigma_n))
    hi = min(n_sites if tj else 2 * n_sites, int(n_fill + 4 * sigma_n) + 1)
    cands, w = [], []
    for N in range(lo, hi + 1):
        smax = N if tj else min(N, 2 * n_sites - N)
        for S2 in range(N % 2, smax + 1, 2):
            s = S2 / 2.0
            wt = np.exp(-((N - n_fill) ** 2) / (2 * sigma_n ** 2)) * (2 * s + 1) * np.exp(-s * (s + 1) / (2 * s_scale ** 2))
            cands.append((N, S2))
            w.append(wt)
    w = np.array(w)
    w /= w.sum()
    dims = np.floor(w * m).astype(int)
    # distribute the remainder to the heaviest sectors, keep sectors with dim >= 1
    rem = m - dims.sum()
    order = np.argsort(-w)
    for i in order[:rem]:
        dims[i] += 1
    if max_dim is not None:
        dims = np.minimum(dims, max_dim)
    out = [(N, S2, int(d)) for (N, S2), d in zip(cands, dims) if d >= 1]
    rng.shuffle(out)
    # block sectors are stored in basis order (descending 2S, then N) in the reference
    out.sort(key=lambda q: (-q[1], -q[0]))
    return out


def lognormal_sectors(n_sites, n_center, n_sectors, median, max_dim, rng, min_dim=8, tj=False):
    """(N, 2S, dim) of a synthetic block: the n_sectors (N, 2S) nearest to
    (n_center, 0) (2S = N mod 2, 2S <= N and <= 2 n_sites - N; t-J: N <=
    n_sites), a region that the rank-1/2 operators (N +- 1, 2S +- 1) connect;
    dims clip(round(exp(ln median + sigma z)), min_dim, max_dim), z ~ N(0, 1)
    seeded, with sigma = ln(max_dim / median) / max z so that the largest
    sector has max_dim states."""
    cands = []
    nmax = n_sites if tj else 2 * n_sites
    for N in range(0, nmax + 1):
        smax = N if tj else min(N, 2 * n_sites - N)
        for S2 in range(N % 2, smax + 1, 2):
            cands.append(((N - n_center) ** 2 / 4.0 + S2 ** 2 / 9.0, N, S2))
    cands.sort()
    chosen = [(N, S2) for _, N, S2 in cands[:n_sectors]]
    z = rng.standard_normal(len(chosen))
    sigma = np.log(max_dim / median) / z.max()
    dims = np.clip(np.round(np.exp(np.log(median) + sigma * z)), min_dim, max_dim).astype(int)
    out = [(N, S2, int(d)) for (N, S2), d in zip(chosen, dims)]
    out.sort(key=lambda q: (-q[1], -q[0]))
    return out


def _herm(rng, d):
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    return (a + a.conj().T) / 2.0


def _rand(rng, r, c):
    return (rng.normal(scale=np.sqrt(0.5), size=(r, c)) + 1j * rng.normal(scale=np.sqrt(0.5), size=(r, c)))


def synthetic_model(length, sectors, slots, rng, names=("elec_up", "elec_down")):
    dims = {(N, S2): d for (N, S2, d) in sectors}
    ham = TotalBlock(length, 0, 0, [SubBlock(N, S2, 0, _herm(rng, d)) for (N, S2, d) in sectors])

    def ndia(up_dif):
        subs = []
        for (N, S2, d) in sectors:
            for dd in (-1, 1):
                tgt = (N + up_dif, S2 + dd)
                if tgt in dims and S2 + dd >= 0:
                    subs.append(SubBlock(N, S2, dd, _rand(rng, dims[tgt], d)))
        return TotalBlock(length, up_dif, 1, subs)

    def spin():
        # rank 1: 2S -> 2S + dd, dd in {-2, 0, 2}, no 0 -> 0
        subs = []
        for (N, S2, d) in sectors:
            for dd in (-2, 0, 2):
                tgt = (N, S2 + dd)
                if tgt in dims and S2 + dd >= 0 and not (S2 == 0 and dd == 0):
                    subs.append(SubBlock(N, S2, dd, _rand(rng, dims[tgt], d)))
        return TotalBlock(length, 0, 2, subs)

    def density():
        return TotalBlock(length, 0, 0, [SubBlock(N, S2, 0, _herm(rng, d)) for (N, S2, d) in sectors])

    sub = {}
    for k in range(1, slots + 1):
        d = {}
        if "elec_up" in names:
            d["elec_up"] = ndia(+1)
        if "elec_down" in names:
            d["elec_down"] = ndia(-1)
        if "spin_sd" in names:
            d["spin_sd"] = spin()
        if "num_sn" in names:
            d["num_sn"] = density()
        sub[k] = d
    return TotalModel(length, ham, sub)


class Workload:
    """A synthetic mid-chain superblock: models, bases, super basis, geometry."""

    def __init__(self, W=4, L=32, n_elec=112, m=2000, U=8.0, phi=0.25, seed=20261203, sys_len=None,
                 model="hubbard", J=0.0, lognormal=None):
        """lognormal = (sectors per block, median, max dim): block sectors
        from lognormal_sectors instead of the finite-size profile (m is then
        unused)."""
        self.W, self.L, self.n_elec, self.m, self.U, self.phi, self.seed = W, L, n_elec, m, U, phi, seed
        self.model, self.J, self.lognormal = model, J, lognormal
        tj = model == "tj"
        if tj:
            self.U = U = 0.0
        rng = np.random.default_rng(seed)
        self.lat = SquareLattice(W, L, model=model, U=U, J=J, phi=phi)
        N = self.lat.N
        ls = N // 2 - 1 if sys_len is None else sys_len
        le = N - ls - 2
        fill = n_elec / N
        names = ("elec_up", "elec_down", "spin_sd", "num_sn") if tj else ("elec_up", "elec_down")
        if lognormal is None:
            self.sys_sectors = block_sectors(ls, fill * ls, m, rng, tj=tj)
            self.env_sectors = block_sectors(le, fill * le, m, rng, tj=tj)
        else:
            ns, med, mx = lognormal
            self.sys_sectors = lognormal_sectors(ls, fill * ls, ns, med, mx, rng, min_dim=min(8, mx), tj=tj)
            self.env_sectors = lognormal_sectors(le, fill * le, ns, med, mx, rng, min_dim=min(8, mx), tj=tj)
        self.sys = synthetic_model(ls, self.sys_sectors, max(1, self.lat.nleg11[ls]), rng, names)
        self.env = synthetic_model(le, self.env_sectors, max(1, self.lat.nleg11[le]), rng, names)
        st = SiteOperators(model)
        self.sys_bs = get_basis(self.sys.ham, st.sz)
        self.env_bs = get_basis(self.env.ham, st.sz)
        self.sup = get_super_basis(self.sys_bs, self.env_bs, n_elec, 0)
        self.geo = self.lat.geometry(ls, le)
        if lognormal is not None:
            ns, med, mx = lognormal
            self.name = (f"synthetic-{W}x{L}-{model}-midchain-{2 * ns}sectors-lognormal-median{med:g}-max{mx}")
        elif tj:
            self.name = f"tj-cylinder-{W}x{L}-phi{phi:.4g}-J{J:g}-Ne{n_elec}-m{m}-midchain"
        else:
            self.name = f"hubbard-cylinder-{W}x{L}-phi{phi:.4g}-U{U:g}-Ne{n_elec}-m{m}-midchain"

    def describe(self):
        return {
            "workload": self.name,
            "block_dims": [sum(d for *_, d in self.sys_sectors), sum(d for *_, d in self.env_sectors)],
            "lattice": f"{self.W}x{self.L} {'ladder' if self.W == 2 else 'cylinder (periodic y, open x)'}, "
                       f"Landau gauge, {self.model}",
            "phi": self.phi, "U": self.U, "J": self.J, "t": 1.0, "n_elec": self.n_elec,
            "kept_multiplets": self.m if self.lognormal is None else None,
            "sys_len": self.sys.len, "env_len": self.env.len,
            "block_sectors": [len(self.sys_sectors), len(self.env_sectors)],
            "enlarged_dims": [self.sys_bs.dim, self.env_bs.dim],
            "wave_sectors": self.sup.num, "wave_dim": self.sup.dim,
            "operators": "synthetic N(0,1) complex, Hermitian block Hamiltonians, seed %d" % self.seed,
        }


def uneven_batch(sup_dim_sectors, nbatch, rng):
    """nbatch uneven wavefunctions over a superblock layout given as the list
    of its sector sizes: N(0,1) complex entries, each sector scaled by a
    lognormal weight drawn per vector and each vector by 10^(b - nbatch/2),
    flattened in layout order; shape (nbatch, total)."""
    total = sum(sup_dim_sectors)
    out = np.empty((nbatch, total), dtype=np.complex128)
    for b in range(nbatch):
        v = rng.normal(scale=np.sqrt(0.5), size=total) + 1j * rng.normal(scale=np.sqrt(0.5), size=total)
        o = 0
        for n in sup_dim_sectors:
            v[o:o + n] *= np.exp(rng.normal())
            o += n
        out[b] = v * 10.0 ** (b - nbatch / 2)
    return out
