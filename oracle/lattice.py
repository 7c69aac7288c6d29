"""Lattice tables, couplings and DMRG site ordering.

Restates ``dmrg_setup`` (code/warm_up.f90:347-666, square branch) and
``dmrg_setup0`` (code/warm_up.f90:311-341) for W x L square-lattice ladders and
cylinders.  Sites are numbered i = y + (x-1)*W (code/warm_up.f90:796-811).

Differences from the reference, by design:
  * the square branch of the reference also lists the two diagonals of every
    plaquette with zero coupling (code/warm_up.f90:445-457); bonds with zero
    coupling contribute nothing, so only nearest-neighbour bonds are listed here;
  * ``get_phase`` (code/quantum.f90:293-438) is specific to the triangular
    lattice; the Landau-gauge table here puts exp(i 2 pi phi x) on every y bond
    at column x (flux phi per square plaquette), 1 on x bonds.
Couplings use the reference's reduced-element normalisation: jt = -sqrt(2) t
(code/quantum.f90:121), jd = -sqrt(3) J and jn = -J/4 for t-J
(code/quantum.f90:92-108).
"""
import numpy as np


class Lattice:
    def __init__(self, W, L, model="hubbard", t=1.0, U=8.0, J=0.0, phi=0.25,
                 open_x=True):
        self.W, self.L = W, L
        self.N = W * L
        self.model = model
        self.tjmodel = model == "tj"
        self.v123 = 1 if self.tjmodel else 0
        self.t, self.U, self.J, self.phi = t, U, J, phi
        self.open_x = open_x
        # full-lattice neighbour table, used by dmrg_setup0 (inb1/nleg11)
        self._full = self._neib(self.L)
        self._setup0()

    # -- couplings -------------------------------------------------------
    def jt_val(self):
        return -np.sqrt(2.0) * self.t

    def _neib(self, nxc):
        """Directional neighbour table for nxc columns: dict lat -> {k: lat}."""
        W = self.W
        nb = {}
        for ix in range(1, nxc + 1):
            for iy in range(1, W + 1):
                nb.setdefault(iy + (ix - 1) * W, {})
        for ix in range(1, nxc + 1):
            for iy in range(1, W + 1):
                ii = iy + (ix - 1) * W
                if W >= 2 and (iy != W or W != 2):
                    jy = ii - iy + (iy % W) + 1
                    nb[ii][1] = jy
                    nb[jy][2] = ii
                jx = ii + W
                if jx > W * nxc:
                    jx = 0
                if jx:
                    nb[ii][3] = jx
                    nb[jx][4] = ii
        return nb

    def _setup0(self):
        """inb1 / nleg11 (code/warm_up.f90:311-341) on the full lattice."""
        self.inb1 = {}
        self.nleg11 = {}
        for ns in range(1, self.N - 1):
            k0 = 0
            for i1 in range(1, ns + 1):
                self.inb1[(i1, ns)] = 10000
                if any(j >= ns for j in self._full.get(i1, {}).values()):
                    k0 += 1
                    self.inb1[(i1, ns)] = k0
            self.nleg11[ns] = k0
        # block length ns = N-1 or N never needs boundary operators
        for ns in (self.N - 1, self.N):
            self.nleg11[ns] = 0

    def phase(self, i, j):
        """pint(i,j): Peierls factor multiplying c+_i c_j (Landau gauge A || y)."""
        W = self.W
        xi, yi = (i - 1) // W + 1, (i - 1) % W + 1
        xj, yj = (j - 1) // W + 1, (j - 1) % W + 1
        if xi != xj:
            return 1.0 + 0.0j
        # y bond inside column xi; orientation +y when j follows i (cyclically
        # only on cylinders: a 2-leg ladder has a single rung and no wrap bond)
        fwd = (yj == yi + 1) or (W > 2 and yi == W and yj == 1)
        a = 2.0 * np.pi * self.phi * xi
        return np.exp(1j * a) if fwd else np.exp(-1j * a)

    def geometry(self, ns, ns21):
        return Geometry(self, ns, ns21)


class Geometry:
    """Tables of one superblock [sys(ns) - site - site - env(ns21)] (dmrg_setup)."""

    def __init__(self, lat, ns, ns21):
        self.lat = lat
        self.tjmodel = lat.tjmodel
        self.v123 = lat.v123
        self.inb1 = lat.inb1
        self.nleg11 = lat.nleg11
        W = lat.W
        nn = ns + ns21 + 2
        nxc = (nn - 1) // W + 1
        if nxc == 1:
            nxc = 2
        self.nxc = nxc
        totsite = W * nxc
        self.totsite = totsite
        self.nposi = {}
        self.nposi_lat = {}
        self.nposi_dm = {}
        for i in range(1, ns + 2):
            self.nposi[i] = 1
            self.nposi_lat[i] = i
            self.nposi_dm[i] = i
        self.nposi[ns + 1] = 2
        for i in range(1, ns21 + 2):
            self.nposi[ns + 1 + i] = 3
            self.nposi_dm[totsite + 1 - i] = i + ns + 1
            self.nposi_lat[i + ns + 1] = totsite + 1 - i
        self.nposi[ns + ns21 + 2] = 4
        self.neib = lat._neib(nxc)
        self.coup_bs = [[0, 0], [0, 0]]
        self.coup_bb = [0, 0]
        self.inb = {}

    # lattice queries -------------------------------------------------
    def bonds(self, latidx):
        d = self.neib.get(latidx, {})
        return [(k, d[k]) for k in sorted(d)]

    def neighbours(self, latidx):
        return [j for _, j in self.bonds(latidx)]

    def region(self, latidx):
        """nposi(nposi_dm(j)): 1 sys block, 2 sys site, 3 env block, 4 env site, 0 none."""
        return self.nposi.get(self.nposi_dm.get(latidx, 0), 0)

    def neiba(self, i, j):
        for k, jj in self.bonds(i):
            if jj == j:
                return k
        return 0

    def jt(self, k, i):
        return self.lat.jt_val() + 0j if k in (1, 2, 3, 4) else 0j

    def jd(self, k, i):
        if self.tjmodel and k in (1, 2, 3, 4):
            return -np.sqrt(3.0) * self.lat.J + 0j
        return 0j

    def jn(self, k, i):
        if self.tjmodel and k in (1, 2, 3, 4):
            return -0.25 * self.lat.J + 0j
        return 0j

    def pint(self, i, j):
        return self.lat.phase(i, j)

    def hubbard(self, i):
        return 0.0 if self.tjmodel else self.lat.U

    def op_names(self):
        names = ["elec_up", "elec_down"]
        if self.tjmodel:
            names.append("spin_sd")
        if self.v123:
            names.append("num_sn")
        return names
