"""Host tables of the superblock geometry: bonds, couplings and DMRG site order.

Plays the role of the reference's module globals that ``hmerge`` and
``model_wave`` read (neib, nposi, nposi_dm, nposi_lat, inb1, nleg11, jt, jd, jn,
pint, hubbard; code/pubdata.f90:36-63, filled by dmrg_setup/dmrg_setup0 at
code/warm_up.f90:311-666).  Square W x L ladders (W=2, one rung per column)
and cylinders (W>2, periodic in y), open in x; sites i = y + (x-1) W.
Flux phi per plaquette in the Landau gauge A || y: the factor multiplying
c+_i c_j on the y bond i -> j of column x is exp(+i 2 pi phi x); x bonds are
real.  Couplings use the reduced-element normalisation of the reference:
jt = -sqrt(2) t, jd = -sqrt(3) J, jn = -J/4 (t-J only).
"""
import numpy as np


class SquareLattice:
    def __init__(self, W, L, model="hubbard", t=1.0, U=8.0, J=0.0, phi=0.25):
        self.W, self.L, self.N = int(W), int(L), int(W) * int(L)
        self.model = model
        self.tjmodel = model == "tj"
        self.v123 = 1 if self.tjmodel else 0
        self.t, self.U, self.J, self.phi = t, U, J, phi
        full = self.neighbour_table(self.L)
        # operator slots of the boundary sites of a block of length ns
        # (dmrg_setup0, code/warm_up.f90:311-341): a site keeps its operators
        # while it has a neighbour numbered >= ns.
        self.inb1, self.nleg11 = {}, {}
        for ns in range(1, self.N + 1):
            k0 = 0
            for i1 in range(1, ns + 1):
                self.inb1[(i1, ns)] = 10000
                if ns < self.N - 1 and any(j >= ns for j in full.get(i1, {}).values()):
                    k0 += 1
                    self.inb1[(i1, ns)] = k0
            self.nleg11[ns] = k0

    def neighbour_table(self, ncol):
        """lat -> {direction: lat}; 1/2 = +y/-y, 3/4 = +x/-x."""
        W = self.W
        nb = {i: {} for i in range(1, W * ncol + 1)}
        for ix in range(1, ncol + 1):
            for iy in range(1, W + 1):
                ii = iy + (ix - 1) * W
                if W >= 2 and (iy != W or W != 2):
                    jy = ii - iy + (iy % W) + 1
                    nb[ii][1] = jy
                    nb[jy][2] = ii
                jx = ii + W
                if jx <= W * ncol:
                    nb[ii][3] = jx
                    nb[jx][4] = ii
        return nb

    def phase(self, i, j):
        W = self.W
        xi, yi = (i - 1) // W + 1, (i - 1) % W + 1
        xj, yj = (j - 1) // W + 1, (j - 1) % W + 1
        if xi != xj:
            return 1.0 + 0.0j
        fwd = (yj == yi + 1) or (W > 2 and yi == W and yj == 1)
        a = 2.0 * np.pi * self.phi * xi
        return np.exp(1j * a) if fwd else np.exp(-1j * a)

    def geometry(self, ns, ne):
        return Geometry(self, ns, ne)


class Geometry:
    """Tables of the superblock [sys(ns) - site - site - env(ne)] (dmrg_setup, code/warm_up.f90:347-420)."""

    def __init__(self, lat, ns, ne):
        self.lat = lat
        self.tjmodel, self.v123 = lat.tjmodel, lat.v123
        self.inb1, self.nleg11 = lat.inb1, lat.nleg11
        W = lat.W
        nxc = max(2, (ns + ne + 1) // W + 1)
        tot = W * nxc
        self.nposi, self.nposi_lat, self.nposi_dm = {}, {}, {}
        for i in range(1, ns + 2):
            self.nposi[i], self.nposi_lat[i], self.nposi_dm[i] = 1, i, i
        self.nposi[ns + 1] = 2
        for i in range(1, ne + 2):
            self.nposi[ns + 1 + i] = 3
            self.nposi_dm[tot + 1 - i] = i + ns + 1
            self.nposi_lat[i + ns + 1] = tot + 1 - i
        self.nposi[ns + ne + 2] = 4
        self.neib = lat.neighbour_table(nxc)

    def bonds(self, latidx):
        d = self.neib.get(latidx, {})
        return [(k, d[k]) for k in sorted(d)]

    def neighbours(self, latidx):
        return [j for _, j in self.bonds(latidx)]

    def region(self, latidx):
        return self.nposi.get(self.nposi_dm.get(latidx, 0), 0)

    def neiba(self, i, j):
        for k, jj in self.bonds(i):
            if jj == j:
                return k
        return 0

    def jt(self, k, i):
        return -np.sqrt(2.0) * self.lat.t + 0j

    def jd(self, k, i):
        return (-np.sqrt(3.0) * self.lat.J + 0j) if self.tjmodel else 0j

    def jn(self, k, i):
        return (-0.25 * self.lat.J + 0j) if self.tjmodel else 0j

    def pint(self, i, j):
        return self.lat.phase(i, j)

    def hubbard(self, i):
        return 0.0 if self.tjmodel else self.lat.U

    def op_names(self):
        n = ["elec_up", "elec_down"]
        if self.tjmodel:
            n.append("spin_sd")
        if self.v123:
            n.append("num_sn")
        return n
