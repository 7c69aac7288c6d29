"""GB300-native superblock step of the SU(2) block DMRG of cfengno1/Hofstadter_Hubbard_TSC.

The compute lives in ``libhh_dmrg.so`` (C ABI: include/hh_dmrg.h); this
package is the host-side mirror of the reference's interfaces for the hot
path: the data model (types), the superblock geometry tables (lattice), the
site operators (sites) and the superblock step (superblock).
"""
from . import _lib  # noqa: F401
from .types import (SubBlock, TotalBlock, SubBasisMap, BasisMap, TotalBasis, SuperBasis,  # noqa: F401
                    SubWave, Wavefunction, TotalModel, get_basis, get_super_basis)

__all__ = ["SubBlock", "TotalBlock", "SubBasisMap", "BasisMap", "TotalBasis", "SuperBasis",
           "SubWave", "Wavefunction", "TotalModel", "get_basis", "get_super_basis"]
