"""lns3d_gb300: GB300-native implicit ADI line solvers of LNS3D.

The compute path is the sm_103a C-ABI library ``lib/liblns3d_gb300.so``
(``include/lns3d_gb300.h``); this package is its host-side mirror with the
reference's solver names and argument conventions.
"""
from ._lib import LnsError, lib, library_path
from .adi3d import Batch3D, ImpDrv3D, ImpDrvLin2D, Server3D
from .impdrv2d import ImpDrv2D
from .penta import (cpenta1bc, cpenta1p, cpenta2bc, cpenta2p, penta1bc, penta1p, penta2bc, penta2p,
                    set_periodic_exact, solve1bc, solve1p, solve2bc, solve2p)

__all__ = ["LnsError", "lib", "library_path", "penta2bc", "penta1bc", "cpenta2bc", "cpenta1bc", "penta2p",
           "penta1p", "cpenta2p", "cpenta1p", "set_periodic_exact", "solve2bc", "solve1bc", "solve2p", "solve1p", "ImpDrv3D", "ImpDrv2D",
           "ImpDrvLin2D", "Batch3D", "Server3D"]
