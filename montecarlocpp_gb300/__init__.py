"""montecarlocpp_gb300: GB300 (sm_103a) particle-advance hot path of the
montecarlocpp deviational phonon Monte Carlo solver.

The compute path is libmc_gb300.so (hand-written CUDA kernels behind the C
ABI in include/mc_gb300.h). This package mirrors the reference's host API
(Material, *Domain, Temp/Flux/Multi/CumTemp/CumFluxProblem) over that ABI.
"""

from .batch import Batch
from .serve import Server
from .domains import (BAC, BOT, DIFF, FRO, INTER, ISOT, LEF, PARALLELEPIPED, PERI, PRISM, PYRAMID, RIG, SPEC,
                      TETRAHEDRON, TOP, TRIANGULAR_PRISM, BulkDomain, CrossPlaneFilmDomain, Domain, FilmDomain,
                      HexDomain, JctDomain, OctetDomain, Pair, Parallelepiped, PoreCellDomain, Prism, PyrDomain, Pyramid,
                      TeeDomain, Tetrahedron, TriangularPrism, TubeDomain)
from .materials import SiliconModel, silicon_tables, write_material_files
from .problem import (CUMFLUX, CUMTEMP, FLUX, MULTI, TEMP, CumFluxProblem, CumTempProblem, FluxProblem,
                      Material, MultiProblem, Session, TempProblem, kappa_from_flux)

__all__ = [
    "BAC", "LEF", "BOT", "FRO", "RIG", "TOP", "SPEC", "DIFF", "ISOT", "PERI", "INTER",
    "Domain", "FilmDomain", "BulkDomain", "CrossPlaneFilmDomain", "PoreCellDomain", "PyrDomain", "HexDomain",
    "JctDomain", "TeeDomain", "TubeDomain", "OctetDomain", "Pair", "Parallelepiped", "TriangularPrism", "Tetrahedron", "Prism",
    "Pyramid", "PARALLELEPIPED", "TRIANGULAR_PRISM", "TETRAHEDRON", "PRISM", "PYRAMID", "SiliconModel", "silicon_tables", "write_material_files", "Material",
    "TempProblem", "FluxProblem", "MultiProblem", "CumTempProblem", "CumFluxProblem", "Session", "TEMP",
    "FLUX", "MULTI", "CUMTEMP", "CUMFLUX",
    "kappa_from_flux", "Batch", "Server",
]
