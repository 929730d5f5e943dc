"""GB300-native RDME timestep (lattice diffusion, per-voxel reactions, species
counts) of javirk/cell_simulation behind a C ABI (include/cellsim.h)."""
from .native import (CellsimError, PREC_FP32, PREC_FP64, PREC_MIXED, RNG_PHILOX, RNG_REFERENCE, load)
from .simulation import (Ensemble, LatticeParams, RegionType, Simulation, SolverStatisticSample, tiling_kinds,
                         tiling_launches, tiling_variants)

__all__ = ["CellsimError", "Ensemble", "LatticeParams", "RegionType", "Simulation", "SolverStatisticSample",
           "PREC_FP32", "PREC_FP64", "PREC_MIXED", "RNG_PHILOX", "RNG_REFERENCE", "load", "tiling_kinds", "tiling_launches",
           "tiling_variants"]
