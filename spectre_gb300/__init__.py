"""GB300-native DG scalar-wave evolution hot path (SpECTRE drop-in for one GPU)."""
from .dgsw import (Brick, DgEvolution, DgswError, Rk3HesthavenSsp, ScalarWaveSystem,
                   UpwindPenalty, differentiation_matrix, index_maps, lgl_points_weights,
                   mortar_projections, PRECISION_FP64, PRECISION_MIXED, PRECISION_DOUBLE_FLOAT)

__all__ = ["Brick", "DgEvolution", "DgswError", "Rk3HesthavenSsp", "ScalarWaveSystem",
           "UpwindPenalty", "differentiation_matrix", "index_maps", "lgl_points_weights",
           "mortar_projections", "PRECISION_FP64", "PRECISION_MIXED", "PRECISION_DOUBLE_FLOAT"]
