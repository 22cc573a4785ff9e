"""fastlem_gb300: fastlem's landscape-evolution solve (TerrainGenerator::generate)
on one GB300 GPU, behind a C ABI (include/fastlem_gb300.h) and fastlem's own API.
"""
from .api import (GenerationError, ModelBuilderError, ParameterArrays, Site2D, Terrain2D,
                  TerrainGenerator, TerrainModel2D, TerrainModel2DBulider, TopographicalParameters)
from ._lib import pinned_empty

__all__ = ["GenerationError", "ModelBuilderError", "ParameterArrays", "Site2D", "Terrain2D",
           "TerrainGenerator", "TerrainModel2D", "TerrainModel2DBulider", "TopographicalParameters",
           "pinned_empty"]
