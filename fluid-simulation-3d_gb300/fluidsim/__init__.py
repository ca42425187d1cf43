"""GB300 SPH substep library: Python side of the C ABI (include/sph_gb300.h).

The compute path is libsph_gb300.so (hand-written sm_103a CUDA); this
package only binds it (`_lib`), mirrors the reference's simulation class and
plug-in (`simulation`), builds the seeded benchmark scenes (`scenes`) and
the camera views of the headless render (`render`).
"""
from . import render, scenes
from ._lib import LIB_PATH, SphError, load
from .simulation import (Batch, FluidSimCUDA, FluidSimulation, default_params,
                         grid_arrangement, to_params)

__all__ = ["Batch", "FluidSimCUDA", "FluidSimulation", "SphError", "LIB_PATH",
           "default_params", "grid_arrangement", "load", "render", "scenes", "to_params"]
