"""GB300-native voxel photon transport with opengate's API (DoseActor path).

    import opengate_gb300 as gate
    sim = gate.Simulation()
    ...
    sim.run()

The transport runs in libgategpu.so (hand-written sm_103a CUDA, C ABI in
include/gate_gpu.h); this package is the host side.
"""

from .api import (Box, DoseActor, GenericSource, HounsfieldUnit_to_material, ImageVolume,  # noqa: F401
                  Simulation, SimulationStatisticsActor)
from .image_io import Image, read_mhd, write_mhd  # noqa: F401
from .units import g4_units  # noqa: F401

__version__ = "0.1.0"
