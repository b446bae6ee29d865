"""GB300-native particle DEM step of BMX (BoltzmannMFX).

The product is libbmxg.so: hand-written sm_103a CUDA kernels behind the C ABI
of include/bmxg.h, standing behind BMXParticleContainer::EvolveParticles
(src/des/bmx_pc_interaction.cpp:13-495).  This package holds its sources
(csrc/), the build script, the ctypes binding and the seeded workload
generators.
"""
from . import abi, configs  # noqa: F401
from .abi import Geometry, Params, Particles  # noqa: F401
from .runtime import BmxgError, Context, load_library  # noqa: F401
