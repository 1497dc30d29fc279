"""GB300-native two-scale weakly compressible SPH (WCSPH) step.

The compute path is hand-written sm_103a CUDA in libtss.so behind a C ABI
(include/tss.h); this package holds the Python host mirror of the reference's
solver interface, the scene generators and the build script.
"""
from ._abi import (TSS_FLAG_Q1_COMPAT, TSS_SCALE_HIGH, TSS_SCALE_LOW, TssConfig, TssError, config_init,
                   load_library)
from .scenes import Scene, make_scene
from .solver import (Batch, CreateParticleBox, CreateParticleBoxCanvas, ParticleSystem, Solver, WCSPHConfig,
                     WCSPHSolver)

__all__ = ["TSS_FLAG_Q1_COMPAT", "TSS_SCALE_HIGH", "TSS_SCALE_LOW", "TssConfig", "TssError", "config_init",
           "load_library", "Scene", "make_scene", "CreateParticleBox", "CreateParticleBoxCanvas", "ParticleSystem",
           "Solver", "Batch", "WCSPHConfig", "WCSPHSolver"]
