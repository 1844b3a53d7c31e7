"""GB300-native Demo4 SPH step (Clavet-style double-density relaxation).

A drop-in for the data-oriented Demo4 solver of f1nalspace/nbodysimulation_experiment
(NBodySimulation/demo4.cpp): the same scene, particle, body and parameter
interface (``BaseSimulation``, NBodySimulation/base.h:8-38), with the step
computed by hand-written CUDA kernels for sm_103a behind the C ABI of
``include/sph_gb300.h``.  ``Simulation`` is the Python face of that ABI;
``BatchSimulation`` advances many independent scenes with one update.
"""
from ._build import build, LIB_PATH
from .simulation import (
    BatchSimulation,
    Domain,
    Mpnn,
    Params,
    SphError,
    Simulation,
    Stats,
    default_params,
    load_library,
    reference_domain,
)
from . import scenes

__all__ = [
    "BatchSimulation", "Domain", "Mpnn", "Params", "SphError", "Simulation", "Stats", "build", "default_params", "load_library",
    "reference_domain", "scenes", "LIB_PATH",
]
