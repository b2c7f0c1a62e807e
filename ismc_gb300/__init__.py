"""ismc_gb300 -- GB300-native integrating-sphere Monte Carlo photon propagator.

Public surface:
  Engine, Layer, Spheres, make_instance, Result   (ismc_gb300.api)
  ismc_gb300.dropin.ISMC.ISMC / ismc_gb300.dropin.ISMLMC.ISMLMC
      drop-in replacements for the reference's ISMC.py / ISMLMC.py entry points
The compute path is libismc.so (hand-written sm_103a CUDA behind a C ABI,
include/ismc.h); build it with ``python -m ismc_gb300.build``.
"""
from .api import (Engine, IsmcError, Layer, Result, Spheres, cap_fraction, default_engine,
                  instance_array, load_library, make_instance, make_solve, make_stack, make_spheres, make_tune,
                  merge_tallies, split_instance, tally_to_result)
from . import _abi

__all__ = ["Engine", "IsmcError", "Layer", "Result", "Spheres", "cap_fraction", "default_engine",
           "instance_array", "load_library", "make_instance", "make_solve", "make_stack", "make_spheres",
           "make_tune", "merge_tallies", "split_instance", "tally_to_result", "_abi"]
