"""openrbc_gb300 -- GB300 (sm_103a) implementation of OpenRBC's per-timestep path.

The product is the CUDA library liborbc_gpu.so (C ABI in include/orbc_gpu.h);
this package is its host-side mirror of the reference's interface
(RTParameter, the containers, the step loop) and its build script.
"""
from .runtime_parameter import ParameterError, RTParameter
from .simulation import Simulation, morton_encode, morton_order, rdf_table, write_rdf
from ._native import OrbcError

__all__ = ["RTParameter", "ParameterError", "Simulation", "OrbcError", "morton_encode", "morton_order", "rdf_table",
           "write_rdf"]
