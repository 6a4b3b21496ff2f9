"""GB300 finite-volume RK stage of the Clemson Kilonova Code (host side).

The compute path is the CUDA library app-kilonova_gb300/_build/libknc_gpu.so
behind the C ABI in include/knc.h; this package is its Python host.
"""
from . import abi
from .config import (Control, JetModel, Mesh, NewtonianHydro, RelativisticHydro, SphereModel,
                     WindModel, ConfigError)
from .solver import HydroError, Solver, build_solver, measure_fp64_peak

__all__ = ["abi", "Control", "JetModel", "Mesh", "NewtonianHydro", "RelativisticHydro", "SphereModel",
           "WindModel", "ConfigError", "HydroError", "Solver", "build_solver", "measure_fp64_peak"]
