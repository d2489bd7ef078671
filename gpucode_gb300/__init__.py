"""GB300-native DEM sphere-packing engine (libdem_gb300).

The product is the CUDA library gpucode_gb300/libdem_gb300.so (sm_103a kernels
behind the C ABI of include/heydem_gb300.h).  This package binds it:

  engine.Setup / engine.Engine  -- the native dem_* API
  capnet.CapNet                 -- the learned capillary closure (dem_capnet_*)
  configs                       -- synthetic packing workloads
  build.build()                 -- compile the library in-tree with nvcc
"""
from ._abi import DemError, load  # noqa: F401
from .capnet import CapNet  # noqa: F401
from .engine import Engine, Setup  # noqa: F401

__all__ = ["Engine", "Setup", "CapNet", "DemError", "load"]
