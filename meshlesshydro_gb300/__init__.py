"""meshlesshydro-gb300: the MFV timestep of jammartin/meshlessHydro on GB300.

The compute path is libmlh.so (hand-written sm_103a CUDA behind the C ABI of
include/mlh.h); `runtime.Simulation` is its Python binding.  Building:
`meshlesshydro_gb300.build.build()`.
"""
from .config import MFVConfig  # noqa: F401

__version__ = "0.1.0"
