"""GB300-native drop-in for the pseudospectral RHS / timestepping hot path of
dedalus-1.0 (Fourier representation, IncompressibleHydro / BoussinesqHydro /
IncompressibleMHD physics, RK2mid / RK2trap / RK4 integrators).

Import name ``dedalus_gb300`` (the directory name is not a Python identifier;
``__graft_entry__.load_package()`` registers it).  All compute runs in
hand-written sm_103a CUDA kernels in ``libdd_gb300.so`` reached through the C
ABI in ``include/dd_gb300.h``; PyTorch provides device buffers and streams.
"""
from . import _lib
from . import kgrid
from . import engine

__all__ = ["_lib", "kgrid", "engine"]
