"""GB300-native drop-in for the pseudospectral RHS / timestepping hot path of
dedalus-1.0 (Fourier and shearing-box Fourier representations,
IncompressibleHydro / BoussinesqHydro / IncompressibleMHD physics with shear
and rotation, RK2mid / RK2trap / RK4 integrators), plus a learned subgrid
closure for 64^3 LES (``closure``, ``physics.LESHydro``).

Import name ``dedalus_gb300`` (the directory name is not a Python identifier;
``__graft_entry__.load_package()`` registers it).  All compute runs in
hand-written sm_103a CUDA kernels in ``libdd_gb300.so`` reached through the C
ABI in ``include/dd_gb300.h``; PyTorch provides device buffers and streams.
"""
from . import _lib
from . import kgrid
from . import config
from . import init_cond

try:  # the device layers need torch; host helpers (kgrid, init_cond) do not
    from . import engine
    from . import representations
    from . import fields
    from . import physics
    from . import time_step
    from . import mods
    from . import diagnostics
    from . import ensemble
    from . import closure
    from . import restart
    from . import generic
except ImportError as e:  # pragma: no cover
    if "torch" not in str(e):
        raise

__all__ = ["_lib", "kgrid", "config", "init_cond", "engine", "representations", "fields", "physics",
           "time_step", "mods", "diagnostics", "ensemble", "closure", "restart", "generic"]
