"""Facade mirroring ``dedalus.mods`` (dedalus/mods.py:24-101) for the names a
run script of the hot path uses:

    from dedalus_gb300.mods import *
    RHS = IncompressibleHydro(shape, FourierRepresentation)
    data = RHS.create_fields(0.)
    ti = RK4(RHS)
    while ti.ok:
        ti.advance(data, dt)
"""
from .config import decfg
from .representations import (FourierRepresentation, GpuFourierRepresentation, FourierShearRepresentation,
                              GpuFourierShearRepresentation)
from .physics import Physics, IncompressibleHydro, BoussinesqHydro, IncompressibleMHD, LESHydro
from .time_step import RK2mid, RK2trap, RK4
from .fields import StateData, create_field_classes
from .kgrid import swap_indices
from . import init_cond
from .restart import restart

__all__ = ["decfg", "FourierRepresentation", "GpuFourierRepresentation", "FourierShearRepresentation",
           "GpuFourierShearRepresentation", "Physics", "IncompressibleHydro",
           "BoussinesqHydro", "IncompressibleMHD", "LESHydro", "RK2mid", "RK2trap", "RK4", "StateData",
           "create_field_classes", "swap_indices", "init_cond", "restart"]
