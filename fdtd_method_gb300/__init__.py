"""GB300-native (sm_103a) engine for the 3-D Yee FDTD step of
Amazingkivas/FDTD_Method, behind the reference solver class's API.

    from fdtd_method_gb300 import FDTD, Parameters, Component
    sim = FDTD(Parameters(...), dt)          # FP64 drop-in
    sim.get_field(Component.EY).assign(e0)
    sim.update_fields()
    ey = sim.get_field(Component.EY).numpy()
"""
from .fdtd import (FDTD, FDTD_PML, FDTDBatch, Axis, Component, Const, CurrentParameters, Field, FDTDError,  # noqa: F401
                   InvalidArgument, LogicError, OutOfMemory, Parameters, Precision,
                   SelectedFields, SeparableSource, fp16_choose_exponents)
from . import sources  # noqa: F401
from .slabs import FDTDSlabs, Slab  # noqa: F401

__all__ = ["FDTD", "FDTD_PML", "FDTDBatch", "Axis", "Component", "Const", "CurrentParameters", "Field", "FDTDError",
           "InvalidArgument", "LogicError", "OutOfMemory", "Parameters", "Precision",
           "SelectedFields", "SeparableSource", "fp16_choose_exponents", "sources", "FDTDSlabs", "Slab"]
