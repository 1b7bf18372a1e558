"""GB300-native time-step engine for the 2-D mantle-convection code
mingming-li/Mantle_Convection_Lab: Uzawa Stokes solve with inner CG on the Q1/P0
viscous operator (with quadtree hanging-node constraints), the SUPG
temperature update, and the viscosity and buoyancy loops that feed them.

The product is libmclg.so (C ABI, include/mclg.h) and the mclg_run driver;
this package holds their sources (csrc/), the in-tree build (_build.py) and a
ctypes binding (api.py).
"""
from .api import Cnn, Config, Ensemble, GrainSize, Mesh, Model, MclgError, StepStats, lib  # noqa: F401
