"""bubbles_gb300 -- GB300-native (sm_103a) Bubbles 3D SPH / PCISPH particle step.

The compute path is libbbg.so (hand-written CUDA kernels behind the C ABI in
include/bbg.h); this package only binds it.  There is no CPU fallback: without the
library or a CUDA device every call raises `BbgError`.
"""
from ._native import BbgError, device_count, load  # noqa: F401
from . import _native as native  # noqa: F401
from .solver import (BatchSolver, PciSphSolver3, Solver, SphSolver3, build_grid,  # noqa: F401
                     compute_delta_denom, compute_mass, desc_from_scene, format_g,
                     frame_section, reconstruct_surface, surface_scene)
from . import scenes  # noqa: F401

FIELD_POSITION = native.FIELD_POSITION
FIELD_VELOCITY = native.FIELD_VELOCITY
FIELD_FORCE = native.FIELD_FORCE
FIELD_INTERACTION = native.FIELD_INTERACTION
FIELD_DENSITY = native.FIELD_DENSITY
FIELD_PRESSURE = native.FIELD_PRESSURE
FIELD_PRED_POSITION = native.FIELD_PRED_POSITION
FIELD_PRESSURE_FORCE = native.FIELD_PRESSURE_FORCE
FIELD_PRED_DENSITY = native.FIELD_PRED_DENSITY
FIELD_DENSITY_ERROR = native.FIELD_DENSITY_ERROR
FIELD_DIVERGENCE = native.FIELD_DIVERGENCE
FRAME_POSITION = native.FRAME_POSITION
FRAME_VELOCITY = native.FRAME_VELOCITY
FRAME_DENSITY = native.FRAME_DENSITY
FRAME_MASS = native.FRAME_MASS
