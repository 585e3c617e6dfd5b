"""GB300-native Galerkin hot path of VortexPanel.jl: the host-side mirror of the reference's Julia API over the
C-ABI library ``libvortexpanel_gpu.so`` (hand-written CUDA for sm_103a). No CPU fallback."""
from . import meshes  # noqa: F401
from .api import (AssemblyOptions, DeviceSystem, Elements, GalerkinFactorization, assemble, assemble_batch,  # noqa: F401
                  build_elements, consistency, element_values, factorize_galerkin, gradient_velocity,
                  kutta_joukowski_force, pressure_coefficient, pressure_force, sheet_strengths, solve_galerkin,
                  source_strengths, surface_loads, surface_velocity, trefftz_drag, wake_loads)
from ._build import build  # noqa: F401
from ._lib import Context, SingularError, VPError, default_context  # noqa: F401
