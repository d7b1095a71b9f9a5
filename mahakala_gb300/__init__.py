"""mahakala_gb300 -- GB300-native (sm_103a) per-ray black-hole imaging path.

Drop-in for the reference package ``mahakala``: the same public names
(mahakala/__init__.py:25-45), with every compute step in hand-written CUDA
kernels behind a C ABI (``include/mahakala_gb300.h``).  FP64 throughout, as
the reference enables ``jax_enable_x64``.  Arrays come back as float64 CUDA
tensors; ``make_image`` returns a NumPy image like the reference.

Importing this package does not need a GPU; calling any compute function
does, and fails loudly without one (there is no CPU fallback).
"""

from .geodesics import (find_shadow_bisection, find_shadow_bisection_angles, geodesic_integrator,
                        initialize_geodesics_at_camera)
from .transfer import solve_attenuated_emissivity, solve_specific_intensity, synchrotron_coefficients

__all__ = [
    "find_shadow_bisection",
    "find_shadow_bisection_angles",
    "geodesic_integrator",
    "initialize_geodesics_at_camera",
    "synchrotron_coefficients",
    "solve_specific_intensity",
    "solve_attenuated_emissivity",
]

__version__ = "0.1.0"
