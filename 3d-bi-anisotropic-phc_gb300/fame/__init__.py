"""FAME GB300: nullspace-free FFT eigensolver for 3D bi-anisotropic photonic
crystals on one GB300 (sm_103a).

The numerical work lives in the CUDA library ``libfame_gb300.so`` (C ABI in
``include/fame.h``); this package is the host-side mirror of the reference's
MATLAB handles (``fncA``, ``fncB``, ``fncinvB``, ``MtxVecMul_FFT``,
``Lanczos``) plus the problem setup.
"""
from ._lib import FameError, lib_path, load  # noqa: F401
from . import adjoint  # noqa: F401
from .handles import Lanczos, Lanczos_gep, MtxVecMul_FFT, fncA, fncB, fncinvB, woodpile_plan  # noqa: F401
from .plan import Plan  # noqa: F401
from .setup import (band_path, bi_isotropic, bloch_angles, constitutive, covariant_blocks,  # noqa: F401
                    fcc_lattice, fcc_point, rasterize, reference_path, sphere_inside, tetra_inside, vertex_positions,
                    woodpile_inside)
from . import interior  # noqa: F401
