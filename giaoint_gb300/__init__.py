"""GB300-native GIAO electron-repulsion integrals.

A drop-in for the electron-repulsion path of GIAOINT (``giao_integrals``):
complex London-orbital shell-quartet ERIs by McMurchie-Davidson, the complex
Boys function, and the streamed pivoted-Cholesky ERI generator, computed by
hand-written sm_103a CUDA kernels behind the C ABI of include/giao_gb300.h.
The names, signatures and error types below follow the reference module.
"""

from ._native import BoysNumericalError
from ._threads import build_info, resolve_num_threads, set_num_threads
from ._types import (
    Basis,
    CartesianExponent,
    MagneticField,
    Nucleus,
    PrimitiveGaussian,
    Shell,
    cartesian_components,
    primitive_normalization,
)
from .boys import BoysRegion, boys, boys_with_diagnostics
from .cholesky import CholeskyERI, cholesky_eri
from .derivative_assembly import eri_derivative_contraction
from .eri import (
    EriBatch,
    EriDerivativeBatch,
    canonical_quartets,
    eri,
    eri_batches,
    eri_center_derivatives_shell,
    eri_derivative_batches,
    eri_magnetic_derivatives_shell,
    eri_mixed_derivatives_shell,
    eri_schwarz_bounds,
    eri_shell,
    primitive_eri,
    primitive_eri_center_derivatives,
    primitive_eri_magnetic_derivatives,
    primitive_eri_mixed_derivatives,
)
from .molecule import Molecule
from .nuclear import nuclear_attraction, nuclear_attraction_shell, primitive_nuclear_attraction

__version__ = "0.1.0"

__all__ = [
    "Basis",
    "BoysNumericalError",
    "BoysRegion",
    "CartesianExponent",
    "CholeskyERI",
    "EriBatch",
    "EriDerivativeBatch",
    "MagneticField",
    "Molecule",
    "Nucleus",
    "PrimitiveGaussian",
    "Shell",
    "boys",
    "boys_with_diagnostics",
    "build_info",
    "canonical_quartets",
    "cartesian_components",
    "cholesky_eri",
    "eri",
    "eri_batches",
    "eri_center_derivatives_shell",
    "eri_derivative_contraction",
    "eri_derivative_batches",
    "eri_magnetic_derivatives_shell",
    "eri_mixed_derivatives_shell",
    "eri_schwarz_bounds",
    "eri_shell",
    "nuclear_attraction",
    "nuclear_attraction_shell",
    "primitive_eri",
    "primitive_eri_center_derivatives",
    "primitive_eri_magnetic_derivatives",
    "primitive_eri_mixed_derivatives",
    "primitive_nuclear_attraction",
    "primitive_normalization",
    "resolve_num_threads",
    "set_num_threads",
]
