"""GB300-native table-mode Kaiser-Bessel NUFFT with the torchkbnufft API.

Drop-in for the table path of mmuckley/torchkbnufft: ``KbNufft``,
``KbNufftAdjoint``, ``KbInterp``, ``KbInterpAdjoint``, ``ToepNufft``,
``calc_toeplitz_kernel``, ``calc_density_compensation_function`` and the
functional ``kb_table_*`` calls keep their signatures, buffers and errors.
All computation runs in hand-written sm_103a CUDA kernels behind the C ABI in
``include/tkbn_gb300.h``; there is no CPU path.
"""

from . import functional, modules
from ._math import absolute, complex_mult, complex_sign, conj_complex_mult, imag_exp, inner_product
from ._setup import init_fn
from .dcomp import calc_density_compensation_function
from .modules import KbInterp, KbInterpAdjoint, KbNufft, KbNufftAdjoint, ToepNufft
from .ragged import RaggedNufft
from .spmat import calc_tensor_spmatrix
from .toep import calc_toeplitz_kernel
from . import autotune
from . import _setup as nufft_utils

__version__ = "0.1.0"


__all__ = [
    "KbInterp",
    "KbInterpAdjoint",
    "KbNufft",
    "KbNufftAdjoint",
    "RaggedNufft",
    "ToepNufft",
    "absolute",
    "calc_density_compensation_function",
    "calc_tensor_spmatrix",
    "calc_toeplitz_kernel",
    "complex_mult",
    "complex_sign",
    "conj_complex_mult",
    "functional",
    "imag_exp",
    "inner_product",
    "modules",
]
