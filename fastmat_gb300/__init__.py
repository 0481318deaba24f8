"""fastmat_gb300: fastmat's structured-operator matvec path on GB300.

Drop-in classes with fastmat's constructors and ``forward``/``backward``/
``reference`` API, backed by hand-written sm_103a CUDA kernels behind a C ABI
(include/fmgpu.h).
"""

from .matrix import (Conjugate, Hermitian, Inverse, Matrix, PseudoInverse,
                     Transpose)
from .operators import (BlockDiag, Blocks, Circulant, Diag, Eye, Fourier,
                        Hadamard, Kron, Partial, Permutation, Product,
                        Sparse, Sum, Toeplitz)
from . import _native
from . import algorithms
from .batch import Batch
from ._build import build

__version__ = '0.1.0'

__all__ = ['Matrix', 'Hermitian', 'Conjugate', 'Transpose', 'Fourier',
           'Circulant', 'Toeplitz', 'Hadamard', 'Diag', 'Eye', 'Partial',
           'Permutation', 'Product', 'Sum', 'Kron', 'Blocks', 'BlockDiag',
           'Sparse',
           'Inverse', 'PseudoInverse',
           'Batch', 'build']


def native_library():
    """Path of the loaded native library (loads it on first call)."""
    _native.load()
    return _native.library_path()
