"""Host-side logic of the drop-in package (no GPU needed): dense references,
type promotion, FFT-size attributes, argument errors and the C ABI exports.
"""

import os
import re

import numpy as np
from scipy.sparse import csr_matrix
import pytest

import fastmat_gb300 as fg
from fastmat_gb300 import _native, fftsize
from oracle import fm_oracle as fo
from tests.golden_cases import load_cases, load_fftsizes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = load_cases()

NS = dict(Fourier=fg.Fourier, Circulant=fg.Circulant, Toeplitz=fg.Toeplitz,
          Hadamard=fg.Hadamard, Kron=fg.Kron, Diag=fg.Diag,
          Partial=fg.Partial, Permutation=fg.Permutation,
          Product=fg.Product, Sum=fg.Sum, Hermitian=fg.Hermitian,
          Conjugate=fg.Conjugate, Transpose=fg.Transpose, Eye=fg.Eye,
          Matrix=fg.Matrix, Blocks=fg.Blocks, BlockDiag=fg.BlockDiag,
          Sparse=fg.Sparse, csr=csr_matrix, np=np)


@pytest.mark.parametrize('case', CASES, ids=lambda c: c.name)
def test_shape_dtype_and_dense_reference(case):
    op = case.build(NS)
    assert op.shape == case.shape
    assert np.dtype(op.dtype) == case.dtype
    # output type contract (fastmat/inspect/test.py:160-170)
    assert np.dtype(op._output_dtype(case.x.dtype)) == case.fwd.dtype or \
        np.dtype(op._output_dtype(case.x.dtype)) == np.dtype(
            fo.promote(case.dtype, case.x.dtype))
    if case.dense is not None:
        d = op.reference()
        assert d.shape == case.dense.shape
        assert fo.rel_err(d, case.dense) <= 1e-12


def test_fft_size_attributes_match_reference():
    g = load_fftsizes()
    sizes = g['sizes']
    assert [fftsize.find_optimal_fft_size(int(n)) for n in sizes] == \
        list(g['opt'])
    numl = [fg.Fourier(int(n))._numL for n in sizes if n <= 70000]
    assert numl == list(g['numl'])


def test_argument_errors():
    C = fg.Circulant(np.ones(8))
    with pytest.raises(ValueError):
        C.forward(np.ones(7))
    with pytest.raises(ValueError):
        C.forward(np.ones((8, 2, 2)))
    with pytest.raises(ValueError):
        fg.Fourier(0)
    with pytest.raises(ValueError):
        fg.Hadamard(0)
    with pytest.raises(ValueError):
        fg.Permutation(np.array([0, 0, 1]))
    with pytest.raises(ValueError):
        fg.Partial(fg.Hadamard(2), rows=np.array([4]))
    with pytest.raises(TypeError):
        fg.Partial(fg.Hadamard(2), rows=np.array([0.5]))
    with pytest.raises(ValueError):
        fg.Kron(fg.Hadamard(2))
    with pytest.raises(ValueError):
        fg.Product(fg.Hadamard(2), fg.Hadamard(3))
    with pytest.raises(ValueError):
        fg.Sum(fg.Hadamard(2), fg.Hadamard(3))
    with pytest.raises(ValueError):
        fg.Toeplitz(np.ones(4))
    with pytest.raises(ValueError):
        fg.Matrix(np.ones(3))


def test_operator_overloads():
    H = fg.Hadamard(2)
    D = fg.Diag(np.arange(4.))
    assert isinstance(H * D, fg.Product)
    assert isinstance(H + D, fg.Sum)
    assert isinstance(H - D, fg.Sum)
    assert isinstance(2 * H, fg.Product)
    assert isinstance(H / 2, fg.Product)
    assert isinstance(H.H, fg.Hermitian)
    F = fg.Fourier(4)
    assert isinstance(F.conj, fg.Conjugate)
    assert H.conj is H
    assert np.allclose((F.T).reference(), F.reference().T)
    assert np.allclose((F.H).reference(), F.reference().conj().T)
    assert np.allclose((H - D).reference(), H.reference() - D.reference())
    # precision option
    assert fg.Fourier(8, precision='fp32')._output_dtype(np.complex128) == \
        np.complex64
    with pytest.raises(ValueError):
        fg.Fourier(8, precision='fp16')


def _declared_symbols():
    with open(os.path.join(ROOT, 'include', 'fmgpu.h')) as f:
        text = f.read()
    return sorted(set(re.findall(r'\b(fm_[a-z_]+)\s*\(', text)))


def test_c_abi_library_exports_every_declared_symbol():
    lib = _native.load()
    declared = _declared_symbols()
    assert set(declared) == set(_native.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.fm_version() >= 100


def test_constants_match_header():
    """Node kinds, element / compute types, directions and status codes of
    the Python binding equal the header's #defines."""
    with open(os.path.join(ROOT, 'include', 'fmgpu.h')) as f:
        defs = dict((k, int(v)) for k, v in re.findall(
            r'#define\s+(FM_[A-Z0-9_]+)\s+(-?\d+)\b', f.read()))
    nodes = {k[len('FM_NODE_'):]: v for k, v in defs.items()
             if k.startswith('FM_NODE_')}
    assert len(nodes) == 16
    for name, v in nodes.items():
        assert getattr(_native, 'NODE_' + name) == v, name
    for name in ('FM_F32_TC', 'FM_F64_DF', 'FM_C128_DF'):
        assert getattr(_native, name) == defs[name], name
    assert (_native.FORWARD, _native.BACKWARD) == (defs['FM_FORWARD'],
                                                  defs['FM_BACKWARD'])
    for dt, name in ((np.int8, 'FM_I8'), (np.int16, 'FM_I16'),
                     (np.int32, 'FM_I32'), (np.int64, 'FM_I64'),
                     (np.float32, 'FM_F32'), (np.float64, 'FM_F64'),
                     (np.complex64, 'FM_C64'), (np.complex128, 'FM_C128')):
        assert _native.DTYPE_CODE[np.dtype(dt)] == defs[name], name


def test_node_struct_layout_matches_header(tmp_path):
    """The ctypes mirrors of fm_node / fm_plan_info have the C layout."""
    import ctypes
    import shutil
    import subprocess
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    src = tmp_path / 'layout.c'
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "fmgpu.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu\\n", sizeof(fm_node),'
        ' offsetof(fm_node, vec1), offsetof(fm_node, scalar_im),'
        ' sizeof(fm_plan_info), offsetof(fm_plan_info, compute_type));'
        ' return 0; }\n')
    exe = tmp_path / 'layout'
    subprocess.run([cc, '-I', os.path.join(ROOT, 'include'), str(src), '-o',
                    str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True,
                                           text=True).stdout.split()]
    assert vals == [ctypes.sizeof(_native.FmNode),
                    _native.FmNode.vec1.offset,
                    _native.FmNode.scalar_im.offset,
                    ctypes.sizeof(_native.FmPlanInfo),
                    _native.FmPlanInfo.compute_type.offset]


def test_block_constructors_validate_like_fastmat():
    """fastmat/Blocks.pyx:65-196 and fastmat/BlockDiag.pyx:95-130."""
    F4, H2, F3 = fg.Fourier(4), fg.Hadamard(2), fg.Fourier(3)
    with pytest.raises(ValueError):
        fg.Blocks(F4)
    with pytest.raises(ValueError):
        fg.Blocks([])
    with pytest.raises(TypeError):
        fg.Blocks([F4, H2])
    with pytest.raises(TypeError):
        fg.Blocks([[F4, np.eye(4)]])
    with pytest.raises(ValueError):
        fg.Blocks([[F4, H2], [H2]])
    with pytest.raises(ValueError):
        fg.Blocks([[F4, F3]])
    with pytest.raises(ValueError):
        fg.Blocks([[F4], [fg.Partial(F3, rows=np.arange(2))]])
    with pytest.raises(ValueError):
        fg.BlockDiag()
    with pytest.raises(ValueError):
        fg.BlockDiag(F4, np.eye(3))
    B = fg.Blocks([[F4, H2], [fg.Diag(np.ones(4)), fg.Eye(4)]])
    assert B.shape == (8, 8) and B.dtype == np.complex128
    assert len(B.content) == 4
    D = fg.BlockDiag(F3, H2, fg.Diag(np.arange(2.0)))
    assert D.shape == (9, 9) and D.dtype == np.complex128
    assert fg.BlockDiag(H2, fg.Eye(2)).dtype == np.int8


def test_accessor_and_solver_argument_errors():
    """Argument checks of the dense accessors, Sparse and the solver-backed
    operators raise before any device work (fastmat/Matrix.pyx:389-658,
    2490-2600; fastmat/Sparse.pyx:95-115)."""
    c = np.arange(1.0, 13.0)
    P = fg.Partial(fg.Circulant(c), rows=np.array([0, 3, 4, 7, 11]))
    with pytest.raises(IndexError):
        P.getCol(12)
    with pytest.raises(IndexError):
        P.getRow(-1)
    with pytest.raises(IndexError):
        P.getCols([0, 12])
    with pytest.raises(IndexError):
        P.getRows(np.array([[0, 1]]))
    with pytest.raises(TypeError):
        P.getCol([1, 2])
    with pytest.raises(IndexError):
        P[1, 2, 3]
    with pytest.raises(IndexError):
        P[()]
    with pytest.raises(IndexError):
        P[1]
    with pytest.raises(TypeError):
        P[[0.5, 1.0], :]
    with pytest.raises(TypeError):
        P[{1: 2}, 0]
    with pytest.raises(TypeError):
        fg.Sparse(np.eye(3))
    with pytest.raises(TypeError):
        fg.Sparse([[1, 0], [0, 1]])
    with pytest.raises(ValueError):
        fg.Inverse(P)
    with pytest.raises(TypeError):
        fg.Inverse(np.eye(3))
    with pytest.raises(TypeError):
        fg.PseudoInverse(np.eye(3))
    C = fg.Circulant(c)
    assert C.inverse.shape == (12, 12) and C.pseudoInverse.shape == (12, 12)
    assert P.pseudoInverse.shape == (12, 5)
    with pytest.raises(NotImplementedError):
        fg.Product(C.inverse, C).forward(np.ones(12))
    wide = fg.Partial(fg.Fourier(4), rows=np.array([0, 1]))
    with pytest.raises(ValueError):
        wide.largestEigenValue
    with pytest.raises(ValueError):
        wide.largestEigenVec
