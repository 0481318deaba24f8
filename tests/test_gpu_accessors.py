"""Dense accessors through the GPU transforms, against the reference's own
outputs (tests/golden/accessors.npz): ``array``, ``getCols`` / ``getRows``,
``A[i, j]`` and the other ``__getitem__`` forms, ``colNorms`` /
``rowNorms``, the normalized operators, ``gram``, the spectral helpers and
the solver-backed ``Inverse`` / ``PseudoInverse``
(fastmat/inspect/test.py:444-700 test the same accessors)."""

import numpy as np
from scipy.sparse import csr_matrix
import pytest

from oracle import fm_oracle as fo
from tests.golden_cases import load_accessors, load_cases

pytestmark = pytest.mark.gpu

ACC = load_accessors()
CASES = [c for c in load_cases() if c.name in ACC]


def _ns():
    import fastmat_gb300 as fg
    return dict(Fourier=fg.Fourier, Circulant=fg.Circulant,
                Toeplitz=fg.Toeplitz, Hadamard=fg.Hadamard, Kron=fg.Kron,
                Diag=fg.Diag, Partial=fg.Partial,
                Permutation=fg.Permutation, Product=fg.Product, Sum=fg.Sum,
                Hermitian=fg.Hermitian, Conjugate=fg.Conjugate,
                Transpose=fg.Transpose, Eye=fg.Eye, Matrix=fg.Matrix,
                Blocks=fg.Blocks, BlockDiag=fg.BlockDiag,
                Sparse=fg.Sparse, csr=csr_matrix, np=np)


def _tol(ref):
    # double-precision results: 1e-12 of the largest entry (fastmat's
    # max|out - ref| / max|ref| metric); integer results exactly
    return 0 if np.issubdtype(ref.dtype, np.integer) else 1e-12


def _same(out, ref):
    out, ref = np.asarray(out), np.asarray(ref)
    assert out.shape == ref.shape, (out.shape, ref.shape)
    if _tol(ref) == 0:
        return np.array_equal(out, ref)
    return fo.rel_err(out, ref) <= 1e-12


@pytest.mark.parametrize('case', CASES, ids=lambda c: c.name)
def test_array_rows_cols_items(case):
    acc = ACC[case.name]
    op = case.build(_ns())
    ci, ri = acc['colidx'], acc['rowidx']
    a = op.array
    assert a.dtype == acc['array'].dtype
    # formed on the GPU (a dense Matrix returns its own array)
    assert op._array is not None or a.flags.f_contiguous
    assert _same(a, acc['array'])
    # a fresh operator (no cached array): columns, rows and elements come
    # from unit vectors on the GPU
    op = case.build(_ns())
    cols = op.getCols(ci)
    assert cols.dtype == acc['cols'].dtype and _same(cols, acc['cols'])
    rows = op.getRows(ri)
    assert rows.dtype == acc['rows'].dtype and _same(rows, acc['rows'])
    items = np.array([op[int(i), int(j)] for i in ri for j in ci])
    assert _same(items, acc['items'])
    assert _same(op.getCol(int(ci[-1])), acc['cols'][:, -1])
    assert _same(op.getRow(int(ri[0])), acc['rows'][0])
    assert op.getCols(int(ci[0])).ndim == 1 and op.getRows(0).ndim == 1


@pytest.mark.parametrize('case', CASES, ids=lambda c: c.name)
def test_norms_and_normalized(case):
    acc = ACC[case.name]
    op = case.build(_ns())
    cn, rn = op.colNorms, op.rowNorms
    # float64, except the closed forms of Diag / Eye / Permutation
    assert cn.dtype == acc['colnorms'].dtype
    assert rn.dtype == acc['rownorms'].dtype
    scale = max(1e-300, float(np.max(np.abs(acc['array']))))
    assert np.allclose(cn, acc['colnorms'], rtol=1e-12, atol=1e-12 * scale)
    assert np.allclose(rn, acc['rownorms'], rtol=1e-12, atol=1e-12 * scale)
    if 'colnormalized' in acc:
        assert fo.rel_err(op.colNormalized.array,
                          acc['colnormalized']) <= 1e-12
    if 'rownormalized' in acc:
        assert fo.rel_err(op.rowNormalized.array,
                          acc['rownormalized']) <= 1e-12
    # zero-norm columns / rows: the reference raises, so must we
    if 'colnormalized_raises' in acc:
        with pytest.raises(ValueError):
            op.colNormalized
    if 'rownormalized_raises' in acc:
        with pytest.raises(ValueError):
            op.rowNormalized


def test_getitem_forms():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(5)
    c = rng.standard_normal(12) + 1j * rng.standard_normal(12)
    ref = fo.Circulant(c).dense()
    # a rectangular composite: 5 rows of the circulant
    rows = np.array([0, 3, 4, 7, 11])
    P = fg.Partial(fg.Circulant(c), rows=rows)
    d = ref[rows]
    assert fo.rel_err(P[...], d) <= 1e-12
    assert fo.rel_err(P[:, :], d) <= 1e-12
    assert abs(P[2, 5] - d[2, 5]) <= 1e-12 * np.abs(d).max()
    assert fo.rel_err(P[1, :], d[1, :]) <= 1e-12
    assert fo.rel_err(P[:, 4], d[:, 4]) <= 1e-12
    assert fo.rel_err(P[1:4, ...], d[1:4]) <= 1e-12
    assert fo.rel_err(P[..., 2:9:3], d[:, 2:9:3]) <= 1e-12
    assert fo.rel_err(P[[0, 4], 3:7], d[[0, 4]][:, 3:7]) <= 1e-12
    assert fo.rel_err(P[1:5, [2, 8, 9, 10, 11, 0]],
                      d[1:5][:, [2, 8, 9, 10, 11, 0]]) <= 1e-12
    assert fo.rel_err(P[[3], :], d[3]) <= 1e-12
    with pytest.raises(IndexError):
        P.getCol(12)
    with pytest.raises(IndexError):
        P.getRow(-1)
    with pytest.raises(IndexError):
        P.getCols([0, 12])
    with pytest.raises(TypeError):
        P.getCol([1, 2])
    with pytest.raises(IndexError):
        P[1, 2, 3]
    with pytest.raises(TypeError):
        P[[0.5, 1.0], :]


def test_integer_array_and_many_blocks():
    import fastmat_gb300 as fg
    H = fg.Hadamard(7)
    a = H.array
    assert a.dtype == np.int8
    assert np.array_equal(a, fo.Hadamard(7).dense().astype(np.int8))
    # blocks of a few columns per engine call: same result
    H2 = fg.Hadamard(7)
    H2._UNIT_BLOCK_BYTES = 128 * 9 * 3
    assert np.array_equal(H2.array, a)
    assert np.allclose(H2.colNorms, np.sqrt(128.0), rtol=1e-15)


def test_gram_and_spectral_helpers():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(8)
    c = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    C = fg.Circulant(c)
    d = fo.Circulant(c).dense()
    assert fo.rel_err(C.gram.array, d.conj().T @ d) <= 1e-12
    ev = np.linalg.eigvals(d)
    assert abs(abs(C.largestEigenValue) - np.abs(ev).max()) <= 1e-9 * np.abs(
        ev).max()
    v = fg.Circulant(c).largestEigenVec
    lam = fg.Circulant(c).largestEigenValue
    assert np.linalg.norm(d @ v - lam * v) <= 1e-8 * abs(lam)
    s = np.linalg.svd(d, compute_uv=False)
    u, vh = fg.Circulant(c).largestSingularVectors
    assert u.shape == (40, 1) and vh.shape == (1, 40)
    assert np.linalg.norm(d @ vh.conj().T[:, 0] - s[0] * u[:, 0]) <= (
        1e-8 * s[0])


def test_inverse_and_pseudo_inverse():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(9)
    n = 48
    c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    c[0] += 4.0 * n  # eigenvalues 4n +- O(sqrt(n)): well conditioned
    C = fg.Circulant(c)
    d = fo.Circulant(c).dense()
    b = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    # scipy's lgmres stops at a relative residual of 1e-5 (fastmat passes
    # only atol=1e-12)
    x = C.inverse.forward(b)
    assert x.shape == (n, 2)
    assert np.linalg.norm(d @ x - b) <= 1e-5 * np.linalg.norm(b)
    xh = C.inverse.backward(b[:, 0])
    assert xh.shape == (n,)
    assert np.linalg.norm(d.conj().T @ xh - b[:, 0]) <= 1e-5 * np.linalg.norm(
        b[:, 0])
    # a device tensor in, a device tensor out
    import torch
    xt = C.inverse.forward(torch.from_numpy(b).cuda())
    assert xt.is_cuda and tuple(xt.shape) == (n, 2)
    assert np.linalg.norm(d @ xt.cpu().numpy() - b) <= 1e-5 * np.linalg.norm(b)
    rows = np.sort(rng.choice(n, 30, replace=False))
    P = fg.Partial(C, rows=rows)
    y = P.pseudoInverse.forward(b[rows, 0])
    ref = np.linalg.lstsq(d[rows], b[rows, 0], rcond=None)[0]
    assert np.linalg.norm(y - ref) <= 1e-6 * np.linalg.norm(ref)
    assert fo.rel_err(C.inverse.reference(), np.linalg.inv(d)) <= 1e-10
    with pytest.raises(ValueError):
        fg.Inverse(P)
    with pytest.raises(NotImplementedError):
        fg.Product(C.inverse, C).forward(b)
