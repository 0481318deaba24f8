"""Blocks and BlockDiag as single GPU plans (fastmat/Blocks.pyx,
fastmat/BlockDiag.pyx): ragged block sizes (odd lengths, Bluestein sizes),
many columns, nesting inside other composites, device tensors, the
single-precision form and the batched launch, against the oracle."""

import numpy as np
import pytest

from oracle import fm_oracle as fo
from tests.golden_cases import tolerance

pytestmark = pytest.mark.gpu


def _c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _pair(rng, kind, n):
    import fastmat_gb300 as fg
    if kind == 0:
        c = _c(rng, n)
        return fg.Circulant(c), fo.Circulant(c)
    if kind == 1:
        vc, vr = _c(rng, n), _c(rng, n - 1)
        return fg.Toeplitz(vc, vr), fo.Toeplitz(vc, vr)
    if kind == 2:
        return fg.Fourier(n), fo.Fourier(n)
    d = _c(rng, n)
    return fg.Diag(d), fo.Diag(d)


def test_blockdiag_ragged_many_columns():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(21)
    sizes = [1, 2, 7, 64, 97, 128, 300, 1021, 33, 4099, 5, 2048]
    pairs = [_pair(rng, i % 4, n) for i, n in enumerate(sizes)]
    D = fg.BlockDiag(*[p[0] for p in pairs])
    O = fo.BlockDiag(*[p[1] for p in pairs])
    x = _c(rng, D.numCols, 37)
    assert fo.rel_err(D.forward(x), O.forward(x)) <= 1e-12
    g = _c(rng, D.numRows, 5)
    assert fo.rel_err(D.backward(g), O.backward(g)) <= 1e-12
    assert fo.rel_err(D.forward(x[:, 3]), O.forward(x[:, 3])) <= 1e-12


def test_blocks_grid_rectangular_and_nested():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(22)
    a, oa = _pair(rng, 0, 40)
    b, ob = _pair(rng, 2, 40)
    r = np.sort(rng.choice(40, 25, replace=False))
    grid = [[a, fg.Partial(b, rows=np.arange(40), cols=np.arange(40))],
            [fg.Partial(b, rows=r), fg.Partial(a, rows=r)]]
    ogrid = [[oa, fo.Partial(ob, rows=np.arange(40), cols=np.arange(40))],
             [fo.Partial(ob, rows=r), fo.Partial(oa, rows=r)]]
    B, OB = fg.Blocks(grid), fo.Blocks(ogrid)
    assert B.shape == (65, 80)
    x = _c(rng, 80, 6)
    assert fo.rel_err(B.forward(x), OB.forward(x)) <= 1e-12
    g = _c(rng, 65, 3)
    assert fo.rel_err(B.backward(g), OB.backward(g)) <= 1e-12
    # inside other composites: Product with a scalar, Sum, Hermitian, Kron
    P = fg.Product(B.H, 2.0 - 1j, B)
    OP = fo.Product(fo.Hermitian(OB), 2.0 - 1j, OB)
    assert fo.rel_err(P.forward(x), OP.forward(x)) <= 1e-12
    D = fg.BlockDiag(B, fg.Fourier(9))
    OD = fo.BlockDiag(OB, fo.Fourier(9))
    S = fg.Sum(fg.Product(D.H, D), fg.Eye(89))
    OS = fo.Sum(fo.Product(fo.Hermitian(OD), OD), fo.Eye(89))
    y = _c(rng, 89, 4)
    assert fo.rel_err(S.forward(y), OS.forward(y)) <= 1e-12


def test_blocks_device_tensors_and_single_precision():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(23)
    c, d = _c(rng, 256), _c(rng, 256)
    h = fg.Hadamard(8)
    grid = [[fg.Circulant(c), h], [fg.Diag(d), fg.Fourier(256)]]
    ogrid = [[fo.Circulant(c), fo.Hadamard(8)],
             [fo.Diag(d), fo.Fourier(256)]]
    B, OB = fg.Blocks(grid), fo.Blocks(ogrid)
    x = _c(rng, 512, 8)
    xt = torch.from_numpy(x).cuda()
    yt = B.forward(xt)
    assert yt.is_cuda and tuple(yt.shape) == (512, 8)
    assert fo.rel_err(yt.cpu().numpy(), OB.forward(x)) <= 1e-12
    B32 = fg.Blocks(grid, precision='fp32')
    y32 = B32.forward(x.astype(np.complex64))
    assert y32.dtype == np.complex64
    # fastmat's single-precision bound (fastmat/inspect/test.py:176-189)
    assert fo.rel_err(y32, OB.forward(x)) <= tolerance(y32, x)


def test_blockdiag_in_a_batch():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(24)
    items, refs = [], []
    for k in range(5):
        pairs = [_pair(rng, (k + i) % 4, int(n))
                 for i, n in enumerate(rng.integers(3, 400, size=3))]
        D = fg.BlockDiag(*[p[0] for p in pairs])
        OD = fo.BlockDiag(*[p[1] for p in pairs])
        x = _c(rng, D.numCols, 2)
        items.append((D, torch.from_numpy(x.T.copy()).cuda().t()))
        refs.append(OD.forward(x))
    outs = fg.Batch(items).run()
    for y, ref in zip(outs, refs):
        assert fo.rel_err(y.cpu().numpy(), ref) <= 1e-11


def test_sparse_shapes_types_and_composites():
    """fastmat/Sparse.pyx: CSR products in both directions, every lane
    group width, empty rows and columns, integer wrap-around, and sparse
    factors inside Blocks / Product / Sum."""
    import scipy.sparse as sps
    import fastmat_gb300 as fg
    rng = np.random.default_rng(25)
    for rows, cols, dens in [(1, 1, 1.0), (300, 7, 0.3), (7, 3000, 0.4),
                             (500, 400, 0.01), (64, 64, 0.0),
                             (1000, 1000, 0.03)]:
        a = (sps.random(rows, cols, density=dens, random_state=rng) +
             1j * sps.random(rows, cols, density=dens, random_state=rng))
        S, O = fg.Sparse(a), fo.Sparse(a)
        x = _c(rng, cols, 3)
        g = _c(rng, rows, 2)
        ref = O.forward(x)
        y = S.forward(x)
        assert y.dtype == np.complex128
        assert fo.rel_err(y, ref) <= 1e-12 or np.abs(ref).max() == 0
        assert fo.rel_err(S.backward(g), O.backward(g)) <= 1e-12 or (
            np.abs(O.backward(g)).max() == 0)
    # integers wrap like fastmat's typed loops
    ai = sps.random(40, 30, density=0.5, random_state=rng,
                    data_rvs=lambda k: rng.integers(-100, 100, k)).astype(
                        np.int8)
    xi = rng.integers(-100, 100, (30, 4)).astype(np.int8)
    yi = fg.Sparse(ai).forward(xi)
    assert yi.dtype == np.int8
    assert np.array_equal(yi, fo.Sparse(ai).forward(xi))
    # in composites
    a = sps.random(50, 50, density=0.1, random_state=rng).astype(np.complex128)
    c = _c(rng, 50)
    S, O = fg.Sparse(a), fo.Sparse(a)
    B = fg.Blocks([[S, fg.Circulant(c)], [fg.Eye(50), S.H]])
    OB = fo.Blocks([[O, fo.Circulant(c)], [fo.Eye(50), fo.Hermitian(O)]])
    x = _c(rng, 100, 5)
    assert fo.rel_err(B.forward(x), OB.forward(x)) <= 1e-12
    assert fo.rel_err(B.backward(x), OB.backward(x)) <= 1e-12
    P = fg.Sum(fg.Product(S, fg.Fourier(50)), fg.Diag(c))
    OP = fo.Sum(fo.Product(O, fo.Fourier(50)), fo.Diag(c))
    assert fo.rel_err(P.forward(x[:50]), OP.forward(x[:50])) <= 1e-12
    # single precision
    S32 = fg.Sparse(a, precision='fp32')
    y32 = S32.forward(x[:50].astype(np.complex64))
    assert y32.dtype == np.complex64
    assert fo.rel_err(y32, O.forward(x[:50])) <= tolerance(y32, x[:50])
