"""A circulant Kron mode and the Hadamard mode before it in one launch
(rkch_kernel, fm_rpair.cuh): the convolution on contiguous vectors, then
the strided FWHT in place, block by block so each block is still in L2
(fastmat/Kron.pyx:284-300 applies the factors mode by mode), complex64.
Against the oracle in the FP32 form (1e-5; the double-float form, which
keeps two launches, at 1e-12), both directions, several columns and a
padded leading dimension, the numpy path (whose chunked host pipeline runs
the pair as two launches), and the separate launches for what the fused
launch is not built for."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _fused(op, dt):
    d = op.plan(dt).describe(0)
    return 'rconv' in d and 'fused-with-next' in d


@pytest.mark.parametrize('k,n', [(8, 128), (7, 128), (8, 256), (7, 256)])
@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_kron_hadamard_circulant(k, n, prec):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(k * 1000 + n)
    c = cplx(rng, n)
    op = fg.Kron(fg.Hadamard(k), fg.Circulant(c), precision=prec)
    oop = fo.Kron(fo.Hadamard(k), fo.Circulant(c))
    dt = np.complex128 if prec == 'native' else np.complex64
    # (complex64 only: the double-float form runs the two launches)
    assert _fused(op, dt) == (prec == 'fp32')
    x = cplx(rng, op.numCols, 5)
    if prec == 'native':
        x[::9] *= 1e-150
    tol = 1e-12 if prec == 'native' else 1e-5
    y = op.forward(x)
    assert y.dtype == dt
    assert fo.rel_err(y, oop.forward(x)) <= tol
    assert fo.rel_err(op.backward(x), oop.backward(x)) <= tol


@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_three_modes_padded_leading_dimension(prec):
    """Fourier, Hadamard and Circulant modes (the Kron workload's shape):
    the F mode runs after the fused pair; columns with a padded leading
    dimension."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(21)
    c = cplx(rng, 128)
    op = fg.Kron(fg.Fourier(16), fg.Hadamard(8), fg.Circulant(c),
                 precision=prec)
    oop = fo.Kron(fo.Fourier(16), fo.Hadamard(8), fo.Circulant(c))
    dt = np.complex128 if prec == 'native' else np.complex64
    assert _fused(op, dt) == (prec == 'fp32')
    n = op.numCols
    big = torch.from_numpy(cplx(rng, 3, n + 8).astype(dt)).cuda()
    xt = big[:, :n].t()                  # leading dimension n + 8
    y = op.forward(xt).cpu().numpy()
    x = xt.cpu().numpy()
    tol = 1e-12 if prec == 'native' else 1e-5
    assert fo.rel_err(y, oop.forward(x.astype(np.complex128))) <= tol


def test_lengths_outside_the_fused_launch_run_separately():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(22)
    c = cplx(rng, 64)
    op = fg.Kron(fg.Hadamard(8), fg.Circulant(c), precision='fp32')
    oop = fo.Kron(fo.Hadamard(8), fo.Circulant(c))
    assert not _fused(op, np.complex64)
    x = cplx(rng, op.numCols, 3)
    assert fo.rel_err(op.forward(x), oop.forward(x)) <= 1e-5


def test_host_pipeline_runs_the_pair_as_two_launches():
    """numpy input (fm_execute_host, column chunks over copy streams): the
    same result as the device call that runs the fused launch."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(23)
    c = cplx(rng, 128)
    op = fg.Kron(fg.Hadamard(8), fg.Circulant(c), precision='fp32')
    x = cplx(rng, op.numCols, 6).astype(np.complex64)
    yh = op.forward(x)
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    yd = op.forward(xt).cpu().numpy()
    assert fo.rel_err(yh, yd) <= 1e-6
    oop = fo.Kron(fo.Hadamard(8), fo.Circulant(c))
    assert fo.rel_err(yh, oop.forward(x.astype(np.complex128))) <= 1e-5
