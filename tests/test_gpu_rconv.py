"""The register-resident convolution kernel (fm_rconv.cuh): circular
convolutions of contiguous power-of-two vectors that fit one warp run there
instead of the shared-memory stage kernel.  Checked against the oracle
(fastmat's algorithm restated) at every built length, in the double-float
form (1e-12) and the FP32 form (1e-5), with zero padding (Toeplitz),
conjugation and chirp products (Bluestein Fourier), type conversions,
leading dimensions and Kron modes with many vectors per column."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _uses_rconv(op, dt):
    return 'rconv' in op.plan(dt).describe()


@pytest.mark.parametrize('n', [8, 16, 32, 64, 128, 256, 512])
@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_circulant_every_length(n, prec):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n)
    c = cplx(rng, n)
    C, O = fg.Circulant(c, precision=prec), fo.Circulant(c)
    x = cplx(rng, n, 37)   # 37 columns: not a multiple of the vectors/warp
    dt = np.complex128 if prec == 'native' else np.complex64
    if prec == 'native':
        assert _uses_rconv(C, dt) == (n <= 256)
        tol = 1e-12
    else:
        assert _uses_rconv(C, dt) == (n >= 16)
        tol = 1e-5
    y, z = C.forward(x), C.backward(x)
    assert y.dtype == dt
    assert fo.rel_err(y, O.forward(x)) <= tol
    assert fo.rel_err(z, O.backward(x)) <= tol


@pytest.mark.parametrize('nr,nc', [(20, 30), (64, 1), (100, 29), (33, 97)])
def test_toeplitz_zero_padded_embedding(nr, nc):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(nr * nc)
    vc, vr = cplx(rng, nr), cplx(rng, nc - 1)
    T, O = fg.Toeplitz(vc, vr), fo.Toeplitz(vc, vr)
    assert _uses_rconv(T, np.complex128)
    x, g = cplx(rng, nc, 5), cplx(rng, nr, 5)
    assert fo.rel_err(T.forward(x), O.forward(x)) <= 1e-12
    assert fo.rel_err(T.backward(g), O.backward(g)) <= 1e-12


@pytest.mark.parametrize('n', [11, 13, 97, 127])
def test_bluestein_fourier(n):
    """Prime sizes: chirp, convolution of length 2^k >= 2n - 1, chirp; the
    adjoint conjugates around it."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n)
    F = fg.Fourier(n)
    assert _uses_rconv(F, np.complex128)
    x = cplx(rng, n, 6)
    assert fo.rel_err(F.forward(x), np.fft.fft(x, axis=0)) <= 1e-12
    assert fo.rel_err(F.backward(x),
                      np.conj(np.fft.fft(np.conj(x), axis=0))) <= 1e-12
    F32 = fg.Fourier(n, precision='fp32')
    assert fo.rel_err(F32.forward(x), np.fft.fft(x, axis=0)) <= 1e-5


def test_input_conversions_and_device_strides():
    """Inputs of other types (converting loads) and column-major device
    tensors with a leading dimension larger than the vector."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(3)
    n = 128
    c = cplx(rng, n)
    C, O = fg.Circulant(c), fo.Circulant(c)
    for x in (rng.standard_normal((n, 4)),
              rng.standard_normal((n, 4)).astype(np.float32),
              cplx(rng, n, 4).astype(np.complex64),
              rng.integers(-5, 5, (n, 4)).astype(np.int16)):
        assert fo.rel_err(C.forward(x), O.forward(x)) <= 1e-12
    big = torch.from_numpy(cplx(rng, 6, n + 40)).cuda()
    xt = big[:, 7:7 + n].t()          # leading dimension n + 40
    y = C.forward(xt).cpu().numpy()
    assert fo.rel_err(y, O.forward(xt.cpu().numpy())) <= 1e-12
    y1 = C.forward(xt[:, 2]).cpu().numpy()
    assert fo.rel_err(y1, O.forward(xt[:, 2].cpu().numpy())) <= 1e-12


@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_kron_mode_with_many_vectors_per_column(prec):
    """The contiguous mode of a Kron: A vectors per column, one launch."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(4)
    c = cplx(rng, 128)
    K = fg.Kron(fg.Fourier(12), fg.Hadamard(3), fg.Circulant(c),
                precision=prec)
    O = fo.Kron(fo.Fourier(12), fo.Hadamard(3), fo.Circulant(c))
    dt = np.complex128 if prec == 'native' else np.complex64
    assert _uses_rconv(K, dt)
    x = cplx(rng, K.numRows, 3)
    tol = 1e-12 if prec == 'native' else 1e-5
    assert fo.rel_err(K.forward(x), O.forward(x)) <= tol
    assert fo.rel_err(K.backward(x), O.backward(x)) <= tol


def test_products_folded_around_the_convolution():
    """Diag before and after a circulant (program-level products), a scalar,
    and the backward direction (conjugate diagonal: stage kernel)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(5)
    n = 64
    c, d1, d2 = cplx(rng, n), cplx(rng, n), cplx(rng, n)
    A = fg.Product(fg.Diag(d2), fg.Circulant(c), fg.Diag(d1), 2.0 - 0.5j)
    O = fo.Product(fo.Diag(d2), fo.Circulant(c), fo.Diag(d1), 2.0 - 0.5j)
    x = cplx(rng, n, 9)
    assert fo.rel_err(A.forward(x), O.forward(x)) <= 1e-12
    assert fo.rel_err(A.backward(x), O.backward(x)) <= 1e-12
