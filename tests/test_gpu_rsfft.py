"""The register FFT of strided complex vectors (rsfft_kernel,
fm_rsfft.cuh): Fourier modes of a Kron (fastmat/Kron.pyx:284-300) at
element strides that are multiples of 32, complex64 (FP32 form, 1e-5) and
double-float complex (FP64 form, 1e-12) against the oracle, both
directions, lengths the kernel is built for and the vector-program fallback
beyond them or when the input needs a type conversion."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _rsfft(op, dt):
    return 'rsfft' in op.plan(dt).describe(0)


@pytest.mark.parametrize('L', [16, 32, 64, 128, 256, 512])
@pytest.mark.parametrize('m', [32, 96])
@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_kron_fourier_mode(L, m, prec):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(L + m)
    op = fg.Kron(fg.Fourier(L), fg.Eye(m), precision=prec)
    oop = fo.Kron(fo.Fourier(L), fo.Eye(m))
    dt = np.complex128 if prec == 'native' else np.complex64
    lo, hi = (16, 256) if prec == 'native' else (32, 512)
    assert _rsfft(op, dt) == (lo <= L <= hi)
    x = cplx(rng, op.numCols, 3)
    if prec == 'native':
        x[::7] *= 1e-150              # exponents far apart within a vector
    tol = 1e-12 if prec == 'native' else 1e-5
    y = op.forward(x)
    assert y.dtype == dt
    assert fo.rel_err(y, oop.forward(x)) <= tol
    assert fo.rel_err(op.backward(x), oop.backward(x)) <= tol


@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_kron_workload_shape(prec):
    """Fourier, Hadamard and Circulant modes as in the Kron workload: the F
    mode strided by the product of the others (all three register
    kernels)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(11)
    c = cplx(rng, 32)
    op = fg.Kron(fg.Fourier(64), fg.Hadamard(6), fg.Circulant(c),
                 precision=prec)
    oop = fo.Kron(fo.Fourier(64), fo.Hadamard(6), fo.Circulant(c))
    dt = np.complex128 if prec == 'native' else np.complex64
    d = op.plan(dt).describe(0)
    assert 'rsfft' in d and 'rconv' in d and 'rfwht' in d, d
    x = cplx(rng, op.numCols, 4)
    tol = 1e-12 if prec == 'native' else 1e-5
    assert fo.rel_err(op.forward(x), oop.forward(x)) <= tol
    assert fo.rel_err(op.backward(x), oop.backward(x)) <= tol


def test_converting_input_uses_the_vector_program():
    """complex64 input to the FP64 form: the loads convert, so the mode runs
    as its vector program, with the same result."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(12)
    op = fg.Kron(fg.Fourier(128), fg.Eye(64))
    oop = fo.Kron(fo.Fourier(128), fo.Eye(64))
    x = cplx(rng, op.numCols, 2).astype(np.complex64)
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    y = op.forward(xt).cpu().numpy()
    assert y.dtype == np.complex128
    assert fo.rel_err(y, oop.forward(x.astype(np.complex128))) <= 1e-12
