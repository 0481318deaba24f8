"""The register FWHT of strided vectors (rsfwht_kernel, fm_rfwht.cuh): the
high index bits of a long Hadamard (fastmat/Hadamard.pyx:164-230, second
pass at stride 2^13) and Hadamard modes of a Kron (fastmat/Kron.pyx:284-300)
at element strides that are multiples of 32, real and complex.  float32
results are compared bit for bit with the oracle's float32 restatement of
fastmat's butterfly order; the double-float form is held to 1e-12 and the
complex FP32 forms to 1e-5 against the FP64 oracle."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.dtype == b.dtype and a.shape == b.shape
    assert np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                          np.ascontiguousarray(b).view(np.uint8))


def _strided_fwht(op, dt):
    d = op.plan(dt).describe(0)
    return [ln for ln in d.splitlines() if 'rfwht' in ln and
            'stride=1 ' not in ln]


@pytest.mark.parametrize('order', [19, 20, 21])
def test_long_hadamard_float32_bit_exact(order):
    """Second pass of 64, 128 and 256 points at stride 8192."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(order)
    x = rng.standard_normal((1 << order, 2)).astype(np.float32)
    H = fg.Hadamard(order)
    assert _strided_fwht(H, np.float32)
    # both passes in one launch, column by column
    assert 'fused-with-next' in H.plan(np.float32).describe(0)
    y = H.forward(x)
    _same(y, fo.Hadamard(order).forward(x))
    _same(H.backward(x), y)


def test_fused_passes_many_columns_and_leading_dimension():
    """The fused two-pass launch over 70 columns with a padded leading
    dimension (the column counters and the column-by-column order), float32
    bit-exact."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(70)
    n = 1 << 19
    big = torch.from_numpy(rng.standard_normal((70, n + 4)).astype(
        np.float32)).cuda()
    xt = big[:, :n].t()                  # leading dimension n + 4
    H = fg.Hadamard(19)
    y = H.forward(xt).cpu().numpy()
    pick = [0, 1, 34, 69]
    x = xt.cpu().numpy()
    _same(y[:, pick], fo.Hadamard(19).forward(np.asfortranarray(x[:, pick])))


@pytest.mark.parametrize('order,strided', [(18, True), (20, True),
                                           (22, True)])
def test_long_hadamard_double_float(order, strided):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(order + 7)
    x = rng.standard_normal((1 << order, 2))
    x[::5] *= 1e-200            # exponents far apart within a vector
    H = fg.Hadamard(order)
    if strided:
        assert _strided_fwht(H, np.float64)
        assert 'fused-with-next' in H.plan(np.float64).describe(0)
    y = H.forward(x)
    assert y.dtype == np.float64
    assert fo.rel_err(y, fo.Hadamard(order).forward(x)) <= 1e-12


@pytest.mark.parametrize('k,m', [(6, 32), (7, 64), (8, 128), (9, 32),
                                 (10, 64), (11, 32), (12, 32), (5, 96)])
@pytest.mark.parametrize('dtype', [np.float32, np.float64])
def test_kron_hadamard_mode_real(k, m, dtype):
    """Kron(Hadamard(k), Eye(m)): 2^k points at stride m."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(k * 100 + m)
    op = fg.Kron(fg.Hadamard(k), fg.Eye(m))
    oop = fo.Kron(fo.Hadamard(k), fo.Eye(m))
    n = (1 << k) * m
    x = rng.standard_normal((n, 3)).astype(dtype)
    lo, hi = (64, 2048) if dtype == np.float32 else (32, 1024)
    assert bool(_strided_fwht(op, dtype)) == (lo <= (1 << k) <= hi)
    y = op.forward(x)
    assert y.dtype == dtype
    if dtype == np.float32:
        # the same butterflies in fastmat's order as the float32 FWHT
        ref = fo.Kron(fo.Hadamard(k), fo.Eye(m)).forward(
            x.astype(np.float64))
        assert fo.rel_err(y, ref) <= 1e-5
    else:
        assert fo.rel_err(y, oop.forward(x)) <= 1e-12
    assert fo.rel_err(op.backward(x), oop.backward(x.astype(np.float64))) \
        <= (1e-5 if dtype == np.float32 else 1e-12)


@pytest.mark.parametrize('prec', ['native', 'fp32'])
def test_kron_hadamard_mode_complex(prec):
    """A complex Hadamard mode between an FFT mode and a circulant mode
    (the shape of the Kron workload): real and imaginary parts as real
    vectors at twice the stride."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(5)
    c = rng.standard_normal(32) + 1j * rng.standard_normal(32)
    op = fg.Kron(fg.Fourier(16), fg.Hadamard(6), fg.Circulant(c),
                 precision=prec)
    oop = fo.Kron(fo.Fourier(16), fo.Hadamard(6), fo.Circulant(c))
    dt = np.complex128 if prec == 'native' else np.complex64
    assert _strided_fwht(op, dt)
    x = rng.standard_normal((op.numCols, 5)) + \
        1j * rng.standard_normal((op.numCols, 5))
    tol = 1e-12 if prec == 'native' else 1e-5
    assert fo.rel_err(op.forward(x), oop.forward(x)) <= tol
    assert fo.rel_err(op.backward(x), oop.backward(x)) <= tol


def test_bf16_form_hadamard_uses_register_fwht():
    """The tensor-core form of a Hadamard runs in the register FWHT kernels
    (float32 pipes: the transform is bound by HBM traffic), with float32
    results bit-identical to the FP32 form."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(3)
    x = rng.standard_normal((1 << 20, 2)).astype(np.float32)
    Hb = fg.Hadamard(20, precision='bf16')
    d = Hb.plan(np.float32).describe(0)
    assert d.count('rfwht') == 2, d
    _same(Hb.forward(x), fg.Hadamard(20).forward(x))
