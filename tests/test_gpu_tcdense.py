"""Dense factors on the tensor cores (precision='bf16' on float32 data):
square dense operators of order <= 64 -- a Kron factor applied mode-wise
(fastmat/Kron.pyx:284-300) or a Matrix on its own -- run as
tcgen05.mma tiles (BF16 three-term splits of both the data and the factor,
FP32 accumulation in tensor memory), kernel class 6.  Held to the FP64
oracle at 1e-5, like every float32 form, in both directions, for orders
that need padding to the MMA's multiples of 16, strided and contiguous
modes; orders above 64 keep the SIMT dense product."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def _check(op, oop, rng, cols=5, tc=True):
    x = rng.standard_normal((op.numCols, cols)).astype(np.float32)
    g = rng.standard_normal((op.numRows, cols)).astype(np.float32)
    desc = op.plan(np.float32).describe(0) + op.plan(np.float32).describe(1)
    assert ('cls=6' in desc) == tc, desc
    y = op.forward(x)
    assert y.dtype == np.float32
    assert fo.rel_err(y, oop.forward(x.astype(np.float64))) <= 1e-5
    z = op.backward(g)
    assert fo.rel_err(z, oop.backward(g.astype(np.float64))) <= 1e-5


@pytest.mark.parametrize('n', [7, 16, 24, 33, 64])
def test_dense_kron_factor_contiguous_mode(n):
    """Kron(Hadamard(5), Matrix(n x n)): the dense factor on contiguous
    vectors of n points (vector-major tiles)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    op = fg.Kron(fg.Hadamard(5), fg.Matrix(a), precision='bf16')
    oop = fo.Kron(fo.Hadamard(5), fo.Dense(a))
    _check(op, oop, rng)


@pytest.mark.parametrize('n,m', [(16, 128), (32, 256), (64, 512), (40, 64)])
def test_dense_kron_factor_strided_mode(n, m):
    """Kron(Matrix(n x n), Eye(m)): vectors of n points at stride m
    (element-major tiles of up to 128 vectors)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n + m)
    a = rng.standard_normal((n, n))
    op = fg.Kron(fg.Matrix(a), fg.Eye(m), precision='bf16')
    oop = fo.Kron(fo.Dense(a), fo.Eye(m))
    _check(op, oop, rng, cols=3)


def test_dense_matrix_on_its_own_and_large_order_fallback():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(9)
    a = rng.standard_normal((48, 48))
    _check(fg.Matrix(a, precision='bf16'), fo.Dense(a), rng, cols=300)
    b = rng.standard_normal((80, 80))   # above 64: SIMT dense product
    _check(fg.Matrix(b, precision='bf16'), fo.Dense(b), rng, tc=False)


def test_dense_factor_with_hadamard_modes_in_one_kron():
    """A Kron mixing tensor-core Hadamard modes (class 4) and a
    tensor-core dense mode (class 6)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(11)
    a = rng.standard_normal((32, 32))
    op = fg.Kron(fg.Hadamard(6), fg.Matrix(a), fg.Hadamard(4),
                 precision='bf16')
    oop = fo.Kron(fo.Hadamard(6), fo.Dense(a), fo.Hadamard(4))
    x = rng.standard_normal((op.numCols, 4)).astype(np.float32)
    desc = op.plan(np.float32).describe(0)
    assert 'cls=6' in desc and 'cls=4' in desc
    assert fo.rel_err(op.forward(x), oop.forward(x.astype(np.float64))) <= 1e-5
