"""Solver callers on the GPU: ISTA / FISTA against a numpy restatement of
fastmat's iterations on the oracle operator, and the scipy LinearOperator /
largest singular value entry points."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def _deconv_problem(n=512, k=3, seed=0):
    rng = np.random.default_rng(seed)
    t = np.linspace(0, 20 * np.pi, n)
    c = np.cos(2 * t) * np.exp(-t ** 2)
    x = np.zeros(n)
    x[rng.choice(n, k, replace=False)] = 1
    return c, x


def _ista_numpy(Aop, b, lam, steps, sigma, fista=False):
    """fastmat/algorithms/ISTA.py:123-160, FISTA.py:123-180 in numpy."""
    L = 1.0 / sigma ** 2
    b = b.reshape(-1, 1) if b.ndim == 1 else b
    x = np.zeros((Aop.shape[1], b.shape[1]), np.promote_types(np.float32,
                                                              b.dtype))
    y = x.copy()
    t = 1.0
    for _ in range(steps):
        xo = x
        src = y if fista else x
        step = src - L * Aop.backward(Aop.forward(src) - b)
        m = np.maximum(np.abs(step) - L * lam * 0.5, 0)
        x = (m / (m + L * lam * 0.5)) * step
        if fista:
            t_old = t
            t = (1 + np.sqrt(1 + 4 * t ** 2)) / 2
            y = x + ((t_old - 1) / t) * (x - xo)
    return np.where(x != 0, step, x)


@pytest.mark.parametrize('cls', ['ISTA', 'FISTA'])
def test_sparse_deconvolution_matches_numpy_iteration(cls):
    import fastmat_gb300 as fg
    c, x = _deconv_problem()
    C = fg.Circulant(c)
    b = C.forward(x)
    sigma_np = np.linalg.svd(fo.Circulant(c).dense(), compute_uv=False)[0]
    assert abs(C.largestSingularValue - sigma_np) <= 1e-9 * sigma_np
    alg = getattr(fg.algorithms, cls)(C, numLambda=0.005, numMaxSteps=100)
    y = alg.process(b)
    ref = _ista_numpy(fo.Circulant(c), b, 0.005, 100,
                      C.largestSingularValue, fista=cls == 'FISTA')
    assert y.shape == x.shape
    assert fo.rel_err(y, ref.reshape(-1)) <= 1e-9
    assert np.linalg.norm(C.forward(y) - b) < np.linalg.norm(b)


def test_device_resident_columns():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(4)
    n = 256
    d = rng.standard_normal(n) + 2
    A = fg.Product(fg.Partial(fg.Fourier(n), rows=np.arange(0, n, 2)),
                   fg.Diag(d))
    X = np.zeros((n, 3))
    for j in range(3):
        X[rng.choice(n, 4, replace=False), j] = 1
    B = A.forward(X)
    tb = torch.from_numpy(B.T.copy()).cuda().t()
    y = fg.algorithms.FISTA(A, numLambda=0.01, numMaxSteps=50).process(tb)
    assert y.is_cuda and tuple(y.shape) == (n, 3)
    ref = _ista_numpy(fo.Product(fo.Partial(fo.Fourier(n),
                                            rows=np.arange(0, n, 2)),
                                 fo.Diag(d)), B, 0.01, 50,
                      A.largestSingularValue, fista=True)
    assert fo.rel_err(y.cpu().numpy(), ref) <= 1e-9


def test_scipy_linear_operator():
    import fastmat_gb300 as fg
    from scipy.sparse.linalg import svds
    rng = np.random.default_rng(5)
    c = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    C = fg.Circulant(c)
    op = C.scipyLinearOperator
    x = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    assert fo.rel_err(op.matvec(x), fo.Circulant(c).forward(x)) <= 1e-12
    assert fo.rel_err(op.rmatvec(x), fo.Circulant(c).backward(x)) <= 1e-12
    s = svds(op, 1, return_singular_vectors=False)[0]
    assert abs(s - C.largestSingularValue) <= 1e-8 * s
