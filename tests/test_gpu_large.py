"""GPU parity at sizes beyond the golden fixtures: long transforms (the
four-step path), Bluestein, the workload shapes, and the reduced-precision
form.  Where a dense oracle is infeasible the checks are np.fft (FFT
accuracy ~1e-16), the oracle's FFT-based restatement, exact-phase DFT rows
and size-independent identities (Hadamard involution, adjoint identity)."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize('n', [2048, 4096, 8192, 16384, 65536, 1 << 18,
                               3 * 4096, 1000, 10000])
def test_fourier_direct_long(n):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n)
    x = cplx(rng, n, 3)
    F = fg.Fourier(n)
    y = F.forward(x)
    assert fo.rel_err(y, np.fft.fft(x, axis=0)) <= 1e-12
    z = F.backward(x)
    assert fo.rel_err(z, np.conj(np.fft.fft(np.conj(x), axis=0))) <= 1e-12


@pytest.mark.parametrize('n', [127, 4099, 9973, 65521])
def test_fourier_bluestein(n):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n)
    x = cplx(rng, n, 2)
    F = fg.Fourier(n)
    y = F.forward(x)
    rows = [0, 1, n // 2, n - 1]
    exact = fo.exact_dft_rows(x, rows)
    assert fo.rel_err(y[rows], exact) <= 1e-12
    assert fo.rel_err(y, np.fft.fft(x, axis=0)) <= 1e-12
    z = F.backward(x)
    assert fo.rel_err(z, np.conj(np.fft.fft(np.conj(x), axis=0))) <= 1e-12


@pytest.mark.parametrize('n', [4097, 5000, 65536, 1 << 18])
def test_circulant_long(n):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(n)
    c = cplx(rng, n)
    x = cplx(rng, n, 2)
    C = fg.Circulant(c)
    ref = np.fft.ifft(np.fft.fft(c)[:, None] * np.fft.fft(x, axis=0), axis=0)
    assert fo.rel_err(C.forward(x), ref) <= 1e-12
    refb = np.fft.ifft(np.conj(np.fft.fft(c))[:, None] *
                       np.fft.fft(x, axis=0), axis=0)
    assert fo.rel_err(C.backward(x), refb) <= 1e-12


@pytest.mark.parametrize('nr,nc', [(4099, 4099), (9000, 3000), (100, 20000)])
def test_toeplitz_long(nr, nc):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(nr + nc)
    vc, vr = cplx(rng, nr), cplx(rng, nc - 1)
    x = cplx(rng, nc, 2)
    g = cplx(rng, nr, 2)
    T = fg.Toeplitz(vc, vr)
    O = fo.Toeplitz(vc, vr)
    assert fo.rel_err(T.forward(x), O.forward(x)) <= 1e-12
    assert fo.rel_err(T.backward(g), O.backward(g)) <= 1e-12


@pytest.mark.parametrize('order', [12, 13, 14, 16, 20])
def test_hadamard_long(order):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(order)
    n = 1 << order
    x = rng.standard_normal((n, 2))
    H = fg.Hadamard(order)
    y = H.forward(x)
    assert fo.rel_err(y, fo.Hadamard(order).forward(x)) <= 1e-12
    # H H = n I
    assert fo.rel_err(H.forward(y) / n, x) <= 1e-12


def test_hadamard_order22_f32_columns():
    """The Hadamard(22) workload shape on two columns (float32)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(22)
    x = rng.standard_normal((1 << 22, 2)).astype(np.float32)
    H = fg.Hadamard(22)
    y = H.forward(x)
    assert y.dtype == np.float32
    ref = fo.Hadamard(22).forward(x.astype(np.float64))
    assert fo.rel_err(y, ref) <= 1e-5


def test_kron_workload_shape_small_and_full_property():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(2)
    # reduced sizes against the oracle
    c = cplx(rng, 16)
    K = fg.Kron(fg.Fourier(32), fg.Hadamard(4), fg.Circulant(c))
    O = fo.Kron(fo.Fourier(32), fo.Hadamard(4), fo.Circulant(c))
    x = cplx(rng, K.numRows, 3)
    assert fo.rel_err(K.forward(x), O.forward(x)) <= 1e-12
    assert fo.rel_err(K.backward(x), O.backward(x)) <= 1e-12
    # dense check at tiny size
    K2 = fg.Kron(fg.Fourier(8), fg.Hadamard(3), fg.Circulant(c[:8]))
    x2 = cplx(rng, K2.numRows, 2)
    assert fo.rel_err(K2.forward(x2), K2.reference() @ x2) <= 1e-12


def test_kron_full_size_one_column():
    """Kron(Fourier(256), Hadamard(8), Circulant(128)), N = 8,388,608: the
    FFT-based oracle on one column and the adjoint identity."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(1)
    c = cplx(rng, 128)
    K = fg.Kron(fg.Fourier(256), fg.Hadamard(8), fg.Circulant(c))
    O = fo.Kron(fo.Fourier(256), fo.Hadamard(8), fo.Circulant(c))
    x = cplx(rng, K.numRows, 1)
    y = K.forward(x)
    assert fo.rel_err(y, O.forward(x)) <= 1e-12
    g = cplx(rng, K.numRows, 1)
    z = K.backward(g)
    lhs = np.vdot(g, y)
    rhs = np.vdot(z, x)
    assert abs(lhs - rhs) / abs(lhs) <= 1e-12


def test_chain_partial_circulant_diag():
    """Partial(rows) . Circulant(c) . Diag(d) at N = 4096 (dense oracle) and
    at N = 2^18 (FFT oracle)."""
    import fastmat_gb300 as fg
    for n, dense in ((4096, True), (1 << 18, False)):
        rng = np.random.default_rng(n)
        c, d = cplx(rng, n), cplx(rng, n)
        rows = np.sort(rng.choice(n, n // 4, replace=False))
        A = fg.Partial(fg.Product(fg.Circulant(c), fg.Diag(d)), rows=rows)
        O = fo.Partial(fo.Product(fo.Circulant(c), fo.Diag(d)), rows=rows)
        x = cplx(rng, n, 4)
        g = cplx(rng, n // 4, 4)
        assert fo.rel_err(A.forward(x), O.forward(x)) <= 1e-12
        assert fo.rel_err(A.backward(g), O.backward(g)) <= 1e-12
        if dense:
            D = A.reference()
            assert fo.rel_err(A.forward(x), D @ x) <= 1e-12


@pytest.mark.parametrize('expr', ['circ', 'four', 'had', 'kron', 'chain'])
def test_fp32_form_error_bound(expr):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(7)
    n = 4096
    c, d = cplx(rng, n), cplx(rng, n)
    if expr == 'circ':
        A, A64 = fg.Circulant(c, precision='fp32'), fg.Circulant(c)
    elif expr == 'four':
        A, A64 = fg.Fourier(n, precision='fp32'), fg.Fourier(n)
    elif expr == 'had':
        A, A64 = fg.Hadamard(12, precision='fp32'), fg.Hadamard(12)
    elif expr == 'kron':
        A = fg.Kron(fg.Fourier(16), fg.Hadamard(4), fg.Circulant(c[:16]),
                    precision='fp32')
        A64 = fg.Kron(fg.Fourier(16), fg.Hadamard(4), fg.Circulant(c[:16]))
    else:
        A = fg.Partial(fg.Product(fg.Circulant(c), fg.Diag(d)),
                       rows=np.arange(0, n, 4), precision='fp32')
        A64 = fg.Partial(fg.Product(fg.Circulant(c), fg.Diag(d)),
                         rows=np.arange(0, n, 4))
    x = cplx(rng, A.numCols, 4)
    y = A.forward(x)
    assert y.dtype in (np.complex64, np.float32)
    assert fo.rel_err(y, A64.forward(x)) <= 1e-5


FOLD_CASES = [
    # (expression in fg/fo namespace, input rows)
    ('Product(Fourier(N), Diag(d))', 'N'),
    ('Product(Diag(d), Fourier(N))', 'N'),
    ('Product(Partial(Eye(N), rows=rows), Fourier(N), Diag(d))', 'N'),
    ('Product(Fourier(N), Hermitian(Partial(Eye(N), rows=rows)))', 'R'),
    ('Product(Fourier(N), Partial(Eye(N), cols=rows))', 'R'),
    ('Partial(Product(Circulant(c), Diag(d)), rows=rows)', 'N'),
    ('Conjugate(Product(Diag(d), Fourier(N), Diag(d)))', 'N'),
    ('Product(Partial(Eye(N), rows=dup), Fourier(N))', 'N'),
    ('Product(Fourier(N), Permutation(perm), Diag(d), 2.0 - 1j)', 'N'),
    ('Product(Hadamard(17), Diag(d[:1 << 17]))', 'H'),
]


@pytest.mark.parametrize('expr,rin', FOLD_CASES)
def test_pointwise_folded_into_long_transforms(expr, rin):
    """Diagonals, selections, conjugation and scalars next to a multi-launch
    transform run inside its first / last launch; results must not
    change."""
    import fastmat_gb300 as fg
    N = 1 << 18
    rng = np.random.default_rng(17)
    c, d = cplx(rng, N), cplx(rng, N)
    rows = np.sort(rng.choice(N, N // 4, replace=False))
    dup = np.concatenate([rows, rows[:100]])
    perm = rng.permutation(N)
    ns = dict(N=N, c=c, d=d, rows=rows, dup=dup, perm=perm)
    gns = dict(ns, **{k: getattr(fg, k) for k in (
        'Fourier', 'Diag', 'Partial', 'Eye', 'Product', 'Hermitian',
        'Circulant', 'Conjugate', 'Permutation', 'Hadamard')})
    ons = dict(ns, Fourier=fo.Fourier, Diag=fo.Diag, Partial=fo.Partial,
               Eye=fo.Eye, Product=fo.Product, Hermitian=fo.Hermitian,
               Circulant=fo.Circulant, Conjugate=fo.Conjugate,
               Permutation=fo.Permutation, Hadamard=fo.Hadamard)
    op, oop = eval(expr, gns), eval(expr, ons)
    n_in = {'N': N, 'R': len(rows), 'H': 1 << 17}[rin]
    x = cplx(rng, n_in, 3)
    g = cplx(rng, op.numRows, 3)
    assert fo.rel_err(op.forward(x), oop.forward(x)) <= 1e-12
    assert fo.rel_err(op.backward(g), oop.backward(g)) <= 1e-12


@pytest.mark.parametrize('order,cols', [(4, 3), (8, 5), (12, 2), (13, 3),
                                        (17, 2), (22, 2)])
def test_hadamard_tensor_core_form(order, cols):
    """precision='bf16': 16-point groups as BF16 MMA (three-term split,
    FP32 accumulation) on the tensor cores where the register FWHT kernels
    do not cover a pass (short or strided-by-less-than-32 vectors; those
    kernels take the others on the FP32 pipes); error against FP64 stated
    and bounded by 1e-5."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(order)
    x = rng.standard_normal((1 << order, cols)).astype(np.float32)
    H = fg.Hadamard(order, precision='bf16')
    y = H.forward(x)
    assert y.dtype == np.float32
    ref = fo.Hadamard(order).forward(x.astype(np.float64))
    err = fo.rel_err(y, ref)
    assert err <= 1e-5, err
    desc = H.plan(np.float32).describe()
    assert ('cls=4' in desc) == (order < 10 or order in (17,)), desc
    z = H.backward(x)
    assert fo.rel_err(z, ref) <= 1e-5


def test_kron_with_tensor_core_hadamard_mode():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(3)
    d = rng.standard_normal(16)
    op = fg.Kron(fg.Hadamard(4), fg.Diag(d), fg.Hadamard(8),
                 precision='bf16')
    oop = fo.Kron(fo.Hadamard(4), fo.Diag(d), fo.Hadamard(8))
    x = rng.standard_normal((op.numCols, 3)).astype(np.float32)
    y = op.forward(x)
    assert y.dtype == np.float32
    assert fo.rel_err(y, oop.forward(x.astype(np.float64))) <= 1e-5


@pytest.mark.parametrize('dims', [(64, 128), (16, 9, 32), (127, 8)])
def test_multilevel_circulant_large(dims):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(sum(dims))
    c = cplx(rng, *dims)
    C = fg.Circulant(c)
    oc = fo.Circulant(c)
    x = cplx(rng, C.numCols, 3)
    assert fo.rel_err(C.forward(x), oc.forward(x)) <= 1e-12
    assert fo.rel_err(C.backward(x), oc.backward(x)) <= 1e-12


def test_multilevel_toeplitz_large():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(21)
    t = cplx(rng, 63, 31)
    T = fg.Toeplitz(t, split=np.array([40, 20]))
    ot = fo.Toeplitz(t, split=np.array([40, 20]))
    assert T.shape == ot.shape == (800, 24 * 12)
    x = cplx(rng, T.numCols, 2)
    g = cplx(rng, T.numRows, 2)
    assert fo.rel_err(T.forward(x), ot.forward(x)) <= 1e-12
    assert fo.rel_err(T.backward(g), ot.backward(g)) <= 1e-12


@pytest.mark.parametrize('pinned', [True, False])
def test_host_entry_point_chunked_pipeline(pinned):
    """fm_execute_host splits large calls into column chunks copied in,
    transformed and copied out on three streams: the result equals the
    device-resident call and the FFT, for page-locked and pageable host
    buffers, in both directions."""
    import torch
    import fastmat_gb300 as fg
    from fastmat_gb300 import _native
    rng = np.random.default_rng(31)
    n, m = 1 << 20, 37  # 592 MiB in and out: several chunks, ragged last
    F = fg.Fourier(n)
    plan = F.plan(np.complex128)
    x = cplx(rng, n, m)
    if pinned:
        xh = torch.empty((m, n), dtype=torch.complex128).pin_memory()
        yh = torch.empty((m, n), dtype=torch.complex128).pin_memory()
        xa, ya = xh.numpy().T, yh.numpy().T
        xa[:] = x
    else:
        xa = np.asfortranarray(x)
        ya = np.empty((n, m), dtype=np.complex128, order='F')
    plan.execute_host(_native.FORWARD, xa, ya)
    ref = F.forward(torch.from_numpy(x.T.copy()).cuda().t()).cpu().numpy()
    assert np.array_equal(ya, ref)
    assert fo.rel_err(ya[:, :3], np.fft.fft(x[:, :3], axis=0)) <= 1e-12
    plan.execute_host(_native.BACKWARD, xa, ya)
    assert fo.rel_err(ya[:, -2:], np.conj(np.fft.fft(np.conj(x[:, -2:]),
                                                     axis=0))) <= 1e-12
