"""Bit-exact results where fastmat's own result is exact or fully ordered.

Index work (Permutation, Partial, Eye and their compositions) only moves
elements, so its outputs must equal fastmat's gathers bit for bit, whatever
the element type and however wide the range of magnitudes in a column
(fastmat/Permutation.pyx:120-124, fastmat/Partial.pyx:268-294).  Single-
precision Hadamard transforms run their a + b / a - b butterflies in
fastmat's order (distance 1, 2, 4, ..., fastmat/Hadamard.pyx:182-228), so
their float32 results equal fastmat's float32 results exactly, at the
workload's full order 22 as well."""

import numpy as np
import pytest

from oracle import fm_oracle as fo
from tests.golden_cases import load_cases

pytestmark = pytest.mark.gpu

DTYPES = [np.float32, np.float64, np.complex64, np.complex128, np.int8,
          np.int16, np.int32, np.int64]


def _data(rng, n, m, dt):
    dt = np.dtype(dt)
    if dt.kind == 'i':
        info = np.iinfo(dt)
        return rng.integers(info.min, info.max, size=(n, m), dtype=dt,
                            endpoint=True)
    x = rng.standard_normal((n, m))
    if dt.kind == 'c':
        x = x + 1j * rng.standard_normal((n, m))
    # magnitudes from 1e-300 (float64) / 1e-38 (float32) to 1e300 / 1e38
    # in every column: far more than the 2^126 span of one float32 exponent
    big = 300 if dt in (np.float64, np.complex128) else 37
    x *= 10.0 ** rng.integers(-big, big, size=(n, m))
    for i, v in enumerate((1.0, 10.0 ** -big, -(10.0 ** big))[:n]):
        x[i] = v
    return x.astype(dt)


def _same(a, b):
    assert a.dtype == b.dtype and a.shape == b.shape
    assert np.array_equal(a, b), np.argwhere(a != b)[:5]


@pytest.mark.parametrize('dt', DTYPES, ids=lambda d: np.dtype(d).name)
def test_permutation_is_a_gather(dt):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(1)
    for n in (1, 7, 1000, 4099, 70000):
        sigma = rng.permutation(n)
        P = fg.Permutation(sigma)
        x = _data(rng, n, 3, dt)
        _same(P.forward(x), x[sigma, :])
        _same(P.backward(x), x[np.argsort(sigma), :])


@pytest.mark.parametrize('dt', DTYPES, ids=lambda d: np.dtype(d).name)
def test_partial_selections_are_exact(dt):
    """Zero fill, scatter and gather of fastmat's Partial over Eye and
    Permutation: row and column index selections, boolean masks,
    duplicated rows, one-sided selections, and a long column."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(2)
    for n in (9, 1000, 1 << 17):
        rows = np.sort(rng.choice(n, max(1, n // 3), replace=False))
        cols = rng.choice(n, max(1, n // 2), replace=False)
        dup = np.concatenate([rows, rows[:5]])
        mask = rng.random(n) < 0.4
        sigma = rng.permutation(n)
        ops = [
            ('rows', lambda M: fg.Partial(M, rows=rows),
             lambda M: fo.Partial(M, rows=rows)),
            ('cols', lambda M: fg.Partial(M, cols=cols),
             lambda M: fo.Partial(M, cols=cols)),
            ('both', lambda M: fg.Partial(M, rows=dup, cols=cols),
             lambda M: fo.Partial(M, rows=dup, cols=cols)),
            ('mask', lambda M: fg.Partial(M, rows=mask, cols=~mask),
             lambda M: fo.Partial(M, rows=mask, cols=~mask)),
        ]
        for name, mk, mko in ops:
            for inner, oinner in ((fg.Eye(n), fo.Eye(n)),
                                  (fg.Permutation(sigma),
                                   fo.Permutation(sigma))):
                A, O = mk(inner), mko(oinner)
                x = _data(rng, A.numCols, 2, dt)
                g = _data(rng, A.numRows, 2, dt)
                if A.numCols == 0 or A.numRows == 0:
                    continue
                _same(A.forward(x), O.forward(x))
                _same(A.backward(g), O.backward(g))


@pytest.mark.parametrize('dt', [np.float64, np.complex128, np.complex64],
                         ids=lambda d: np.dtype(d).name)
def test_compositions_of_index_operators_are_exact(dt):
    """Hermitian / Transpose / Conjugate, Product with +-1 and +-i, Sum,
    Kron and Blocks of index operators only move (and, for Sum, add) data:
    they compute in the I/O type, in fastmat's order."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(3)
    n = 777
    s1, s2 = rng.permutation(n), rng.permutation(n)
    rows = np.sort(rng.choice(n, 300, replace=False))
    ns_g = dict(vars(fg))
    ns_o = dict(Permutation=fo.Permutation, Partial=fo.Partial, Eye=fo.Eye,
                Hermitian=fo.Hermitian, Transpose=fo.Transpose,
                Conjugate=fo.Conjugate, Product=fo.Product, Sum=fo.Sum,
                Kron=fo.Kron, Blocks=fo.Blocks)
    exprs = [
        'Hermitian(Permutation(s1))',
        'Transpose(Partial(Permutation(s2), rows=rows))',
        'Conjugate(Permutation(s1))',
        'Product(Permutation(s1), Permutation(s2))',
        'Product(Permutation(s1), -1)',
        'Product(Permutation(s1), 1j)',
        'Product(Partial(Eye(n), rows=rows), Permutation(s2), -1j)',
        'Sum(Permutation(s1), Permutation(s2), Eye(n))',
        'Kron(Permutation(np.array([2, 0, 1])), Permutation(s2))',
        'Blocks([[Permutation(s1), Eye(n)], [Eye(n), Permutation(s2)]])',
    ]
    for e in exprs:
        env_g = dict(ns_g, s1=s1, s2=s2, rows=rows, n=n, np=np)
        env_o = dict(ns_o, s1=s1, s2=s2, rows=rows, n=n, np=np)
        A, O = eval(e, env_g), eval(e, env_o)
        x = _data(rng, A.numCols, 2, dt)
        # keep sums finite: Sum adds elements of one column
        if 'Sum' in e:
            x = (rng.standard_normal((A.numCols, 2)) * 1e3).astype(dt)
        g = x[:A.numRows] if A.numRows <= A.numCols else _data(
            rng, A.numRows, 2, dt)
        y, yo = A.forward(x), O.forward(x)
        assert y.dtype == yo.dtype, e
        assert np.array_equal(y, yo), e
        assert np.array_equal(A.backward(g), O.backward(g)), e


def test_index_plans_compute_in_the_io_type():
    """The plans of index-only trees report the I/O type as their compute
    type; a tree with arithmetic keeps double-float."""
    import fastmat_gb300 as fg
    from fastmat_gb300 import _native
    rng = np.random.default_rng(4)
    P = fg.Partial(fg.Permutation(rng.permutation(64)), rows=np.arange(9))
    assert P.plan(np.complex128).info().compute_type == _native.FM_C128
    assert P.plan(np.float64).info().compute_type == _native.FM_F64
    D = fg.Product(fg.Permutation(rng.permutation(64)),
                   fg.Diag(rng.standard_normal(64)))
    assert D.plan(np.float64).info().compute_type == _native.FM_F64_DF


def test_golden_index_cases_bit_exact():
    """The reference's own outputs of its Permutation cases (float64 and
    complex128) and of Partial(Hadamard(4)) on float32 (computed by fastmat
    in float32): equal bit for bit."""
    import fastmat_gb300 as fg
    cases = {c.name: c for c in load_cases()}
    ns = dict(Permutation=fg.Permutation, Partial=fg.Partial,
              Hadamard=fg.Hadamard, np=np)
    for name in ('perm', 'perm_c', 'partial_bool'):
        c = cases[name]
        op = c.build(ns)
        _same(op.forward(c.x), c.fwd)
        _same(op.backward(c.g), c.bwd)


@pytest.mark.parametrize('order', [1, 4, 9, 13, 14, 17])
def test_hadamard_float32_bit_exact(order):
    """Single- and two-pass float32 FWHT equal the oracle's float32
    restatement of fastmat's butterfly order exactly (and so fastmat's own
    float32 results)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(order)
    x = rng.standard_normal((1 << order, 3)).astype(np.float32)
    H = fg.Hadamard(order)
    y = H.forward(x)
    _same(y, fo.Hadamard(order).forward(x))
    _same(H.backward(x), y)


def test_hadamard_order22_float32_bit_exact_columns():
    """The Hadamard(22) workload: float32 results on 4 of its 64 columns
    (the GPU transforms all 64) equal the oracle's float32 FWHT exactly."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(22)
    n = 1 << 22
    x = rng.standard_normal((n, 64), dtype=np.float32)
    y = fg.Hadamard(22).forward(x)
    pick = [0, 21, 42, 63]
    _same(y[:, pick], fo.Hadamard(22).forward(np.asfortranarray(x[:, pick])))


@pytest.mark.parametrize('order', [10, 12, 13])
def test_hadamard_float32_unaligned_columns_bit_exact(order):
    """Columns with a leading dimension that breaks 16-byte alignment run
    the FWHT through the stage kernel instead of the register kernel: the
    same butterflies in the same order, so the same bits."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(order + 100)
    n = 1 << order
    big = torch.from_numpy(rng.standard_normal((3, n + 1)).astype(
        np.float32)).cuda()
    xt = big[:, :n].t()                  # leading dimension n + 1
    H = fg.Hadamard(order)
    y = H.forward(xt).cpu().numpy()
    x = xt.cpu().numpy()
    _same(y, fo.Hadamard(order).forward(np.asfortranarray(x)))
    # and the aligned call agrees bit for bit
    ya = H.forward(torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t())
    _same(ya.cpu().numpy(), y)
