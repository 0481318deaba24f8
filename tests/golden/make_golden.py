"""Generate the golden fixtures in this folder from the reference fastmat.

Run in a container where the reference is built (``oracle/build_reference.sh``
builds it into ``baseline/_ref/src``):

    python tests/golden/make_golden.py               # everything
    python tests/golden/make_golden.py --accessors   # accessors.npz only

Each case is an operator expression over named parameter arrays, written in
the class vocabulary that fastmat, the oracle and ``fastmat_gb300`` share
(``Fourier``, ``Circulant``, ``Toeplitz``, ``Hadamard``, ``Kron``, ``Diag``,
``Partial``, ``Permutation``, ``Product``, ``Sum``, ``Hermitian``,
``Conjugate``, ``Transpose``, ``Eye``, ``Matrix``).  For every case the file
stores the seeded input, the reference's forward and backward outputs and,
for small operators, the reference's dense ``.reference()`` matrix.
"""

import json
import os
import sys

import numpy as np
import scipy.sparse

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, 'baseline', '_ref', 'src'))

import fastmat as fm  # noqa: E402  (the reference, built locally)


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def namespace():
    return dict(
        Fourier=fm.Fourier, Circulant=fm.Circulant, Toeplitz=fm.Toeplitz,
        Hadamard=fm.Hadamard, Kron=fm.Kron, Diag=fm.Diag, Partial=fm.Partial,
        Permutation=fm.Permutation, Product=fm.Product, Sum=fm.Sum,
        Hermitian=fm.Hermitian, Conjugate=fm.Conjugate,
        Transpose=fm.Transpose, Eye=fm.Eye, Matrix=fm.Matrix,
        Blocks=fm.Blocks, BlockDiag=fm.BlockDiag, Sparse=fm.Sparse,
        csr=scipy.sparse.csr_matrix, np=np)


def cases():
    """(name, expression, params, input-dtype, columns, dense?)"""
    rng = np.random.default_rng(1234)
    out = []

    def add(name, expr, params, xdtype=np.complex128, m=3, dense=True):
        out.append((name, expr, params, np.dtype(xdtype), m, dense))

    # Fourier: direct and Bluestein, including fastmat's own test sizes
    # (fastmat/Fourier.pyx:249-270: 35 and 127, optimize on/off)
    for n in (1, 2, 3, 5, 7, 8, 16, 35, 64, 97, 127, 128, 210, 243, 1000,
              1024):
        add('fourier_%d' % n, 'Fourier(%d)' % n, {})
    add('fourier_127_noopt', 'Fourier(127, optimize=False)', {})
    add('fourier_35_noopt', 'Fourier(35, optimize=False)', {})
    add('fourier_4099', 'Fourier(4099)', {}, m=2, dense=False)
    add('fourier_f32in', 'Fourier(35)', {}, xdtype=np.float32)
    add('fourier_i16in', 'Fourier(16)', {}, xdtype=np.int16)

    # Circulant: fastmat's 1-level test sizes (fastmat/Circulant.pyx:428-467)
    for n in (1, 2, 7, 41, 64, 97, 100, 257, 1024):
        add('circulant_%d' % n, 'Circulant(c)', {'c': cplx(rng, n)})
    add('circulant_real', 'Circulant(c)', {'c': rng.standard_normal(41)},
        xdtype=np.float64)
    add('circulant_noopt', 'Circulant(c, optimize=False)',
        {'c': cplx(rng, 41)})

    # Toeplitz (vecC, vecR): square and rectangular
    for nr, nc in ((1, 1), (3, 3), (5, 8), (8, 5), (40, 25), (97, 97),
                   (64, 64)):
        add('toeplitz_%dx%d' % (nr, nc), 'Toeplitz(tc, tr)',
            {'tc': cplx(rng, nr), 'tr': cplx(rng, nc - 1)})
    add('toeplitz_real', 'Toeplitz(tc, tr)',
        {'tc': rng.standard_normal(9), 'tr': rng.standard_normal(6)},
        xdtype=np.float32)

    # Hadamard over several dtypes (fastmat/Hadamard.pyx:251-267)
    for order in (1, 2, 4, 6, 10):
        add('hadamard_%d' % order, 'Hadamard(%d)' % order, {},
            xdtype=np.float64, dense=order <= 10)
    add('hadamard_f32', 'Hadamard(7)', {}, xdtype=np.float32)
    add('hadamard_c128', 'Hadamard(5)', {}, xdtype=np.complex128)
    add('hadamard_c64', 'Hadamard(5)', {}, xdtype=np.complex64)
    add('hadamard_i16', 'Hadamard(6)', {}, xdtype=np.int16)
    add('hadamard_i32', 'Hadamard(6)', {}, xdtype=np.int32)
    add('hadamard_i8', 'Hadamard(3)', {}, xdtype=np.int8)

    # Diag, Permutation, Partial (fastmat/Partial.pyx:306-362 uses Hadamard)
    add('diag_c', 'Diag(d)', {'d': cplx(rng, 33)})
    add('diag_r', 'Diag(d)', {'d': rng.standard_normal(33)},
        xdtype=np.float32)
    add('diag_i', 'Diag(d)', {'d': rng.integers(-3, 4, 17).astype(np.int16)},
        xdtype=np.int16)
    add('perm', 'Permutation(s)', {'s': rng.permutation(29)},
        xdtype=np.float64)
    add('perm_c', 'Permutation(s)', {'s': rng.permutation(64)})
    add('partial_idx', 'Partial(Hadamard(4), rows=r, cols=k)',
        {'r': np.array([1, 3, 4, 9, 15]), 'k': np.array([0, 2, 5, 6, 7, 11])},
        xdtype=np.float64)
    add('partial_bool', 'Partial(Hadamard(4), rows=rb, cols=kb)',
        {'rb': rng.random(16) > 0.5, 'kb': rng.random(16) > 0.3},
        xdtype=np.float32)
    # a one-sided Partial's dense reference indexes with np.s_, which numpy 2
    # rejects (fastmat/Partial.pyx:297-303), so only forward/backward are kept
    add('partial_rows_only', 'Partial(Fourier(12), rows=r)',
        {'r': np.array([11, 0, 5, 6])}, dense=False)
    add('partial_cols_only', 'Partial(Circulant(c), cols=k)',
        {'c': cplx(rng, 20), 'k': np.array([3, 1, 19, 7, 8])}, dense=False)

    # compositions
    add('product_scalar', 'Product(Hadamard(3), 2.5j, Diag(d))',
        {'d': cplx(rng, 8)})
    add('product_chain', 'Product(Fourier(16).H, Diag(d), Fourier(16))',
        {'d': cplx(rng, 16)})
    add('product_real_scalar', 'Product(Hadamard(4), -1.5)', {},
        xdtype=np.float32)
    add('sum_ops', 'Sum(Circulant(c), Fourier(24), Diag(d))',
        {'c': cplx(rng, 24), 'd': cplx(rng, 24)})
    add('sum_real', 'Sum(Hadamard(3), Diag(d), Eye(8))',
        {'d': rng.standard_normal(8)}, xdtype=np.float64)
    add('hermitian', 'Hermitian(Circulant(c))', {'c': cplx(rng, 30)})
    add('transpose', 'Transpose(Toeplitz(tc, tr))',
        {'tc': cplx(rng, 10), 'tr': cplx(rng, 6)})
    add('conjugate', 'Conjugate(Fourier(20))', {})
    add('kron_fhc', 'Kron(Fourier(4), Hadamard(2), Circulant(c))',
        {'c': cplx(rng, 5)})
    add('kron_cfg2_small', 'Kron(Fourier(8), Hadamard(3), Circulant(c))',
        {'c': cplx(rng, 8)})
    add('kron_dense', 'Kron(Matrix(a), Matrix(b), Matrix(e))',
        {'a': cplx(rng, 5, 5), 'b': rng.standard_normal((4, 4)),
         'e': cplx(rng, 3, 3)})
    add('kron_diag', 'Kron(Diag(d1), Diag(d2))',
        {'d1': np.array([1., 2.]), 'd2': np.array([1., 10., 100.])},
        xdtype=np.float64)
    add('chain_cfg4_small',
        'Partial(Product(Circulant(c), Diag(d)), rows=r)',
        {'c': cplx(rng, 64), 'd': cplx(rng, 64),
         'r': np.sort(rng.choice(64, 16, replace=False))}, dense=False)
    add('dense_matrix', 'Matrix(a)', {'a': cplx(rng, 6, 9)})
    # multi-level Circulant and Toeplitz (fastmat/Circulant.pyx:138-215,
    # fastmat/Toeplitz.pyx:180-322)
    add('circulant_ml_3x4', 'Circulant(cm)', {'cm': cplx(rng, 3, 4)})
    add('circulant_ml_2x3x5', 'Circulant(cm)', {'cm': cplx(rng, 2, 3, 5)})
    add('circulant_ml_real', 'Circulant(cm)',
        {'cm': rng.standard_normal((4, 6))}, xdtype=np.float64)
    add('circulant_ml_8x16', 'Circulant(cm)', {'cm': cplx(rng, 8, 16)})
    add('circulant_ml_7x9', 'Circulant(cm)', {'cm': cplx(rng, 7, 9)},
        dense=False)
    add('toeplitz_ml_split', 'Toeplitz(tm, split=sp)',
        {'tm': cplx(rng, 3, 5), 'sp': np.array([2, 3])})
    add('toeplitz_ml_cube', 'Toeplitz(tm)', {'tm': cplx(rng, 3, 5, 3)})
    add('toeplitz_ml_rect', 'Toeplitz(tm, split=sp)',
        {'tm': cplx(rng, 4, 3), 'sp': np.array([4, 1])})
    add('toeplitz_ml_9x7', 'Toeplitz(tm)', {'tm': cplx(rng, 9, 7)})
    # block compositions (fastmat/Blocks.pyx, fastmat/BlockDiag.pyx)
    add('blockdiag_mixed',
        'BlockDiag(Circulant(c), Fourier(5), Diag(d), Hadamard(2))',
        {'c': cplx(rng, 7), 'd': cplx(rng, 4)})
    add('blockdiag_real', 'BlockDiag(Hadamard(3), Diag(d))',
        {'d': rng.standard_normal(5)}, xdtype=np.float64)
    add('blockdiag_one', 'BlockDiag(Toeplitz(tc, tr))',
        {'tc': cplx(rng, 6), 'tr': cplx(rng, 4)})
    add('blocks_2x3',
        'Blocks([[Circulant(c1), Partial(Fourier(9), rows=r6, cols=k9), '
        'Partial(Hadamard(3), rows=r6b, cols=k4)], '
        '[Partial(Circulant(c2), rows=r4, cols=k6), '
        'Partial(Fourier(9), rows=r4b, cols=k9), Diag(d4)]])',
        {'c1': cplx(rng, 6), 'c2': cplx(rng, 6), 'd4': cplx(rng, 4),
         'r6': np.sort(rng.choice(9, 6, replace=False)),
         'r6b': np.sort(rng.choice(8, 6, replace=False)),
         'k4': np.sort(rng.choice(8, 4, replace=False)),
         'r4': np.sort(rng.choice(6, 4, replace=False)),
         'r4b': np.sort(rng.choice(9, 4, replace=False)),
         'k6': np.arange(6), 'k9': np.arange(9)})
    add('blocks_nested',
        'Blocks([[Product(Fourier(4), Diag(d4)), '
        'Kron(Hadamard(1), Circulant(c2))], '
        '[Eye(4), BlockDiag(Fourier(3), Diag(d1))]])',
        {'d4': cplx(rng, 4), 'c2': cplx(rng, 2), 'd1': cplx(rng, 1)})
    add('blocks_real', 'Blocks([[Hadamard(2), Diag(d)], [Diag(e), Eye(4)]])',
        {'d': rng.standard_normal(4), 'e': rng.standard_normal(4)},
        xdtype=np.float64)
    add('blocks_large', 'Blocks([[Circulant(c), Fourier(300)], '
        '[Toeplitz(tc, tr), Diag(d)]])',
        {'c': cplx(rng, 300), 'tc': cplx(rng, 300), 'tr': cplx(rng, 299),
         'd': cplx(rng, 300)}, dense=False)
    # sparse matrices (fastmat/Sparse.pyx), CSR arrays as parameters
    def csr_params(a):
        a = a.tocsr()
        return {'v': a.data, 'ix': a.indices.astype(np.int64),
                'ip': a.indptr.astype(np.int64), 'sh': np.array(a.shape)}
    import scipy.sparse as sps
    sp_c = (sps.random(40, 30, density=0.15, random_state=rng,
                       format='csr') +
            1j * sps.random(40, 30, density=0.15, random_state=rng,
                            format='csr'))
    add('sparse_c', 'Sparse(csr((v, ix, ip), shape=tuple(sh)))',
        csr_params(sp_c))
    add('sparse_real', 'Sparse(csr((v, ix, ip), shape=tuple(sh)))',
        csr_params(sps.random(64, 64, density=0.05, random_state=rng,
                              format='csr')), xdtype=np.float64)
    sp_i = sps.random(20, 25, density=0.3, random_state=rng, format='csr',
                      data_rvs=lambda k: rng.integers(-3, 4, k))
    add('sparse_int', 'Sparse(csr((v, ix, ip), shape=tuple(sh)))',
        csr_params(sp_i.astype(np.int16)), xdtype=np.int8)
    add('sparse_empty_rows', 'Sparse(csr((v, ix, ip), shape=tuple(sh)))',
        csr_params(sps.random(50, 40, density=0.02, random_state=rng,
                              format='csr').astype(np.complex128)))
    add('sparse_product',
        'Product(Sparse(csr((v, ix, ip), shape=tuple(sh))), Fourier(30))',
        csr_params(sp_c))
    add('sparse_long_rows', 'Sparse(csr((v, ix, ip), shape=tuple(sh)))',
        csr_params(sps.random(16, 2000, density=0.5, random_state=rng,
                              format='csr').astype(np.complex128)))
    return out


def main():
    ns = namespace()
    rng = np.random.default_rng(99)
    records = {}
    meta = []
    for name, expr, params, xdt, m, dense in cases():
        env = dict(ns)
        env.update(params)
        op = eval(expr, env)  # noqa: S307 (fixed expressions above)
        n_rows, n_cols = op.shape
        if xdt.kind == 'c':
            x = cplx(rng, n_cols, m).astype(xdt)
            g = cplx(rng, n_rows, m).astype(xdt)
        elif xdt.kind == 'f':
            x = rng.standard_normal((n_cols, m)).astype(xdt)
            g = rng.standard_normal((n_rows, m)).astype(xdt)
        else:
            x = rng.integers(-2, 3, (n_cols, m)).astype(xdt)
            g = rng.integers(-2, 3, (n_rows, m)).astype(xdt)
        y = op.forward(x)
        z = op.backward(g)
        for k, v in params.items():
            records['%s__p_%s' % (name, k)] = np.asarray(v)
        records['%s__x' % name] = x
        records['%s__g' % name] = g
        records['%s__fwd' % name] = y
        records['%s__bwd' % name] = z
        if dense and n_rows * n_cols <= 128 * 128:
            records['%s__dense' % name] = op.reference()
        meta.append(dict(name=name, expr=expr, params=sorted(params),
                         dense=bool(dense and n_rows * n_cols <= 128 * 128), dtype=str(np.dtype(op.dtype)),
                         shape=[int(n_rows), int(n_cols)]))
    np.savez_compressed(os.path.join(HERE, 'operators.npz'), **records)

    # FFT size heuristics (fastmat/core/cmath.pyx:35-214,
    # fastmat/Fourier.pyx:109-122, fastmat/Circulant.pyx:107-124,
    # fastmat/Toeplitz.pyx:225-237)
    from fastmat.core.cmath import _findOptimalFFTSize, _getFFTComplexity
    sizes = np.unique(np.concatenate([
        np.arange(1, 700), np.geomspace(700, 300000, 400).astype(np.int64),
        [1023, 1024, 1025, 4095, 4096, 4097, 4099, 65521, 65536, 65537,
         131041, 131071, 131072, 262143, 262144]]))
    opt = np.array([_findOptimalFFTSize(int(n), 4) for n in sizes])
    opt5 = np.array([_findOptimalFFTSize(int(n), 5) for n in sizes[:600]])
    cpx = np.array([_getFFTComplexity(int(n)) for n in sizes])
    numl = np.array([fm.Fourier(int(n))._numL for n in sizes
                     if n <= 70000])
    circ_sizes = sizes[(sizes <= 70000)][::3]
    circl = np.array([fm.Circulant(np.ones(int(n))).content[0].numRows
                      for n in circ_sizes])
    np.savez_compressed(
        os.path.join(HERE, 'fftsizes.npz'), sizes=sizes, opt=opt, opt5=opt5,
        complexity=cpx, numl=numl, circ_sizes=circ_sizes, circl=circl)

    # the small circulant workload (N = 1024, X 1024 x 16 complex128, seed 0)
    r0 = np.random.default_rng(0)
    c = r0.standard_normal(1024) + 1j * r0.standard_normal(1024)
    x = r0.standard_normal((1024, 16)) + 1j * r0.standard_normal((1024, 16))
    op = fm.Circulant(c)
    np.savez_compressed(os.path.join(HERE, 'circulant1024.npz'), c=c, x=x,
                        fwd=op.forward(x), bwd=op.backward(x))

    with open(os.path.join(HERE, 'operators.json'), 'w') as f:
        json.dump(meta, f, indent=1)
    print('wrote %d operator cases' % len(meta))


def accessors():
    """The reference's dense accessors on the small cases with a dense
    reference (fastmat/Matrix.pyx:360-658 and 1035-1206): ``array``,
    ``getCols`` / ``getRows`` of a few indices, elements ``A[i, j]``,
    ``colNorms`` / ``rowNorms`` and (up to 64 x 64) the normalized
    operators' arrays, written to accessors.npz.  The operators are rebuilt from the
    parameters stored in operators.npz."""
    ns = namespace()
    data = np.load(os.path.join(HERE, 'operators.npz'))
    with open(os.path.join(HERE, 'operators.json')) as f:
        meta = json.load(f)
    rec = {}
    names = []
    for m in meta:
        if not m['dense']:
            continue
        name = m['name']
        env = dict(ns)
        env.update({k: data['%s__p_%s' % (name, k)] for k in m['params']})
        op = eval(m['expr'], env)  # noqa: S307 (fixture expressions)
        n_rows, n_cols = op.shape
        cols = np.unique(np.array([0, n_cols // 2, n_cols - 1]))
        rows = np.unique(np.array([0, n_rows // 3, n_rows - 1]))
        got = {}
        for key, fn in (
                ('array', lambda: op.array),
                ('cols', lambda: op.getCols(cols)),
                ('rows', lambda: op.getRows(rows)),
                ('items', lambda: np.array([op[int(i), int(j)]
                                            for i in rows for j in cols])),
                ('colnorms', lambda: op.colNorms),
                ('rownorms', lambda: op.rowNorms),
                ('colnormalized', lambda: op.colNormalized.array),
                ('rownormalized', lambda: op.rowNormalized.array)):
            try:
                got[key] = np.asarray(fn())
            except ValueError:
                # e.g. normalizing a zero-norm column: the GPU form must
                # raise too
                got[key + '_raises'] = np.array(1)
            except Exception as e:  # noqa: BLE001 (recorded as absent)
                print('%s.%s: reference raised %s' % (name, key,
                                                      type(e).__name__))
        if n_rows * n_cols > 64 * 64:
            # the normalized arrays only for the smaller operators
            for k in ('colnormalized', 'rownormalized'):
                got.pop(k, None)
                got.pop(k + '_raises', None)
        for key, v in got.items():
            rec['%s__%s' % (name, key)] = v
        rec['%s__colidx' % name] = cols
        rec['%s__rowidx' % name] = rows
        names.append(name)
    np.savez_compressed(os.path.join(HERE, 'accessors.npz'), **rec)
    print('wrote accessors for %d cases' % len(names))


if __name__ == '__main__':
    if sys.argv[1:] == ['--accessors']:
        accessors()
    else:
        main()
        accessors()
