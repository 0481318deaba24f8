"""Pin the CPU oracle against the reference's own outputs (golden fixtures).
"""

import numpy as np
from scipy.sparse import csr_matrix
import pytest

from oracle import fm_oracle as fo
from tests.golden_cases import (load_accessors, load_cases,
                                load_circulant1024, load_fftsizes, tolerance)

CASES = load_cases()

NS = dict(Fourier=fo.Fourier, Circulant=fo.Circulant, Toeplitz=fo.Toeplitz,
          Hadamard=fo.Hadamard, Kron=fo.Kron, Diag=fo.Diag,
          Partial=fo.Partial, Permutation=fo.Permutation,
          Product=fo.Product, Sum=fo.Sum, Hermitian=fo.Hermitian,
          Conjugate=fo.Conjugate, Transpose=fo.Transpose, Eye=fo.Eye,
          Matrix=fo.Dense, Blocks=fo.Blocks, BlockDiag=fo.BlockDiag,
           Sparse=fo.Sparse, csr=csr_matrix, np=np)


def expected_dtype(op_dtype, x_dtype):
    """fastmat's output-type contract (fastmat/inspect/test.py:160-170)."""
    return np.dtype(fo.promote(op_dtype, x_dtype))


@pytest.mark.parametrize('case', CASES, ids=lambda c: c.name)
def test_oracle_matches_reference(case):
    op = case.build(NS)
    assert op.shape == case.shape
    y = op.forward(case.x)
    z = op.backward(case.g)
    assert y.shape == case.fwd.shape and z.shape == case.bwd.shape
    assert y.dtype == expected_dtype(case.dtype, case.x.dtype)
    if np.issubdtype(case.fwd.dtype, np.integer):
        assert np.array_equal(y, case.fwd)
        assert np.array_equal(z, case.bwd)
    else:
        assert fo.rel_err(y, case.fwd) <= tolerance(case.fwd, case.x)
        assert fo.rel_err(z, case.bwd) <= tolerance(case.bwd, case.g)
    if case.dense is not None:
        d = op.dense()
        assert fo.rel_err(d, case.dense) <= 1e-12


ACC = load_accessors()


@pytest.mark.parametrize('case', [c for c in CASES if c.name in ACC],
                         ids=lambda c: c.name)
def test_oracle_pins_accessor_fixtures(case):
    """The reference's array / getCols / getRows / elements / norms agree
    with the oracle's dense matrix."""
    acc = ACC[case.name]
    d = case.build(NS).dense()
    scale = max(1e-300, float(np.max(np.abs(d))))

    def close(a, b):
        return float(np.max(np.abs(np.asarray(a) - np.asarray(b)),
                            initial=0.0)) / scale <= 1e-12

    ci, ri = acc['colidx'], acc['rowidx']
    assert close(acc['array'], d)
    assert close(acc['cols'], d[:, ci])
    assert close(acc['rows'], d[ri, :])
    assert close(acc['items'], d[np.ix_(ri, ci)].reshape(-1))
    assert np.allclose(acc['colnorms'], np.linalg.norm(d, axis=0),
                       rtol=1e-12, atol=1e-12 * scale)
    assert np.allclose(acc['rownorms'], np.linalg.norm(d, axis=1),
                       rtol=1e-12, atol=1e-12 * scale)
    if 'colnormalized' in acc:
        assert close(acc['colnormalized'] * np.linalg.norm(d, axis=0), d)
    if 'rownormalized' in acc:
        assert close(acc['rownormalized'] *
                     np.linalg.norm(d, axis=1)[:, None], d)
    if 'colnormalized_raises' in acc:
        assert np.any(np.linalg.norm(d, axis=0) == 0)
    if 'rownormalized_raises' in acc:
        assert np.any(np.linalg.norm(d, axis=1) == 0)


def test_fft_size_heuristics_match_reference():
    g = load_fftsizes()
    sizes = g['sizes']
    opt = [fo.optimal_fft_size(int(n), 4) for n in sizes]
    assert np.array_equal(opt, g['opt'])
    opt5 = [fo.optimal_fft_size(int(n), 5) for n in sizes[:600]]
    assert np.array_equal(opt5, g['opt5'])
    cpx = [fo.fft_complexity(int(n)) for n in sizes]
    assert np.array_equal(np.float32(cpx), np.float32(g['complexity']))
    numl = [fo.fourier_bluestein_length(int(n)) for n in sizes
            if n <= 70000]
    assert np.array_equal(numl, g['numl'])
    circl = [fo.circulant_length(int(n)) for n in g['circ_sizes']]
    assert np.array_equal(circl, g['circl'])


def test_circulant1024_workload():
    g = load_circulant1024()
    op = fo.Circulant(g['c'])
    assert fo.rel_err(op.forward(g['x']), g['fwd']) <= 1e-13
    assert fo.rel_err(op.backward(g['x']), g['bwd']) <= 1e-13
    assert fo.rel_err(op.dense() @ g['x'], g['fwd']) <= 1e-13


def test_exact_dft_anchor():
    rng = np.random.default_rng(5)
    for n in (127, 4099):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        rows = [0, 1, n // 3, n - 1]
        ex = fo.exact_dft_rows(x, rows)
        assert fo.rel_err(np.fft.fft(x)[rows], ex[:, 0]) < 1e-13
        assert fo.rel_err(fo.Fourier(n).forward(x)[rows], ex[:, 0]) < 5e-12
