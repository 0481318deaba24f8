"""Many operators in one persistent launch: every result must equal the
operator's own forward/backward, and match the oracle (FP64) within the
complex64 bound."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def _next_prime_below(n):
    def prime(k):
        if k < 2:
            return False
        i = 2
        while i * i <= k:
            if k % i == 0:
                return False
            i += 1
        return True
    while not prime(n):
        n -= 1
    return n


def _mixed_ops(rng, count, prec, max_n=65536, max_cols=4):
    """Circulant / Toeplitz / Fourier operators, sizes log-uniform in
    [64, max_n], 30% prime or non-power-of-two, the rest powers of two."""
    import fastmat_gb300 as fg
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(64), np.log(max_n)))))
        if rng.uniform() < 0.3:
            n = _next_prime_below(n) if i % 2 else n + (n % 2 == 0) * 6 + 3
        else:
            n = 1 << int(round(np.log2(n)))
        kind = i % 3
        if kind == 0:
            c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            op, oop = fg.Circulant(c, precision=prec), fo.Circulant(c)
        elif kind == 1:
            vc = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            vr = rng.standard_normal(n - 1) + 1j * rng.standard_normal(n - 1)
            op, oop = (fg.Toeplitz(vc, vr, precision=prec),
                       fo.Toeplitz(vc, vr))
        else:
            op, oop = fg.Fourier(n, precision=prec), fo.Fourier(n)
        m = int(rng.integers(1, max_cols + 1))
        out.append((op, oop, m))
    return out


@pytest.mark.parametrize('backward', [False, True])
def test_batch_matches_single_operator_calls(backward):
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(5)
    ops = _mixed_ops(rng, 36, 'fp32')
    xs = []
    for op, _, m in ops:
        n = op.numRows if backward else op.numCols
        x = (rng.standard_normal((n, m)) +
             1j * rng.standard_normal((n, m))).astype(np.complex64)
        xs.append(x)
    items = [(op, torch.from_numpy(x.T.copy()).cuda().t())
             for (op, _, _), x in zip(ops, xs)]
    b = fg.Batch(items, backward=backward)
    launches, levels, tiles = b.info()
    assert levels >= 2 and launches >= len(ops)
    outs = [y.cpu().numpy() for y in b.run()]
    b.check()
    for (op, oop, _), x, y in zip(ops, xs, outs):
        single = (op.backward(x) if backward else op.forward(x))
        assert y.dtype == np.complex64 and y.shape == single.shape
        assert fo.rel_err(y, single) <= 1e-6, repr(op)
        ref = oop.backward(x) if backward else oop.forward(x)
        assert fo.rel_err(y, ref) <= 1e-5, repr(op)


def test_batch_graph_replay_and_rebinding():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(6)
    ops = _mixed_ops(rng, 12, 'fp32', max_n=5000)
    items = []
    for op, _, m in ops:
        x = torch.randn(m, op.numCols, dtype=torch.complex64,
                        device='cuda').t()
        items.append((op, x))
    b = fg.Batch(items)
    first = [y.clone() for y in b.run(graph=True)]
    for _, x in items:
        x.mul_(2)
    second = b.run(graph=True)
    torch.cuda.synchronize()
    b.check()
    for y1, y2 in zip(first, second):
        assert torch.allclose(2 * y1, y2, rtol=1e-5, atol=1e-4)


def test_batch_double_float():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(7)
    ops = _mixed_ops(rng, 9, 'native', max_n=20000, max_cols=2)
    xs = [rng.standard_normal((op.numCols, m)) +
          1j * rng.standard_normal((op.numCols, m)) for op, _, m in ops]
    items = [(op, torch.from_numpy(x.T.copy()).cuda().t())
             for (op, _, _), x in zip(ops, xs)]
    outs = [y.cpu().numpy() for y in fg.Batch(items).run()]
    for (op, oop, _), x, y in zip(ops, xs, outs):
        assert y.dtype == np.complex128
        assert fo.rel_err(y, oop.forward(x)) <= 1e-11, repr(op)


def test_batch_rejects_mixed_compute_types():
    import torch
    import fastmat_gb300 as fg
    a = fg.Fourier(64, precision='fp32')
    b = fg.Fourier(64)
    x = torch.zeros(64, 1, dtype=torch.complex64, device='cuda')
    with pytest.raises(ValueError):
        fg.Batch([(a, x), (b, x.to(torch.complex128))])
