"""Parity at the benchmark configurations' full sizes, against the oracle
(the numpy restatement of fastmat's CPU algorithm), not against another GPU
form:

* Hadamard(22) on all 64 float32 columns: the FP32 and BF16 tensor-core
  forms against the FP64 oracle (1e-5), the FP32 form bit-identical to the
  oracle's float32 transform (fastmat's own butterfly order) on 8 columns;
* Kron(Fourier(256), Hadamard(8), Circulant(128)), N = 8,388,608: the FP32
  form on 2 full columns against the FP64 oracle (1e-5) and the FP64 form
  (double-float) on the same columns (1e-12);
* Partial(rows) Circulant Diag at N = 2^18 on all 32 columns;
* the 512-operator batch (sizes up to 65536, up to 32 columns each): every
  8th operator, all its columns, against the oracle."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_hadamard22_all_64_columns_fp32_and_bf16():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(22)
    n, M = 1 << 22, 64
    x = rng.standard_normal((n, M), dtype=np.float32)
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    y32 = fg.Hadamard(22, precision='fp32').forward(xt).cpu().numpy()
    ybf = fg.Hadamard(22, precision='bf16').forward(xt).cpu().numpy()
    del xt
    H = fo.Hadamard(22)
    worst32 = worstbf = 0.0
    for c0 in range(0, M, 8):
        cols = slice(c0, c0 + 8)
        ref = H.forward(x[:, cols].astype(np.float64))
        worst32 = max(worst32, fo.rel_err(y32[:, cols], ref))
        worstbf = max(worstbf, fo.rel_err(ybf[:, cols], ref))
    assert worst32 <= 1e-5, worst32
    assert worstbf <= 1e-5, worstbf
    pick = np.arange(0, M, 8)
    assert np.array_equal(y32[:, pick],
                          H.forward(np.asfortranarray(x[:, pick])))


def test_kron_workload_fp32_form_two_full_columns_against_oracle():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(1)
    c = cplx(rng, 128)
    O = fo.Kron(fo.Fourier(256), fo.Hadamard(8), fo.Circulant(c))
    x = cplx(rng, 256 * 256 * 128, 2)
    ref = O.forward(x)
    K32 = fg.Kron(fg.Fourier(256), fg.Hadamard(8), fg.Circulant(c),
                  precision='fp32')
    y32 = K32.forward(x.astype(np.complex64))
    assert y32.dtype == np.complex64
    assert fo.rel_err(y32, ref) <= 1e-5
    K64 = fg.Kron(fg.Fourier(256), fg.Hadamard(8), fg.Circulant(c))
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    y64 = K64.forward(xt).cpu().numpy()
    assert fo.rel_err(y64, ref) <= 1e-12


def test_chain_all_32_columns():
    import fastmat_gb300 as fg
    rng = np.random.default_rng(3)
    n = 1 << 18
    c, d = cplx(rng, n), cplx(rng, n)
    rows = np.sort(rng.choice(n, n // 4, replace=False))
    A = fg.Partial(fg.Product(fg.Circulant(c), fg.Diag(d)), rows=rows)
    A32 = fg.Partial(fg.Product(fg.Circulant(c), fg.Diag(d)), rows=rows,
                     precision='fp32')
    O = fo.Partial(fo.Product(fo.Circulant(c), fo.Diag(d)), rows=rows)
    x = cplx(rng, n, 32)
    g = cplx(rng, n // 4, 32)
    ref = O.forward(x)
    assert fo.rel_err(A.forward(x), ref) <= 1e-12
    assert fo.rel_err(A32.forward(x.astype(np.complex64)), ref) <= 1e-5
    assert fo.rel_err(A.backward(g), O.backward(g)) <= 1e-12


def _batch_specs():
    """The benchmark's 512-operator batch (seed 0): Circulant / Toeplitz /
    Fourier uniformly, sizes log-uniform in [64, 65536], 30% prime or
    non-power-of-two, 1-32 columns."""
    import importlib.util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        'bench_module', os.path.join(root, 'bench.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, mod.batched_specs(seed=0)


def test_full_512_operator_batch_against_oracle():
    import torch
    import fastmat_gb300 as fg
    mod, specs = _batch_specs()
    ops = mod.batched_ops(fg, specs, 'fp32')
    oops = mod.batched_ops(fo, specs)
    rng = np.random.default_rng(100)
    xs = [torch.from_numpy((rng.standard_normal((m, op.numCols)) +
                            1j * rng.standard_normal((m, op.numCols)))
                           .astype(np.complex64)).cuda().t()
          for op, m in ops]
    batch = fg.Batch([(op, x) for (op, _), x in zip(ops, xs)])
    batch.run(graph=True)
    batch.check()
    ys = batch.outputs
    assert len(ys) == 512
    worst = 0.0
    for i in range(0, 512, 8):
        x = xs[i].cpu().numpy().astype(np.complex128)
        worst = max(worst, fo.rel_err(ys[i].cpu().numpy(),
                                      oops[i][0].forward(x)))
    assert worst <= 1e-5, worst
    # the graph replays the same launch: identical results
    first = [ys[i].clone() for i in range(0, 512, 64)]
    batch.run(graph=True)
    batch.check()
    for k, i in enumerate(range(0, 512, 64)):
        assert torch.equal(batch.outputs[i], first[k])
