"""Host logic of the differentiable path (no GPU): how an operator tree is
cut into engine plans, parameter registration and the Toeplitz embedding."""

import numpy as np
import pytest

torch = pytest.importorskip('torch')

import fastmat_gb300 as fg  # noqa: E402
from fastmat_gb300 import autograd as fa  # noqa: E402


def test_smooth_length():
    assert fa._smooth_at_least(1) == 1
    assert fa._smooth_at_least(193) == 196
    assert fa._smooth_at_least(8191) == 8192
    for n in range(1, 400):
        v = fa._smooth_at_least(n)
        assert v >= n
        m = v
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        assert m == 1


@pytest.mark.parametrize('nr,nc,L', [(5, 4, 8), (3, 1, 3), (1, 6, 7),
                                     (7, 7, 16)])
def test_toeplitz_embedding(nr, nc, L):
    rng = np.random.default_rng(nr * nc)
    vc = rng.standard_normal(nr) + 1j * rng.standard_normal(nr)
    vr = rng.standard_normal(nc - 1) + 1j * rng.standard_normal(nc - 1)
    emb = fa._toeplitz_embedding(vc, vr, L)
    i = np.arange(L)
    C = emb[(i[:, None] - i[None, :]) % L]
    T = fg.Toeplitz(vc, vr).reference() if nc > 1 else vc[:, None]
    assert np.array_equal(C[:nr, :nc], T)


def test_embedding_too_short():
    with pytest.raises(ValueError):
        fa._toeplitz_embedding(np.ones(4), np.ones(3), 6)


def test_diag_chain_segments():
    d = np.arange(1, 9) * (1 + 0.5j)
    D = fg.Diag(d)
    op = fg.Product(fg.Hadamard(3), D, fg.Fourier(8))
    mod = fa.Operator(op, device='cpu')
    names = [n for n, _ in mod.named_parameters()]
    assert names == ['diag0']
    prog = mod._program()
    assert len(prog.segs) == 2
    s0, s1 = prog.segs
    assert s0.head is None and [type(t) for t in s0.terms] == [fg.Fourier]
    assert s1.head[0] == 'diag' and s1.head[1] is D
    assert [type(t) for t in s1.terms] == [fg.Diag, fg.Hadamard]
    # the adjoint plan of segment 0 carries the pivot of segment 1
    assert isinstance(s0.bop, fg.Product)
    assert [type(t) for t in s0.bop._content] == [fg.Diag, fg.Fourier]


def test_partial_expansion_and_frozen_leaves():
    d1 = np.ones(16) * 2.0
    d2 = np.arange(16.0)
    D1, D2 = fg.Diag(d1), fg.Diag(d2)
    op = fg.Partial(fg.Product(D1, fg.Hadamard(4), D2), rows=[1, 5, 7],
                    cols=np.arange(10))
    mod = fa.Operator(op, trainable=[D2], device='cpu')
    assert [n for n, _ in mod.named_parameters()] == ['diag0']
    prog = mod._program()
    # scatter(cols) | D2 pivot: [D2, Hadamard, D1, gather(rows)]
    assert len(prog.segs) == 2
    s0, s1 = prog.segs
    assert len(s0.terms) == 1 and isinstance(s0.terms[0], fg.Partial)
    assert s0.terms[0].shape == (16, 10)
    assert s1.terms[0] is D2
    assert s1.terms[-1].shape == (3, 16)
    assert s1.terms[2] is D1


def test_no_trainable_is_one_plan():
    op = fg.Product(fg.Hadamard(3), fg.Diag(np.ones(8)))
    mod = fa.Operator(op, trainable=False, device='cpu')
    prog = mod._program()
    assert len(prog.segs) == 1 and prog.segs[0].op is op


def test_rebuild_replaces_leaves_only():
    D = fg.Diag(np.ones(4))
    H = fg.Hadamard(2)
    op = fg.Product(H, D, 3.0)
    new, mapping = fa._rebuild(op, {id(D): np.full(4, 2.0)})
    assert new is not op
    assert new._content[0] is H
    nd = new._content[1]
    assert np.array_equal(nd.vecD, np.full(4, 2.0))
    assert mapping[id(nd)] == id(D)
    assert complex(new._scalar) == 3.0


def test_parameter_changes_rebuild_program():
    D = fg.Diag(np.ones(4, dtype=np.complex128))
    mod = fa.Operator(fg.Product(fg.Hadamard(2), D), device='cpu')
    p1 = mod._program()
    assert mod._program() is p1
    with torch.no_grad():
        mod.diag0.mul_(3)
    p2 = mod._program()
    assert p2 is not p1
    leaf = p2.segs[1].head[1]
    assert np.allclose(leaf.vecD, 3.0)


def test_fp32_parameters_are_single():
    op = fg.Product(fg.Diag(np.ones(4, dtype=np.complex128)),
                    fg.Hadamard(2), precision='fp32')
    mod = fa.Operator(op, device='cpu')
    assert mod.diag0.dtype == torch.complex64
