"""Differentiable path: gradients of the engine's matvec against autograd
through the dense matrix and against FP64 central finite differences.

The chain is the one of the differentiable workload: y = Partial(rows) *
Circulant(c) * Diag(d) * x with a loss ||y - b||^2, here at N = 4096 where
the dense matrix is affordable; further cases cover Toeplitz, Sum, Kron
factors, adjoint wrappers and a dense term.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _rel(a, b):
    a = a.detach().cpu().numpy() if hasattr(a, 'detach') else np.asarray(a)
    b = b.detach().cpu().numpy() if hasattr(b, 'detach') else np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _chain(fg, N, seed=0, prec='native', form='partial'):
    rng = np.random.default_rng(seed)
    c, d = _cplx(rng, N), _cplx(rng, N)
    rows = np.sort(rng.choice(N, N // 4, replace=False))
    C, D = fg.Circulant(c), fg.Diag(d)
    if form == 'partial':
        op = fg.Partial(fg.Product(C, D), rows=rows, precision=prec)
    else:
        op = fg.Product(fg.Partial(fg.Eye(N), rows=rows), C, D,
                        precision=prec)
    return op, c, d, rows, rng


def _dense_loss(c, d, rows, x, b):
    """Dense reference of the chain in torch (complex128, autograd)."""
    torch = _torch()
    N = c.shape[0]
    i = torch.arange(N, device=c.device)
    Cm = c[(i[:, None] - i[None, :]) % N]
    A = (Cm * d[None, :])[torch.as_tensor(rows, device=c.device)]
    y = A @ x
    return (y - b).abs().pow(2).sum()


@pytest.mark.parametrize('form', ['partial', 'product'])
def test_chain_grads_match_dense_autograd(form):
    torch = _torch()
    import fastmat_gb300 as fg
    from fastmat_gb300 import autograd as fa
    N, M = 4096, 4
    op, c, d, rows, rng = _chain(fg, N, form=form)
    x0, b0 = _cplx(rng, N, M), _cplx(rng, len(rows), M)
    mod = fa.Operator(op)
    x = torch.tensor(x0, device='cuda', requires_grad=True)
    b = torch.tensor(b0, device='cuda')
    y = mod(x)
    loss = (y - b).abs().pow(2).sum()
    loss.backward()
    # dense reference
    ct = torch.tensor(c, device='cuda', requires_grad=True)
    dt = torch.tensor(d, device='cuda', requires_grad=True)
    xr = torch.tensor(x0, device='cuda', requires_grad=True)
    lr = _dense_loss(ct, dt, rows, xr, b)
    lr.backward()
    assert abs(loss.item() - lr.item()) <= 1e-10 * lr.item()
    params = dict(mod.named_parameters())
    assert _rel(x.grad, xr.grad) <= 1e-10
    assert _rel(params['circulant0'].grad, ct.grad) <= 1e-10
    assert _rel(params['diag0'].grad, dt.grad) <= 1e-10


def test_chain_grads_match_finite_differences():
    """Directional derivatives Re<grad, delta> vs central differences of
    the FP64 loss evaluated by the engine's forward."""
    torch = _torch()
    import fastmat_gb300 as fg
    from fastmat_gb300 import autograd as fa
    N, M = 4096, 2
    op, c, d, rows, rng = _chain(fg, N, seed=1)
    x0, b0 = _cplx(rng, N, M), _cplx(rng, len(rows), M)
    mod = fa.Operator(op)
    x = torch.tensor(x0, device='cuda', requires_grad=True)
    b = torch.tensor(b0, device='cuda')
    loss = (mod(x) - b).abs().pow(2).sum()
    loss.backward()
    P = dict(mod.named_parameters())
    gc, gd, gx = (P['circulant0'].grad.cpu().numpy(),
                  P['diag0'].grad.cpu().numpy(), x.grad.cpu().numpy())

    def L(cc, dd, xx):
        o = fg.Partial(fg.Product(fg.Circulant(cc), fg.Diag(dd)), rows=rows)
        y = o.forward(xx)
        return float(np.sum(np.abs(y - b0) ** 2))

    eps = 1e-6
    for which in range(3):
        for kind in (1.0, 1j):
            delta = [np.zeros_like(c), np.zeros_like(d), np.zeros_like(x0)]
            delta[which] = kind * (
                rng.standard_normal(delta[which].shape))
            up = L(c + eps * delta[0], d + eps * delta[1],
                   x0 + eps * delta[2])
            dn = L(c - eps * delta[0], d - eps * delta[1],
                   x0 - eps * delta[2])
            fd = (up - dn) / (2 * eps)
            g = (gc, gd, gx)[which]
            an = float(np.real(np.vdot(g, delta[which])))
            assert abs(fd - an) <= 1e-6 * max(abs(an), 1.0), (which, kind,
                                                              fd, an)


def test_fp32_grads_within_stated_bound():
    """The complex64 form of the chain: gradients within 1e-5 (relative to
    the largest entry) of the FP64 gradients."""
    torch = _torch()
    import fastmat_gb300 as fg
    from fastmat_gb300 import autograd as fa
    N, M = 1 << 14, 8
    out = {}
    for prec in ('native', 'fp32'):
        op, c, d, rows, rng = _chain(fg, N, seed=2, prec=prec)
        x0, b0 = _cplx(rng, N, M), _cplx(rng, len(rows), M)
        dt = torch.complex64 if prec == 'fp32' else torch.complex128
        mod = fa.Operator(op)
        x = torch.tensor(x0, device='cuda', dtype=dt, requires_grad=True)
        b = torch.tensor(b0, device='cuda', dtype=dt)
        y = mod(x)
        assert y.dtype == dt
        (y - b).abs().pow(2).sum().backward()
        P = dict(mod.named_parameters())
        out[prec] = (x.grad, P['circulant0'].grad, P['diag0'].grad)
    for g32, g64 in zip(out['fp32'], out['native']):
        assert g32.dtype == torch.complex64
        assert _rel(g32, g64) <= 1e-5


def _check_against_dense(op, build_dense, params_np, shape_x, seed, tol):
    """Gradients of Operator(op) vs autograd through a torch dense matrix
    built from the same parameter values by build_dense(*tensors)."""
    torch = _torch()
    from fastmat_gb300 import autograd as fa
    rng = np.random.default_rng(seed)
    x0 = _cplx(rng, *shape_x)
    mod = fa.Operator(op)
    x = torch.tensor(x0, device='cuda', requires_grad=True)
    y = mod(x)
    b0 = _cplx(rng, *tuple(y.shape))
    b = torch.tensor(b0, device='cuda')
    (y - b).abs().pow(2).sum().backward()
    ts = [torch.tensor(p, device='cuda', dtype=torch.complex128,
                       requires_grad=True) for p in params_np]
    xr = torch.tensor(x0, device='cuda', requires_grad=True)
    A = build_dense(*ts)
    ((A @ xr) - b).abs().pow(2).sum().backward()
    assert _rel(x.grad, xr.grad) <= tol
    for p, t in zip(mod.parameters(), ts):
        assert _rel(p.grad, t.grad) <= tol, type(p)


def _toeplitz_dense(tenT, nr, nc):
    torch = _torch()
    vc, vr = tenT[:nr], tenT[nr:]
    full = torch.cat([vr, vc])
    i = torch.arange(nr, device=tenT.device)[:, None]
    j = torch.arange(nc, device=tenT.device)[None, :]
    return full[i - j + nc - 1]


def _circ_dense(c):
    torch = _torch()
    n = c.shape[0]
    i = torch.arange(n, device=c.device)
    return c[(i[:, None] - i[None, :]) % n]


@pytest.mark.parametrize('nr,nc', [(97, 60), (64, 64), (33, 120)])
def test_toeplitz_grads(nr, nc):
    import fastmat_gb300 as fg
    rng = np.random.default_rng(nr + nc)
    vc, vr = _cplx(rng, nr), _cplx(rng, nc - 1)
    d = _cplx(rng, nc)
    op = fg.Product(fg.Toeplitz(vc, vr), fg.Diag(d))
    tenT = np.concatenate([vc, vr])
    _check_against_dense(
        op, lambda t, dd: _toeplitz_dense(t, nr, nc) * dd[None, :],
        [tenT, d], (nc, 3), 5, 1e-10)


def test_sum_and_adjoint_terms():
    import fastmat_gb300 as fg
    n = 300
    rng = np.random.default_rng(7)
    c, d = _cplx(rng, n), _cplx(rng, n)
    op = fg.Product(fg.Sum(fg.Circulant(c), fg.Hermitian(fg.Diag(d))),
                    fg.Fourier(n))
    i = np.arange(n)
    F = np.exp(-2j * np.pi * np.outer(i, i) / n)

    def dense(ct, dt):
        torch = _torch()
        Ft = torch.tensor(F, device='cuda')
        return (_circ_dense(ct) + torch.diag(dt.conj())) @ Ft

    _check_against_dense(op, dense, [c, d], (n, 2), 8, 1e-10)


def test_kron_factor_grads():
    torch = _torch()
    import fastmat_gb300 as fg
    rng = np.random.default_rng(9)
    c, d = _cplx(rng, 16), _cplx(rng, 8)
    Md = _cplx(rng, 4, 4)
    op = fg.Kron(fg.Circulant(c), fg.Diag(d), fg.Matrix(Md))

    def dense(ct, dt, mt):
        return torch.kron(torch.kron(_circ_dense(ct), torch.diag(dt)), mt)

    _check_against_dense(op, dense, [c, d, Md], (16 * 8 * 4, 3), 10, 1e-10)


def test_partial_columns_and_scalar():
    torch = _torch()
    import fastmat_gb300 as fg
    rng = np.random.default_rng(11)
    n = 128
    c = _cplx(rng, n)
    cols = np.sort(rng.choice(n, 40, replace=False))
    op = fg.Product(fg.Partial(fg.Circulant(c), cols=cols), 2.5 - 1j)

    def dense(ct):
        return (2.5 - 1j) * _circ_dense(ct)[:, torch.as_tensor(
            cols, device='cuda')]

    _check_against_dense(op, dense, [c], (40, 3), 12, 1e-10)


def test_input_only_matvec_and_param_update():
    """matvec(op, x) differentiates x only; after an in-place parameter
    update the plans are rebuilt from the new values."""
    torch = _torch()
    import fastmat_gb300 as fg
    from fastmat_gb300 import autograd as fa
    rng = np.random.default_rng(13)
    n = 256
    c = _cplx(rng, n)
    C = fg.Circulant(c)
    x = torch.tensor(_cplx(rng, n, 2), device='cuda', requires_grad=True)
    y = fa.matvec(C, x)
    g = torch.tensor(_cplx(rng, n, 2), device='cuda')
    (y.conj() * g).real.sum().backward()
    want = C.backward(g.cpu().numpy())
    assert _rel(x.grad, want) <= 1e-12
    mod = fa.Operator(C)
    p = mod.circulant0
    with torch.no_grad():
        p.mul_(2.0)
    y2 = mod(x.detach())
    assert _rel(y2, 2 * C.forward(x.detach().cpu().numpy())) <= 1e-12
