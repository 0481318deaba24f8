"""Differentiable matvec: torch.autograd on the GB300 engine.

``Operator(op)`` wraps a fastmat operator tree as a ``torch.nn.Module``
whose defining vectors become parameters:

* ``Diag``: the diagonal ``vecD``;
* ``Circulant`` (1-level): the defining column ``tenC``;
* ``Toeplitz`` (1-level): ``tenT`` = [vecC, vecR] (fastmat's order);
* a dense ``Matrix``: its array (used as a Kron factor or a chain term).

``Operator(op)(x)`` computes ``op.forward(x)`` for a CUDA tensor ``x`` of
shape (n,) or (n, M) and is differentiable with respect to ``x`` and every
parameter.  Gradients follow torch's convention for complex tensors
(d/dRe + i d/dIm of a real loss): the input gradient is the adjoint matvec
``A^H g`` (fastmat's backward, fastmat/Matrix.pyx:1937-2007, run by the
engine) and the parameter gradients are

* Diag:      grad_d[j] = sum over columns of g[j] * conj(x[j]);
* Circulant: grad_c = F^H (sum_cols conj(F x) * (F g)) / n, the circular
  cross-correlation of g with x (F the unnormalised DFT);
* Toeplitz:  the same in the circulant of size L >= rows + cols - 1 that
  embeds the Toeplitz matrix, read back at the lags of vecC and vecR;
* Kron factors: the same formulas along the factor's mode, the other
  factors applied to the input first (they commute);
* a dense matrix M: sum_cols g x^H.

The column sums run in the engine's reduction kernel (fm_reduce_mulconj),
every transform in the engine's plans.

How a chain is evaluated.  A Product (fastmat/Product.pyx:205-240) is
flattened into its terms; Partial wrappers (fastmat/Partial.pyx:268-294)
become a scatter, the inner chain and a gather.  The chain is cut at every
trainable term ("pivot") into segments, each run as one fused engine plan.
A trainable Circulant C = F^H diag(S) F / n (S = F c) is split across two
segments: the one before it ends with F and saves the spectrum of C's
input, the one after starts with diag(S / n) and F^H.  The backward pass
walks the segments from the output: one plan per segment computes the
gradient at the segment's pivot (the next segment's pivot adjoint fused in),
the reduction kernel turns it and the saved segment input into the pivot's
parameter gradient.  For Partial(rows) * Circulant * Diag the forward is
two plans, the backward two plans, one reduction and one fused
reduction + diagonal adjoint that gives grad_x and grad_d together.

Parameters that changed since the last call (an optimiser step) rebuild
the engine plans from their current values.
"""

import numpy as np

from . import _native
from . import types as T
from .matrix import (Conjugate, Hermitian, Matrix, Transpose, _numpy_dtype,
                     _torch_dtype)
from .operators import (Circulant, Diag, Eye, Fourier, Kron, Partial,
                        Product, Sum, Toeplitz)


def _torch():
    import torch
    return torch


# ---------------------------------------------------------------- tree
def _children(m):
    if isinstance(m, (Circulant, Toeplitz)):
        return ()
    if isinstance(m, (Product, Sum, Kron, Partial, Hermitian, Conjugate)):
        return tuple(m._content)
    return ()


def _is_dense(m):
    return type(m) is Matrix and m._array is not None


def _is_param_leaf(m):
    # multi-level Circulant / Toeplitz are applied but not trained
    if isinstance(m, Circulant):
        return m.tenC.ndim == 1
    if isinstance(m, Toeplitz):
        return m.tenT.ndim == 1
    return isinstance(m, Diag) or _is_dense(m)


def _leaves(m, out=None):
    if out is None:
        out = []
    if _is_param_leaf(m):
        if all(m is not o for o in out):
            out.append(m)
        return out
    for c in _children(m):
        _leaves(c, out)
    return out


def _leaf_value(m):
    if isinstance(m, Diag):
        return m.vecD
    if isinstance(m, Circulant):
        return m.tenC
    if isinstance(m, Toeplitz):
        return m.tenT
    return m._array


def _props(m):
    return {'minType': m._minType, 'precision': m._precision}


def _rebuild(m, vals):
    """Copy of the tree with the leaves in `vals` (id -> array) replaced;
    returns (new tree, {id(new leaf): id(old leaf)})."""
    mapping = {}

    def rec(m):
        if _is_param_leaf(m):
            v = vals.get(id(m))
            if v is None:
                mapping[id(m)] = id(m)
                return m
            if isinstance(m, Diag):
                new = Diag(v, **_props(m))
            elif isinstance(m, Circulant):
                new = Circulant(v, optimize=m._optimize,
                                maxStage=m._maxStage, **_props(m))
            elif isinstance(m, Toeplitz):
                new = Toeplitz(v, split=m._split, optimize=m._optimize,
                               maxStage=m._maxStage, **_props(m))
            else:
                new = Matrix(v, **_props(m))
            mapping[id(new)] = id(m)
            return new
        kids = _children(m)
        if not kids:
            return m
        new_kids = [rec(c) for c in kids]
        if all(a is b for a, b in zip(new_kids, kids)):
            return m
        if isinstance(m, Product):
            args = list(new_kids)
            if m._scalar != 1:
                args.append(m._scalar[()])
            return Product(*args, typeExpansion=m.dtype, **_props(m))
        if isinstance(m, Sum):
            return Sum(*new_kids, **_props(m))
        if isinstance(m, Kron):
            return Kron(*new_kids, typeExpansion=m.dtype, **_props(m))
        if isinstance(m, Partial):
            return Partial(new_kids[0], rows=m._rowSelection,
                           cols=m._colSelection, **_props(m))
        if isinstance(m, Transpose):
            return Transpose(new_kids[0])
        if isinstance(m, Hermitian):
            return Hermitian(new_kids[0])
        return Conjugate(new_kids[0])

    return rec(m), mapping


# ---------------------------------------------------------------- kernels
def _fcontig(t):
    """2-D column-major (Fortran-order) view of a CUDA tensor."""
    if t.dim() == 1:
        t = t.unsqueeze(1)
    if t.stride(0) == 1 and (t.shape[1] <= 1 or t.stride(1) >= t.shape[0]):
        return t
    return t.t().contiguous().t()


def _ld(t):
    return max(t.stride(1), t.shape[0]) if t.shape[1] > 1 else t.shape[0]


def _reduce(u, v, pre, n, post, d=None, w=None):
    """out[j] = sum_{a, c, col} u * conj(v) over the (pre, n, post) view
    (fm_reduce_mulconj); with d, also w = conj(d) * u."""
    torch = _torch()
    u, v = _fcontig(u), _fcontig(v)
    if v.dtype != u.dtype:
        v = _fcontig(v.to(u.dtype))
    code = _native.DTYPE_CODE[_numpy_dtype(u.dtype)]
    out = torch.empty(n, dtype=u.dtype, device=u.device)
    stream = torch.cuda.current_stream(u.device).cuda_stream
    dp = wp = None
    ldw = 0
    if d is not None:
        d = d.to(u.dtype).contiguous()
        dp, wp, ldw = d.data_ptr(), w.data_ptr(), _ld(w)
    _native.reduce_mulconj(pre, n, post, u.shape[1], code, u.data_ptr(),
                           _ld(u), v.data_ptr(), _ld(v), out.data_ptr(), 1.0,
                           dp, wp, ldw, stream)
    return out


def _tuned(op, x):
    """Tile shapes of op's plan tuned for x's column count (once per
    operator and column count; the choice is cached in memory and on
    disk), as the plain operators are when their caller autotunes."""
    cols = 1 if x.dim() == 1 else x.shape[1]
    key = (cols, x.dtype)
    if getattr(op, '_grad_tuned', None) != key:
        op.autotune(cols, out_dtype=op._output_dtype(_numpy_dtype(x.dtype)))
        op._grad_tuned = key
    return op


def _fwd(op, x):
    return _tuned(op, x).forward(x)


def _bwd(op, x):
    return _tuned(op, x).backward(x)


def _smooth_at_least(n):
    """Smallest 2^a 3^b 5^c 7^d >= n (a fast length for the embedding)."""
    best = 1 << max(0, int(n - 1).bit_length())
    p7 = 1
    while p7 < best:
        p5 = p7
        while p5 < best:
            p3 = p5
            while p3 < best:
                v = p3
                while v < n:
                    v *= 2
                best = min(best, v)
                p3 *= 3
            p5 *= 5
        p7 *= 7
    return best


def _toeplitz_embedding(vecC, vecR, L):
    """Defining column of the L x L circulant whose leading
    len(vecC) x (len(vecR) + 1) block is Toeplitz(vecC, vecR)
    (T[i, j] = vecC[i - j] for i >= j, vecR[len(vecR) + i - j] else)."""
    nr, nc = len(vecC), len(vecR) + 1
    if L < nr + nc - 1:
        raise ValueError("embedding too short")
    emb = np.zeros(L, dtype=np.complex128)
    emb[:nr] = vecC
    emb[L - nc + 1:] = vecR
    return emb


def _mode(F, pre, post, prec):
    """F applied along one mode of a (pre, n, post) block."""
    terms = ([Eye(pre, precision=prec)] if pre > 1 else []) + [F] + (
        [Eye(post, precision=prec)] if post > 1 else [])
    return terms[0] if len(terms) == 1 else Kron(*terms, precision=prec)


class _Spectral:
    """A trainable Circulant or Toeplitz term written as
    R F^H diag(S / L) F Z (R keeps the first rows, Z zero-pads)."""

    def __init__(self, term, prec):
        self.term = term
        self.prec = prec
        if isinstance(term, Circulant):
            n = term.numRows
            self.L, self.nr, self.nc = n, n, n
            emb = term.tenC
        else:
            nr, nc = term.shape
            L = _smooth_at_least(nr + nc - 1)
            self.L, self.nr, self.nc = L, nr, nc
            emb = _toeplitz_embedding(term.vecC, term.vecR, L)
        self.F = Fourier(self.L, precision=prec)
        spec = Fourier(self.L).forward(emb)     # engine, native precision
        self.head = Diag(spec / self.L, precision=prec)
        L = self.L
        self.pre = []                           # input side first
        if self.nc < L:
            self.pre.append(Partial(Eye(L), cols=np.arange(self.nc),
                                    precision=prec))
        self.pre.append(self.F)
        self.post = [Hermitian(self.F)]
        if self.nr < L:
            self.post.append(Partial(Eye(L), rows=np.arange(self.nr),
                                     precision=prec))

    def grad(self, W):
        """Defining-vector gradient from W = sum conj(F Z a) * (F R^H g)."""
        g = _bwd(self.F, W) / self.L
        if isinstance(self.term, Circulant):
            return g
        torch = _torch()
        return torch.cat([g[:self.nr], g[self.L - self.nc + 1:]])


# ---------------------------------------------------------------- program
class _Seg:
    def __init__(self):
        self.terms = []      # input side first
        self.head = None     # (kind, payload) of the pivot opening it
        self.op = None       # forward plan (fastmat operator) or None
        self.bop = None      # adjoint plan for the backward pass or None


class _Program:
    """A differentiable operator tree cut into engine plans (see module
    docstring)."""

    def __init__(self, op, trainable):
        self.op = op
        self.prec = op._precision
        self.trainable = trainable           # id(leaf) -> parameter index
        self._dcache = {}
        scalar, chain = self._chain(op)
        segs = [_Seg()]
        for term in chain:
            kind = self._pivot_kind(term)
            if kind is None:
                segs[-1].terms.append(term)
            elif kind == 'diag':
                s = _Seg()
                s.head = ('diag', term)
                s.terms = [term]
                segs.append(s)
            elif kind == 'spec':
                sp = _Spectral(term, self.prec)
                segs[-1].terms.extend(sp.pre)
                s = _Seg()
                s.head = ('spec', sp)
                s.terms = [sp.head] + sp.post
                segs.append(s)
            else:
                s = _Seg()
                s.head = ('gen', term)
                s.terms = [term]
                segs.append(s)
        self.segs = segs
        self.scalar = scalar
        last = len(segs) - 1
        for i, s in enumerate(segs):
            sc = [scalar[()]] if (i == last and scalar != 1) else []
            if s.terms or sc:
                s.op = self._product(s.terms, sc, s)
            rest = s.terms[1:] if s.head is not None else list(s.terms)
            nxt = segs[i + 1].terms[0] if i < last else None
            bterms = rest + ([nxt] if nxt is not None else [])
            if bterms or sc:
                s.bop = self._product(bterms, sc, s)

    def _product(self, terms, sc, seg):
        if not terms:
            n = self.op.numRows
            terms = [Eye(n, precision=self.prec)]
        if len(terms) == 1 and not sc:
            t = terms[0]
            if t._precision == self.prec:
                return t
        return Product(*(list(reversed(terms)) + sc), precision=self.prec)

    def _has_trainable(self, m):
        return any(id(x) in self.trainable for x in _leaves(m))

    def _chain(self, m):
        """(scalar, terms input side first) of m, flattened where the
        flattening exposes trainable terms."""
        if not self._has_trainable(m):
            return np.array(1), [m]
        if isinstance(m, Product):
            s = np.array(m._scalar)
            terms = []
            for c in reversed(m._content):
                s2, t = self._chain(c)
                s = s * s2
                terms += t
            return s, terms
        if isinstance(m, Partial) and not isinstance(m, (Circulant,
                                                        Toeplitz)):
            inner = m._content[0]
            s, terms = self._chain(inner)
            out = []
            if m._colSelection is not None:
                out.append(Partial(Eye(inner.numCols), cols=m._colSelection,
                                   precision=self.prec))
            out += terms
            if m._rowSelection is not None:
                out.append(Partial(Eye(inner.numRows), rows=m._rowSelection,
                                   precision=self.prec))
            return s, out
        return np.array(1), [m]

    def _pivot_kind(self, term):
        if not self._has_trainable(term):
            return None
        if isinstance(term, Diag):
            return 'diag'
        if isinstance(term, (Circulant, Toeplitz)):
            return 'spec'
        return 'gen'

    # -------------------------------------------------------- forward
    def forward(self, x):
        """(y, saved inputs of every segment)."""
        acts = []
        a = x
        for s in self.segs:
            acts.append(a)
            if s.op is not None:
                a = _fwd(s.op, a)
        return a, acts

    # -------------------------------------------------------- backward
    def backward(self, gy, acts, need_x, grads):
        """Returns grad_x (or None); accumulates parameter gradients into
        `grads` (index -> tensor)."""
        t = gy
        segs = self.segs
        for i in range(len(segs) - 1, -1, -1):
            s = segs[i]
            if s.head is None:
                if not need_x:
                    return None
                return _bwd(s.bop, t) if s.bop is not None else t
            kind, payload = s.head
            fuse = (kind == 'diag' and i == 1 and segs[0].op is None and
                    need_x)
            G = _bwd(s.bop, t) if s.bop is not None else t
            a = acts[i]
            if kind == 'diag':
                leaf = payload
                n = leaf.numRows
                if fuse:
                    torch = _torch()
                    G = _fcontig(G)
                    w = torch.empty((G.shape[1], n), dtype=G.dtype,
                                    device=G.device).t()
                    d = self._diag_tensor(leaf, G)
                    gd = _reduce(G, a, 1, n, 1, d=d, w=w)
                    self._add(grads, leaf, gd)
                    return w
                self._add(grads, leaf, _reduce(G, a, 1, n, 1))
            elif kind == 'spec':
                W = _reduce(G, a, 1, payload.L, 1)
                self._add(grads, payload.term, payload.grad(W))
            else:
                self._vjp(payload, a, G, grads)
            t = G
        return None

    def _diag_tensor(self, leaf, like):
        d = self._dcache.get(id(leaf))
        if d is None or d.dtype != like.dtype or d.device != like.device:
            d = _torch().as_tensor(leaf.vecD).to(device=like.device,
                                                 dtype=like.dtype)
            self._dcache[id(leaf)] = d
        return d

    def _add(self, grads, leaf, g):
        k = self.trainable.get(id(leaf))
        if k is None:
            return
        grads[k] = g if grads.get(k) is None else grads[k] + g

    # generic pivots: Sum, Kron, dense, adjoint wrappers
    def _vjp(self, m, a, G, grads, pre=1, post=1):
        """Parameter gradients of the term m, with input a and upstream
        gradient G (the input gradient is handled by the segment plans)."""
        if not self._has_trainable(m):
            return
        torch = _torch()
        if isinstance(m, Transpose):
            return self._vjp(m._content[0], G.conj(), a.conj(), grads,
                             pre, post)
        if isinstance(m, Hermitian):
            return self._vjp(m._content[0], G, a, grads, pre, post)
        if isinstance(m, Conjugate):
            return self._vjp(m._content[0], a.conj(), G.conj(), grads,
                             pre, post)
        if isinstance(m, Sum):
            for c in m._content:
                self._vjp(c, a, G, grads, pre, post)
            return
        if isinstance(m, Kron):
            if pre != 1 or post != 1:
                raise NotImplementedError(
                    "nested Kron with trainable factors")
            dims = [f.numRows for f in m._content]
            for k, f in enumerate(m._content):
                if not self._has_trainable(f):
                    continue
                others = [Eye(d, precision=self.prec) if j == k else g
                          for j, (g, d) in enumerate(zip(m._content, dims))]
                ak = _fwd(Kron(*others, precision=self.prec), a)
                self._vjp(f, ak, G, grads, int(np.prod(dims[:k])),
                          int(np.prod(dims[k + 1:])))
            return
        if isinstance(m, Diag):
            self._add(grads, m, _reduce(G, a, pre, m.numRows, post))
            return
        if isinstance(m, Circulant):
            n = m.numRows
            Fm = _mode(Fourier(n, precision=self.prec), pre, post, self.prec)
            W = _reduce(_fwd(Fm, G), _fwd(Fm, a), pre, n, post)
            self._add(grads, m, _bwd(Fourier(n, precision=self.prec), W) / n)
            return
        if isinstance(m, Toeplitz):
            if pre != 1 or post != 1:
                raise NotImplementedError("Toeplitz Kron factor gradient")
            sp = _Spectral(m, self.prec)
            up = Product(*reversed(sp.pre), precision=self.prec)
            Gh = _bwd(sp.post[1], G) if len(sp.post) > 1 else G
            W = _reduce(_fwd(sp.F, Gh), _fwd(up, a), 1, sp.L, 1)
            self._add(grads, m, sp.grad(W))
            return
        if _is_dense(m):
            rows, cols = m.shape
            Gf, af = _fcontig(G), _fcontig(a)
            M = Gf.shape[1]
            Gm = Gf.t().reshape(M, pre, rows, post).permute(2, 0, 1, 3)
            Am = af.t().reshape(M, pre, cols, post).permute(2, 0, 1, 3)
            Gm = Gm.reshape(rows, -1)
            Am = Am.reshape(cols, -1).to(Gm.dtype)
            self._add(grads, m, torch.matmul(Gm, Am.conj().t()))
            return
        raise NotImplementedError(
            "gradient through %s is not supported" % type(m).__name__)


# ---------------------------------------------------------------- autograd
def _function():
    torch = _torch()

    class MatvecFunction(torch.autograd.Function):
        """y = A x with hand-written backward (adjoint matvec and
        parameter gradients on the engine)."""

        @staticmethod
        def forward(ctx, module, x, *params):
            prog = module._program()
            x2 = x if x.dim() == 2 else x.unsqueeze(1)
            y, acts = prog.forward(x2)
            want = _torch_dtype(prog.op._output_dtype(_numpy_dtype(x.dtype)))
            if y.dtype != want:
                y = y.to(want)
            ctx.prog = prog
            ctx.acts = acts
            ctx.flat = x.dim() == 1
            ctx.x_dtype = x.dtype
            ctx.param_dtypes = [p.dtype for p in params]
            return y.squeeze(1) if ctx.flat else y

        @staticmethod
        @torch.autograd.function.once_differentiable
        def backward(ctx, gy):
            prog = ctx.prog
            g2 = gy.unsqueeze(1) if ctx.flat else gy
            need_x = ctx.needs_input_grad[1]
            grads = {}
            gx = prog.backward(g2, ctx.acts, need_x, grads)
            out = [None, None]
            if need_x and gx is not None:
                if not ctx.x_dtype.is_complex and gx.is_complex():
                    gx = gx.real
                gx = gx.to(ctx.x_dtype)
                out[1] = gx.squeeze(1) if ctx.flat else gx
            for k, dt in enumerate(ctx.param_dtypes):
                g = grads.get(k)
                if g is not None and ctx.needs_input_grad[2 + k]:
                    if not dt.is_complex and g.is_complex():
                        g = g.real
                    g = g.to(dt)
                out.append(g)
            ctx.acts = None
            return tuple(out)

    return MatvecFunction


_FN = None


def _fn():
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN


def _module_base():
    return _torch().nn.Module


class Operator(_module_base()):
    """A fastmat operator as a differentiable torch module (see module
    docstring).  ``trainable``: True (all defining vectors), False (none:
    only the input is differentiated) or a collection of the leaf
    operators to train."""

    def __init__(self, op, trainable=True, device='cuda'):
        super().__init__()
        torch = _torch()
        if not isinstance(op, Matrix):
            raise TypeError("Operator: fastmat Matrix required")
        self._op = op
        leaves = _leaves(op)
        if trainable is True:
            chosen = leaves
        elif trainable is False or trainable is None:
            chosen = []
        else:
            sel = list(trainable)
            chosen = [m for m in leaves if any(m is s for s in sel)]
        self._leaf_ids = []
        names = {}
        for m in chosen:
            v = np.asarray(_leaf_value(m))
            dt = v.dtype if v.dtype.kind in 'fc' else np.dtype(np.float64)
            if op._precision == 'fp32' or m._precision == 'fp32':
                dt = T.single(dt)
            base = type(m).__name__.lower()
            k = names.get(base, 0)
            names[base] = k + 1
            p = torch.nn.Parameter(
                torch.as_tensor(np.array(v, dtype=dt)).to(device))
            self.register_parameter('%s%d' % (base, k), p)
            self._leaf_ids.append(id(m))
        self._built_key = None
        self._prog = None
        self._values_key = self._key()

    @property
    def op(self):
        """The wrapped operator with the current parameter values."""
        return self._program().op

    def _key(self):
        return tuple((p.data_ptr(), p._version) for p in self.parameters())

    def _program(self):
        key = self._key()
        if self._prog is not None and key == self._built_key:
            return self._prog
        params = list(self.parameters())
        if self._prog is None and key == self._values_key:
            op, mapping = self._op, {i: i for i in self._leaf_ids}
        else:
            vals = {i: p.detach().cpu().numpy()
                    for i, p in zip(self._leaf_ids, params)}
            op, mapping = _rebuild(self._op, vals)
        index = {old: k for k, old in enumerate(self._leaf_ids)}
        trainable = {new: index[old] for new, old in mapping.items()
                     if old in index}
        self._prog = _Program(op, trainable)
        self._built_key = key
        return self._prog

    def forward(self, x):
        return _fn().apply(self, x, *self.parameters())


def matvec(op, x):
    """y = op x for a CUDA tensor x, differentiable with respect to x
    (backward = the engine's adjoint matvec)."""
    mod = getattr(op, '_autograd_module', None)
    if mod is None:
        mod = Operator(op, trainable=False)
        op._autograd_module = mod
    return mod(x)
