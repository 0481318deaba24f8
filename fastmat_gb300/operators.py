"""The structured operator classes, with fastmat's constructors.

Each class keeps fastmat's constructor signature, dtype rule and the
attributes callers read, and describes itself to the native engine as one
node of an operator tree (``_emit``).  ``_reference`` builds the dense
matrix directly from the defining data, as fastmat's ``.reference()`` does.
"""

import numpy as np

from . import _native
from . import fftsize
from . import types as T
from .matrix import Hermitian, Matrix


def _squeezed_copy(a):
    a = np.array(a)
    return np.squeeze(a).copy() if a.ndim > 1 else a.copy()


def _level_diff_matrix(ten, rows, cols):
    """Dense multi-level difference matrix M[i, j] = ten[((i_k - j_k) mod
    ten.shape[k])_k], with i = (i_1, ..., i_d) < rows and j < cols
    enumerated in C order (the block structure of a multi-level circulant,
    fastmat/Circulant.pyx:344-425, and of the Toeplitz matrices embedded in
    one, fastmat/Toeplitz.pyx:628-734)."""
    ri = np.unravel_index(np.arange(int(np.prod(rows))), rows)
    ci = np.unravel_index(np.arange(int(np.prod(cols))), cols)
    idx = tuple((r[:, None] - c[None, :]) % n
                for r, c, n in zip(ri, ci, ten.shape))
    return ten[idx]


class Fourier(Matrix):
    """Unnormalised DFT matrix F[n, k] = exp(-2 pi i n k / N)
    (fastmat/Fourier.pyx:26-285).  ``_numL`` is fastmat's Bluestein length
    decision (0 = direct); the GPU picks its own algorithm for every order.
    """

    def __init__(self, order, **options):
        if order < 1:
            raise ValueError("Fourier order cannot be smaller than 1.")
        self._order = int(order)
        self._numL = fftsize.bluestein_length(
            self._order, options.get('optimize', True),
            options.get('maxStage', 4))
        self._init_properties(self._order, self._order, np.complex128,
                              **options)

    @property
    def order(self):
        return self._order

    def _emit(self, b):
        return b.add(_native.NODE_FOURIER, self, n=self._order)

    def _reference(self):
        k = np.arange(self._order, dtype=np.int64)
        ph = np.outer(k, k) % self._order
        return np.exp(ph * (-2j * np.pi / self._order)).astype(self.dtype)


class Diag(Matrix):
    """Diagonal matrix (fastmat/Diag.pyx:29-174)."""

    def __init__(self, vecD, **options):
        self._vecD = _squeezed_copy(vecD)
        if np.ndim(vecD) != 1 or self._vecD.ndim != 1:
            raise ValueError(
                "Diag: Definition vector must have exactly one dimension.")
        self._vecD = self._vecD.astype(T.supported(self._vecD.dtype),
                                       copy=False)
        n = self._vecD.size
        self._init_properties(n, n, self._vecD.dtype.type, **options)

    @property
    def vecD(self):
        return self._vecD

    def _emit(self, b):
        return b.add(_native.NODE_DIAG, self, vec0=self._vecD)

    def _reference(self):
        return np.diag(self._vecD)

    # closed forms (fastmat/Diag.pyx:126-139)
    def _getColNorms(self):
        return np.abs(self._vecD)

    _getRowNorms = _getColNorms

    def _getColNormalized(self):
        if np.iscomplexobj(self._vecD):
            return Diag((self._vecD / np.abs(self._vecD)).astype(self.dtype))
        return Diag(np.sign(self._vecD).astype(self.dtype))

    _getRowNormalized = _getColNormalized


class Eye(Matrix):
    """Identity (fastmat/Eye.pyx)."""

    def __init__(self, order, **options):
        self._init_properties(order, order, np.int8, **options)

    def _emit(self, b):
        return b.add(_native.NODE_EYE, self)

    def _reference(self):
        return np.eye(self.numRows, dtype=self.dtype)

    # closed forms (fastmat/Eye.pyx:92-102)
    def _getColNorms(self):
        return np.ones((self.numCols, ), dtype=self.dtype)

    _getRowNorms = _getColNorms

    def _getColNormalized(self):
        return self

    _getRowNormalized = _getColNormalized


class Hadamard(Matrix):
    """Sylvester-ordered Hadamard matrix of size 2^order, int8
    (fastmat/Hadamard.pyx:63-248)."""

    def __init__(self, order, **options):
        if order < 1:
            raise ValueError("Hadamard: Order must be larger than 0.")
        max_order = 62
        if order > max_order:
            raise ValueError(
                "Hadamard: Order exceeds maximum for this platform: %d" %
                max_order)
        self._order = int(order)
        n = 2 ** self._order
        self._init_properties(n, n, np.int8, **options)

    @property
    def order(self):
        return self._order

    def _emit(self, b):
        return b.add(_native.NODE_HADAMARD, self, n=self._order)

    def _reference(self):
        h = np.ones((1, 1), dtype=np.int8)
        for _ in range(self._order):
            h = np.block([[h, h], [h, -h]])
        return h


class Permutation(Matrix):
    """Permutation matrix, forward x[sigma] (fastmat/Permutation.pyx)."""

    def __init__(self, sigma, **options):
        sigma = np.array(sigma)
        self._sigma = _squeezed_copy(sigma)
        if sigma.ndim != 1 or self._sigma.ndim != 1:
            raise ValueError(
                "Diag: Definition vector must have exactly one dimension.")
        n = sigma.shape[0]
        if not np.array_equal(np.sort(sigma), np.arange(n)):
            raise ValueError("Not a permutation.")
        self._tau = np.argsort(sigma)
        self._init_properties(n, n, np.int8, **options)

    @property
    def sigma(self):
        return self._sigma

    @property
    def tau(self):
        return self._tau

    def _emit(self, b):
        return b.add(_native.NODE_PERMUTATION, self, vec0=self._sigma,
                     int0=True)

    def _reference(self):
        return np.eye(self.numRows, dtype=self.dtype)[self._sigma, :]

    # closed forms (fastmat/Permutation.pyx:104-114)
    def _getColNorms(self):
        return np.ones((self.numCols, ), dtype=self.dtype)

    _getRowNorms = _getColNorms

    def _getColNormalized(self):
        return self

    _getRowNormalized = _getColNormalized


class Partial(Matrix):
    """Row/column sub-selection of a matrix (fastmat/Partial.pyx:25-303)."""

    def __init__(self, mat, **options):
        if not isinstance(mat, Matrix):
            raise TypeError("Partial: fastmat Matrix required.")
        self._content = (mat,)
        if 'N' in options:
            options['rows'] = options['N']
        if 'M' in options:
            options['cols'] = options['M']

        def check(sel, size, name):
            if sel is None:
                return None
            sel = np.array(sel)
            if sel.dtype == bool:
                sel = np.arange(size)[sel]
            elif sel.dtype.kind not in 'iu':
                raise TypeError(
                    "Partial: Type of %s indices must be int or bool." % name)
            if np.any((sel >= size) | (sel < 0)):
                raise ValueError(
                    "Partial: A %s index exceeds matrix dimensions." % name)
            return sel

        self._rowSelection = check(options.pop('rows', None), mat.numRows,
                                   'row')
        self._colSelection = check(options.pop('cols', None), mat.numCols,
                                   'col')
        options.pop('N', None)
        options.pop('M', None)
        self._init_properties(
            mat.numRows if self._rowSelection is None
            else len(self._rowSelection),
            mat.numCols if self._colSelection is None
            else len(self._colSelection),
            mat.dtype, **options)

    @property
    def rowSelection(self):
        return (self._rowSelection if self._rowSelection is not None
                else np.arange(self.numRows))

    @property
    def colSelection(self):
        return (self._colSelection if self._colSelection is not None
                else np.arange(self.numCols))

    def _emit(self, b):
        return b.add(_native.NODE_PARTIAL, self, children=self._content,
                     vec0=self._rowSelection, vec1=self._colSelection,
                     int0=True, int1=True)

    def _reference(self):
        a = self._content[0].reference()
        if self._rowSelection is not None:
            a = a[self._rowSelection, :]
        if self._colSelection is not None:
            a = a[:, self._colSelection]
        return a


class Product(Matrix):
    """Matrix product with an optional scalar (fastmat/Product.pyx)."""

    def __init__(self, *matrices, **options):
        factors = []
        scalar = np.int8(1)
        dtype = [np.int8]

        def add(items):
            nonlocal scalar
            for f in items:
                if np.isscalar(f):
                    dtype[0] = T.promote(dtype[0], np.array(f).dtype)
                    scalar = np.inner(scalar, f)
                    continue
                if not isinstance(f, Matrix):
                    raise TypeError("Product: Term not scalar nor Matrix.")
                if isinstance(f, Product):
                    if f._scalar != 1:
                        scalar = scalar * f._scalar
                    add(f.content)
                else:
                    factors.append(f)
                dtype[0] = T.promote(dtype[0], f.dtype)

        add(matrices)
        dt = dtype[0]
        expansion = options.pop('typeExpansion', T.safe_type_expansion(dt))
        if expansion is not None:
            dt = T.promote(dt, expansion)
        if not factors:
            raise ValueError("Product has no terms.")
        for i in range(1, len(factors)):
            if factors[i].numRows != factors[i - 1].numCols:
                raise ValueError(
                    "Product: Dimension mismatch for term %d [%dx%d]" % (
                        i, factors[0].numRows, factors[i - 1].numCols))
        self._scalar = np.array(scalar).astype(dt)
        self._content = tuple(factors)
        self._init_properties(factors[0].numRows, factors[-1].numCols, dt,
                              **options)

    def _emit(self, b):
        return b.add(_native.NODE_PRODUCT, self, children=self._content,
                     scalar=complex(self._scalar))

    def _reference(self):
        dt = T.promote(np.float64, self.dtype)
        a = np.inner(self._content[-1].reference(), self._scalar.astype(dt))
        for term in reversed(self._content[:-1]):
            a = term.reference().dot(a)
        return a


class Sum(Matrix):
    """Sum of matrices (fastmat/Sum.pyx)."""

    def __init__(self, *matrices, **options):
        terms = []

        def add(items):
            for m in items:
                if not isinstance(m, Matrix):
                    raise TypeError("Sum: Term is not a fastmat Matrix.")
                if isinstance(m, Sum):
                    add(m.content)
                else:
                    terms.append(m)

        add(matrices)
        if not terms:
            raise ValueError("Sum: No terms given.")
        for m in terms[1:]:
            if m.shape != terms[0].shape:
                raise ValueError("Sum: Term dimension mismatch: " + repr(m))
        dt = np.int8
        for m in terms:
            dt = T.promote(dt, m.dtype)
        self._content = tuple(terms)
        options.setdefault('widenInputDatatype', True)
        self._init_properties(terms[0].numRows, terms[0].numCols, dt,
                              **options)

    def _emit(self, b):
        return b.add(_native.NODE_SUM, self, children=self._content)

    def _reference(self):
        a = np.zeros(self.shape, dtype=self.dtype)
        for m in self._content:
            a = a + m.reference()
        return a


class Kron(Matrix):
    """Kronecker product, factor 0 most significant (fastmat/Kron.pyx)."""

    def __init__(self, *matrices, **options):
        if len(matrices) < 2:
            raise ValueError("Kronecker: Product must have at least two terms")
        dt = np.int8
        n = 1
        for m in matrices:
            if m.numRows != m.numCols:
                raise ValueError("Kronecker: Product terms must be symmetric")
            n *= m.numRows
            dt = T.promote(dt, m.dtype)
        expansion = options.pop('typeExpansion', T.safe_type_expansion(dt))
        if expansion is not None:
            dt = T.promote(dt, expansion)
        self._content = tuple(matrices)
        self._dims = tuple(m.numRows for m in matrices)
        options.setdefault('widenInputDatatype', True)
        self._init_properties(n, n, dt, **options)

    def _emit(self, b):
        return b.add(_native.NODE_KRON, self, children=self._content)

    def _reference(self):
        a = self._content[0].reference().astype(
            T.promote(self.dtype, np.float64))
        for m in self._content[1:]:
            a = np.kron(a, m.reference())
        return a


class Circulant(Partial):
    """Circulant matrix C[i, j] = c[(i - j) mod n]
    (fastmat/Circulant.pyx:32-227); a d-dimensional tenC defines a d-level
    circulant.  The GPU convolves with the FFT of the
    defining vector; ``content`` builds fastmat's Fourier-domain structure
    (Partial of Product(F.H, Diag(fft(c)/L), F)) on demand."""

    def __init__(self, tenC, **options):
        c = _squeezed_copy(tenC)
        if np.ndim(tenC) < 1 or c.ndim < 1:
            raise ValueError("Column-definition tensor must be at least 1D.")
        self._optimize = options.get('optimize', True)
        self._maxStage = options.get('maxStage', 4)
        self._tenC = c.astype(np.complex128)
        self._rowSelection = None
        self._colSelection = None
        self._structure = None
        self._ml = None
        opts = {k: v for k, v in options.items()
                if k not in ('optimize', 'maxStage', 'rows', 'cols')}
        self._init_properties(c.size, c.size, np.complex128, **opts)

    @property
    def tenC(self):
        return self._tenC

    @property
    def vecC(self):
        return self._tenC

    def _multilevel(self):
        """Multi-level circulant (fastmat/Circulant.pyx:138-215) as
        Kron(F_n1, ..., F_nd)^H diag(fftn(tenC) / N) Kron(F_n1, ..., F_nd):
        block (i, j) of level k uses tenC[.., (i - j) mod n_k, ..].  The
        spectrum is computed on the GPU by the same Kron of Fouriers."""
        if self._ml is None:
            dims = self._tenC.shape
            prec = self._precision
            KF = Kron(*[Fourier(int(n)) for n in dims])
            spec = KF.forward(self._tenC.reshape(-1)) / self._tenC.size
            KFp = Kron(*[Fourier(int(n)) for n in dims], precision=prec)
            self._ml = Product(Hermitian(KFp), Diag(spec, precision=prec),
                               KFp, precision=prec)
        return self._ml

    @property
    def content(self):
        if self._tenC.ndim > 1:
            return (self._multilevel(),)
        if self._structure is None:
            n = self._tenC.size
            L = fftsize.circulant_length(n, self._optimize, self._maxStage)
            c = self._tenC
            if L != n:
                c = np.concatenate([c, np.zeros(L - 2 * n + 1, c.dtype),
                                    c[1:]])
            F = Fourier(L, optimize=self._optimize, maxStage=self._maxStage)
            spec = F.forward(c) / L
            self._structure = (Product(Hermitian(F), Diag(spec), F),)
        return self._structure

    @property
    def rowSelection(self):
        return np.arange(self.numRows)

    @property
    def colSelection(self):
        return np.arange(self.numCols)

    def _emit(self, b):
        if self._tenC.ndim > 1:
            return self._multilevel()._emit(b)
        return b.add(_native.NODE_CIRCULANT, self, vec0=self._tenC)

    def _reference(self):
        return _level_diff_matrix(self._tenC, self._tenC.shape,
                                  self._tenC.shape).astype(self.dtype)


class Toeplitz(Partial):
    """Toeplitz matrix (fastmat/Toeplitz.pyx:31-734), one or more levels.

    ``Toeplitz(vecC, vecR)``: first column vecC and first row
    [vecC[0], vecR[-1], vecR[-2], ...] (T[0, j] = vecR[-j]);
    ``Toeplitz(tenT, split=n_rows)`` with tenT = [vecC, vecR]."""

    def __init__(self, *args, **options):
        split = options.pop('split', None)
        if len(args) == 2:
            if not all(isinstance(a, np.ndarray) for a in args):
                raise ValueError(
                    "You must specify two 1D-ndarrays containing the " +
                    "column- and row-definition vectors or one ndarray tensor")
            if split is not None:
                raise ValueError(
                    "You must not define split points when supplying " +
                    "column- and row-definition vectors.")
            dt = np.promote_types(args[0].dtype, args[1].dtype)
            vc = np.atleast_1d(np.squeeze(args[0].astype(dt)))
            vr = np.atleast_1d(np.squeeze(args[1].astype(dt)))
            if vc.ndim != 1 or vr.ndim > 1:
                raise ValueError(
                    "Column- and row-definition vectors must be 1D.")
            vr = vr.reshape(-1)
            tenT = np.hstack((vc, vr))
            split = vc.size
        elif len(args) == 1 and np.ndim(args[0]) > 1:
            self._init_multilevel(np.asarray(args[0]), split, options)
            return
        elif len(args) == 1:
            tenT = np.asarray(args[0])
            if split is None:
                if (tenT.size + 1) % 2 != 0:
                    raise ValueError(
                        "Defining a tensor with non-square levels requires " +
                        "explicit split points.")
                split = (tenT.size + 1) // 2
            split = int(np.atleast_1d(split)[0])
            if split < 1 or split > tenT.size:
                raise ValueError(
                    "Entry in split vector outside of defining tensor bounds")
        else:
            raise ValueError(
                "Invalid number of arguments to Toeplitz: Expecting exactly " +
                "one or two fixed arguments")
        self._tenT = tenT.astype(np.complex128)
        self._split = split
        self._ml = None
        nr = split
        nc = tenT.size - nr + 1
        self._optimize = options.get('optimize', True)
        self._maxStage = options.get('maxStage', 4)
        self._rowSelection = None
        self._colSelection = None
        opts = {k: v for k, v in options.items()
                if k not in ('optimize', 'maxStage', 'rows', 'cols')}
        self._init_properties(nr, nc, np.complex128, **opts)

    def _init_multilevel(self, tenT, split, options):
        """Multi-level Toeplitz (fastmat/Toeplitz.pyx:180-322): level k has
        split[k] rows and tenT.shape[k] - split[k] + 1 columns, and
        T[i, j] = tenT[((i_k - j_k) mod tenT.shape[k])_k] -- the rows with
        i_k < split[k] and columns with j_k < cols[k] of the multi-level
        circulant of tenT, which is how it is applied."""
        dims = np.array(tenT.shape)
        sp = np.atleast_1d(np.array([] if split is None else split))
        if sp.size == 0:
            if not all((d + 1) % 2 == 0 for d in dims):
                raise ValueError(
                    "Defining a tensor with non-square levels requires " +
                    "explicit split points.")
            sp = (dims + 1) // 2
        if sp.ndim != 1:
            raise ValueError("The split point vector must be 1D")
        if sp.size != tenT.ndim:
            raise ValueError(
                "The split point vector must have one entry for each " +
                "dimension of the defining tensor")
        if any(v < 1 or v > dims[i] for i, v in enumerate(sp)):
            raise ValueError(
                "Entry in split vector outside of defining tensor bounds")
        self._tenT = tenT.astype(np.complex128)
        self._split = sp.astype(np.int64)
        self._rows_lv = tuple(int(v) for v in sp)
        self._cols_lv = tuple(int(d - v + 1) for d, v in zip(dims, sp))
        self._optimize = options.get('optimize', True)
        self._maxStage = options.get('maxStage', 4)
        self._rowSelection = None
        self._colSelection = None
        self._ml = None
        opts = {k: v for k, v in options.items()
                if k not in ('optimize', 'maxStage', 'rows', 'cols')}
        self._init_properties(int(np.prod(self._rows_lv)),
                              int(np.prod(self._cols_lv)), np.complex128,
                              **opts)

    def _multilevel(self):
        if self._ml is None:
            dims = self._tenT.shape

            def sel(lv):
                idx = np.unravel_index(np.arange(int(np.prod(dims))), dims)
                keep = np.ones(int(np.prod(dims)), dtype=bool)
                for k, n in enumerate(lv):
                    keep &= idx[k] < n
                return np.arange(int(np.prod(dims)))[keep]

            C = Circulant(self._tenT, precision=self._precision)
            self._ml = Partial(C, rows=sel(self._rows_lv),
                               cols=sel(self._cols_lv),
                               precision=self._precision)
        return self._ml

    @property
    def tenT(self):
        return self._tenT

    @property
    def vecC(self):
        return self._tenT[:self._split]

    @property
    def vecR(self):
        return self._tenT[self._split:]

    @property
    def content(self):
        if self._tenT.ndim > 1:
            return (self._multilevel(),)
        raise NotImplementedError(
            "Toeplitz content structure is not materialised by "
            "fastmat_gb300")

    @property
    def rowSelection(self):
        return np.arange(self.numRows)

    @property
    def colSelection(self):
        return np.arange(self.numCols)

    def _emit(self, b):
        if self._tenT.ndim > 1:
            return self._multilevel()._emit(b)
        return b.add(_native.NODE_TOEPLITZ, self, vec0=self.vecC,
                     vec1=self.vecR)

    def _reference(self):
        if self._tenT.ndim > 1:
            return _level_diff_matrix(self._tenT, self._rows_lv,
                                      self._cols_lv).astype(self.dtype)
        nr, nc = self.shape
        d = np.arange(nr)[:, None] - np.arange(nc)[None, :]
        full = np.concatenate([self.vecR, self.vecC])
        return full[d + nc - 1].astype(self.dtype)


class Blocks(Matrix):
    """A grid of operators (fastmat/Blocks.pyx:27-312): the inner iterables
    are block rows; blocks of a row share their height, blocks of a column
    their width.  One GPU plan: output block row r is the sum over c of
    block (r, c) applied to input segment c (the first block writes, later
    ones accumulate); the adjoint runs the transposed grid of adjoints."""

    def __init__(self, arrMatrices, **options):
        if not isinstance(arrMatrices, (list, tuple)):
            raise ValueError("Blocks: Not a nested list of fastmat matrices.")
        if len(arrMatrices) < 1:
            raise ValueError("Blocks: Contains no matrices.")
        for rr, row in enumerate(arrMatrices):
            if isinstance(row, Matrix):
                raise TypeError(
                    "Blocks.row(%d) is of type %s. Instantiate Blocks with a "
                    "2D structure of iterables (e.g. nested lists) holding "
                    "fastmat Matrix instances in their second level." % (
                        rr, repr(row)))
            for cc, item in enumerate(row):
                if not isinstance(item, Matrix):
                    raise TypeError(
                        "Blocks[%d, %d] is of type %s and not a fastmat "
                        "Matrix isntance." % (rr, cc, repr(item)))
        self._rows = tuple(tuple(r) for r in arrMatrices)
        first = self._rows[0]
        self._rowSize = tuple(r[0].numRows for r in self._rows)
        self._colSize = tuple(t.numCols for t in first)
        dtype = np.int8
        for rr, row in enumerate(self._rows):
            if len(row) != len(first):
                raise ValueError(
                    "Blocks.row(%d) has incompatible number of entries" % rr)
            for cc, term in enumerate(row):
                if term.numRows != row[0].numRows:
                    raise ValueError(
                        "Blocks[%d,%d] with shape %s is incompatible with row "
                        "height (%d,:)" % (rr, cc, str(term.shape),
                                           row[0].numRows))
                if term.numCols != first[cc].numCols:
                    raise ValueError(
                        "Blocks[%d,%d] with shape %s is incompatible with "
                        "column width (:,%d)" % (rr, cc, str(term.shape),
                                                 first[cc].numCols))
                dtype = np.promote_types(dtype, term.dtype)
        self._cols = tuple(tuple(r[cc] for r in self._rows)
                           for cc in range(len(first)))
        self._content = tuple(t for r in self._rows for t in r)
        self._init_properties(sum(self._rowSize), sum(self._colSize),
                              dtype, **options)
        self._widenInputDatatype = True

    def _emit(self, b):
        return b.add(_native.NODE_BLOCKS, self, children=self._content,
                     n=len(self._rows))

    def _reference(self):
        return np.block([[t.reference() for t in r] for r in self._rows]
                        ).astype(self.dtype)


class BlockDiag(Matrix):
    """Operators along the block diagonal (fastmat/BlockDiag.pyx:27-200),
    planned as a Blocks grid whose off-diagonal blocks are zero: every
    block reads and writes its own row segment, one GPU plan."""

    def __init__(self, *matrices, **options):
        if len(matrices) < 1:
            raise ValueError("You must specify at least one matrix.")
        dtype = np.int8
        for term in matrices:
            if not isinstance(term, Matrix):
                raise ValueError(
                    "Only fastmat matrices supported, %s given." % str(term))
            dtype = np.promote_types(dtype, term.dtype)
        self._content = tuple(matrices)
        self._init_properties(sum(t.numRows for t in matrices),
                              sum(t.numCols for t in matrices), dtype,
                              **options)
        self._widenInputDatatype = True

    def _emit(self, b):
        k = len(self._content)
        grid = [self._content[i] if i == j else None
                for i in range(k) for j in range(k)]
        return b.add(_native.NODE_BLOCKS, self, children=grid, n=k)

    def _reference(self):
        out = np.zeros(self.shape, dtype=self.dtype)
        r = c = 0
        for t in self._content:
            out[r:r + t.numRows, c:c + t.numCols] = t.reference()
            r += t.numRows
            c += t.numCols
        return out


class Sparse(Matrix):
    """A scipy.sparse matrix as an operator (fastmat/Sparse.pyx:25-185),
    applied on the GPU as a CSR product; the adjoint is the conjugate
    transpose, stored as a second CSR when the plan is built."""

    def __init__(self, matSparse, **options):
        import scipy.sparse as sps
        if not sps.issparse(matSparse):
            raise TypeError("Sparse: Use Matrix() for numpy ndarrays."
                            if isinstance(matSparse, np.ndarray)
                            else "Sparse: Matrix is not a scipy spmatrix")
        self._spArray = matSparse.tocsr()
        self._spArrayH = None
        self._init_properties(self._spArray.shape[0],
                              self._spArray.shape[1],
                              T.supported(self._spArray.dtype), **options)

    @property
    def spArray(self):
        return self._spArray

    @property
    def spArrayH(self):
        if self._spArrayH is None:
            self._spArrayH = self._spArray.T.conj().tocsr()
        return self._spArrayH

    def _emit(self, b):
        a = self._spArray
        data = np.asarray(a.data).astype(self.dtype, copy=False)
        idx = np.concatenate([np.asarray(a.indptr, dtype=np.int64),
                              np.asarray(a.indices, dtype=np.int64)])
        return b.add(_native.NODE_SPARSE, self, n=int(a.nnz),
                     vec0=data if data.size else None, vec1=idx, int1=True)

    def _reference(self):
        return self._spArray.toarray().astype(self.dtype, copy=False)
