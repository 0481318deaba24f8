"""CPU oracle for the fastmat structured-operator matvec path.

TEST INFRASTRUCTURE ONLY.  This module restates, in plain numpy, the
algorithms the reference fastmat package runs on its CPU path for the
operators this project accelerates.  It is imported by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py`` --
always as the checker, never as the thing measured or shipped.  The product
package ``fastmat_gb300`` never imports it.

Parity of this restatement is pinned against fixtures produced by the real
reference (``tests/golden/make_golden.py`` writes ``tests/golden/*.npz``) and
checked by ``tests/test_oracle_golden.py``.

Every function cites the reference file:line (paths relative to the fastmat
project root) whose behaviour it follows.
"""

import math

import numpy as np

# ----------------------------------------------------------------------------
# type handling  (fastmat/core/types.pxd:45-55, fastmat/core/types.pyx:423-453)
# ----------------------------------------------------------------------------

#: fastmat's eight supported element types, in ftype order
#: (fastmat/core/types.pxd:45-55)
FTYPES = (np.int8, np.int16, np.int32, np.int64,
          np.float32, np.float64, np.complex64, np.complex128)


def supported_dtype(dtype):
    """Map a numpy dtype onto the fastmat type it is handled as.

    fastmat classifies every numpy type by kind and size
    (fastmat/core/types.pyx:423-426, approximateType); the supported types
    map to themselves and booleans/unsigned types map to the signed integer
    type of the next size that can hold them.
    """
    dt = np.dtype(dtype)
    if dt.type in FTYPES:
        return dt.type
    if dt.kind == 'b':
        return np.int8
    if dt.kind == 'u':
        return {1: np.int16, 2: np.int32, 4: np.int64}.get(dt.itemsize,
                                                             np.int64)
    raise TypeError("unsupported dtype %s" % dt)


def promote(a, b):
    """Binary type promotion (fastmat/core/types.pyx:443-453)."""
    return supported_dtype(np.promote_types(supported_dtype(a),
                                            supported_dtype(b)))


def safe_type_expansion(dtype):
    """fastmat/core/types.pyx:378-394: widen small ints to float."""
    dt = np.dtype(dtype).type
    if dt in (np.int8, np.int16):
        return np.float32
    if dt in (np.int32, np.int64):
        return np.float64
    return dt


# ----------------------------------------------------------------------------
# FFT size heuristics  (fastmat/core/cmath.pyx:35-214)
# ----------------------------------------------------------------------------

def _factor_search(target, max_factor, state, best):
    """Greedy recursion of fastmat/core/cmath.pyx:35-82 (_findFFTFactors).

    ``state``/``best`` pack (complexity << 16) + length into one integer so
    that comparing the packed values compares complexity first.
    """
    for ff in range(max_factor, 0, -1):
        length = (state & 0xFFFF) * ff
        complexity = (state >> 16) + ff + 1
        new_state = (complexity << 16) + length
        if new_state <= best and length < target:
            best = _factor_search(target, ff, new_state, best)
        elif new_state < best:
            best = new_state
    return best


def optimal_fft_size(order, max_stage=4):
    """fastmat/core/cmath.pyx:85-153 (_findOptimalFFTSize).

    The remaining size is tracked in single precision exactly as the
    reference does (a C ``float``), then the last factor is searched.
    """
    padded = 1
    remaining = np.float32(order)
    four = np.float32(4)
    while remaining > 64:
        padded *= 4
        remaining = np.float32(remaining / four)
    x = int(math.ceil(float(remaining)))
    if x != 1:
        best = (3 * (4 + 1) << 16) + 64
        padded *= _factor_search(x, max_stage, 1, best) & 0xFFFF
    return padded


def fft_complexity(n):
    """fastmat/core/cmath.pyx:156-209 (_getFFTComplexity), as float32."""
    nn = int(n)
    complexity = 0
    while nn % 4 == 0 and nn > 0:
        complexity += 5
        nn //= 4
    if nn > 1 and nn % 2 == 0:
        complexity += 3
        nn //= 2
    ii = 3
    # the reference stops at ii * ii < nn (strict), so a remaining square of
    # a prime is counted as one factor of size nn
    while nn > 1 and ii * ii < nn:
        if nn % ii == 0:
            complexity += ii + 1
            nn //= ii
        else:
            ii += 2
    if nn > 1:
        complexity += nn + 1
    return float(np.float32(n) * np.float32(complexity + 1))


def fourier_bluestein_length(order, optimize=True, max_stage=4):
    """The ``_numL`` decision of fastmat/Fourier.pyx:109-122.

    Returns 0 for a direct FFT, else the padded convolution length L.
    """
    if not optimize:
        return 0
    padded = optimal_fft_size(order * 2 - 1, max_stage)
    direct = fft_complexity(order)
    conv = 2 * fft_complexity(padded) + 2 * padded + 2 * order
    return 0 if direct < conv else padded


def circulant_length(n, optimize=True, max_stage=4):
    """Embedding length of a 1-level circulant (fastmat/Circulant.pyx:107-124).
    """
    if not optimize:
        return n
    padded = optimal_fft_size(2 * n - 1, max_stage)
    return padded if fft_complexity(n) > fft_complexity(padded) else n


def toeplitz_length(dd, optimize=True, max_stage=4):
    """Embedding length of a 1-level Toeplitz (fastmat/Toeplitz.pyx:225-237).
    ``dd`` is the defining vector length (rows + cols - 1)."""
    if not optimize:
        return dd
    opt = optimal_fft_size(dd, max_stage)
    return opt if fft_complexity(opt) < fft_complexity(dd) else dd


# ----------------------------------------------------------------------------
# operator model
# ----------------------------------------------------------------------------

def _as2d(x):
    x = np.asarray(x)
    if x.ndim == 1:
        return x.reshape(-1, 1), True
    return x, False


class Op:
    """Base of the oracle operators: dense shape, dtype, forward/backward.

    Mirrors the dispatch of fastmat/Matrix.pyx:1844-2007: inputs are 1-D or
    2-D, are promoted to the operator's type and return 1-D for 1-D input.
    """
    dtype = np.float64
    min_type = np.int8
    widen_input = False

    def out_dtype(self, x_dtype):
        """fastmat/Matrix.pyx:1799-1808: internal = promote(in, minType),
        output = promote(internal, self.dtype)."""
        internal = promote(x_dtype, self.min_type)
        return promote(internal, self.dtype)

    def forward(self, x):
        x2, flat = _as2d(x)
        if x2.shape[0] != self.shape[1]:
            raise ValueError("size mismatch")
        y = self._fwd(x2).astype(self.out_dtype(x2.dtype), copy=False)
        return y.reshape(-1) if flat else y

    def backward(self, x):
        x2, flat = _as2d(x)
        if x2.shape[0] != self.shape[0]:
            raise ValueError("size mismatch")
        y = self._bwd(x2).astype(self.out_dtype(x2.dtype), copy=False)
        return y.reshape(-1) if flat else y

    @property
    def H(self):
        return Hermitian(self)


class Fourier(Op):
    """fastmat/Fourier.pyx: unnormalised DFT, direct or Bluestein."""

    def __init__(self, order, optimize=True, max_stage=4):
        self.order = order
        self.shape = (order, order)
        self.dtype = np.complex128
        self.numL = fourier_bluestein_length(order, optimize, max_stage)
        if self.numL:
            # chirp exactly as fastmat/Fourier.pyx:127-156 forms it:
            # phase n^2 * pi / N evaluated in float64
            n = np.linspace(0, order - 1, order)
            arg = (n ** 2) * np.pi / order
            conv = np.zeros(self.numL, np.complex128)
            conv[:order] = np.cos(arg) + 1j * np.sin(arg)
            conv[self.numL - order + 1:] = conv[1:order][::-1]
            self.pre = np.cos(arg) - 1j * np.sin(arg)
            self.conv_hat = np.fft.fft(conv)

    def _fwd(self, x):
        x = x.astype(np.complex128)
        if not self.numL:
            return np.fft.fft(x, axis=0)
        # fastmat/Fourier.pyx:215-231
        buf = np.zeros((self.numL, x.shape[1]), np.complex128)
        buf[:self.order] = self.pre[:, None] * x
        buf = self.conv_hat[:, None] * np.fft.fft(buf, axis=0)
        return self.pre[:, None] * np.fft.ifft(buf, axis=0)[:self.order]

    def _bwd(self, x):
        # fastmat/Fourier.pyx:235-238: conj(F conj(x))
        return np.conj(self._fwd(np.conj(x.astype(np.complex128))))

    def dense(self):
        # fastmat/Fourier.pyx:241-246
        k = np.arange(self.order)
        return np.exp(np.multiply(*np.meshgrid(k, k)) * -2j * np.pi /
                      self.order)


class Diag(Op):
    """fastmat/Diag.pyx:149-174."""

    def __init__(self, d):
        self.d = np.array(d).reshape(-1)
        self.shape = (self.d.size, self.d.size)
        self.dtype = supported_dtype(self.d.dtype)

    def _fwd(self, x):
        return self.d[:, None] * x

    def _bwd(self, x):
        return np.conj(self.d)[:, None] * x

    def dense(self):
        return np.diag(self.d)


class Hadamard(Op):
    """fastmat/Hadamard.pyx:164-248: Sylvester-ordered Walsh-Hadamard."""

    def __init__(self, order):
        if order < 1:
            raise ValueError("order")
        self.order = order
        n = 1 << order
        self.shape = (n, n)
        self.dtype = np.int8

    def _fwd(self, x):
        # per-stage a+b / a-b butterflies at distance 2^s
        # (fastmat/Hadamard.pyx:36-61, :182-228)
        y = x.astype(self.out_dtype(x.dtype)).copy()
        n = y.shape[0]
        h = 1
        while h < n:
            y = y.reshape(n // (2 * h), 2, h, -1)
            a = y[:, 0].copy()
            b = y[:, 1]
            y[:, 0] += b
            y[:, 1] = a - b
            y = y.reshape(n, -1)
            h *= 2
        return y

    _bwd = _fwd

    def dense(self):
        n = self.shape[0]
        i = np.arange(n)
        bits = np.bitwise_and(i[:, None], i[None, :])
        par = np.zeros_like(bits)
        while np.any(bits):
            par ^= bits & 1
            bits >>= 1
        return (1 - 2 * par).astype(np.int8)


class Permutation(Op):
    """fastmat/Permutation.pyx:76-129."""

    def __init__(self, sigma):
        self.sigma = np.array(sigma).reshape(-1)
        if not np.array_equal(np.sort(self.sigma), np.arange(self.sigma.size)):
            raise ValueError("Not a permutation.")
        self.tau = np.argsort(self.sigma)
        self.shape = (self.sigma.size, self.sigma.size)
        self.dtype = np.int8

    def _fwd(self, x):
        return x[self.sigma]

    def _bwd(self, x):
        return x[self.tau]

    def dense(self):
        return np.eye(self.shape[0], dtype=np.int8)[self.sigma]


class Partial(Op):
    """fastmat/Partial.pyx:141-303: row/column sub-selection."""

    def __init__(self, mat, rows=None, cols=None):
        self.mat = mat

        def sel(v, size):
            if v is None:
                return None
            v = np.array(v)
            if v.dtype == bool:
                v = np.arange(size)[v]
            return v.astype(np.int64)

        self.rows = sel(rows, mat.shape[0])
        self.cols = sel(cols, mat.shape[1])
        self.shape = (mat.shape[0] if self.rows is None else self.rows.size,
                      mat.shape[1] if self.cols is None else self.cols.size)
        self.dtype = mat.dtype

    def _fwd(self, x):
        if self.cols is not None:
            full = np.zeros((self.mat.shape[1], x.shape[1]), x.dtype)
            full[self.cols] = x
            x = full
        y = self.mat.forward(x)
        return y if self.rows is None else y[self.rows]

    def _bwd(self, x):
        if self.rows is not None:
            full = np.zeros((self.mat.shape[0], x.shape[1]), x.dtype)
            full[self.rows] = x
            x = full
        y = self.mat.backward(x)
        return y if self.cols is None else y[self.cols]

    def dense(self):
        a = self.mat.dense()
        if self.rows is not None:
            a = a[self.rows]
        if self.cols is not None:
            a = a[:, self.cols]
        return a


class Product(Op):
    """fastmat/Product.pyx:53-257: right-to-left chain with a scalar."""

    def __init__(self, *terms):
        self.scalar = np.int8(1)
        self.terms = []
        dtype = np.int8
        for t in terms:
            if np.isscalar(t):
                dtype = promote(dtype, np.array(t).dtype)
                self.scalar = np.inner(self.scalar, t)
            elif isinstance(t, Product):
                self.scalar = self.scalar * t.scalar
                self.terms.extend(t.terms)
                dtype = promote(dtype, t.dtype)
            else:
                self.terms.append(t)
                dtype = promote(dtype, t.dtype)
        dtype = promote(dtype, safe_type_expansion(dtype))
        self.dtype = dtype
        self.scalar = np.array(self.scalar).astype(dtype)
        self.shape = (self.terms[0].shape[0], self.terms[-1].shape[1])

    def _fwd(self, x):
        y = (np.inner(x, self.scalar) if self.scalar != 1
             else x.astype(promote(x.dtype, self.dtype)))
        for t in reversed(self.terms):
            y = t.forward(y)
        return y

    def _bwd(self, x):
        s = np.conj(self.scalar)
        y = (np.inner(x, s) if self.scalar != 1
             else x.astype(promote(x.dtype, self.dtype)))
        for t in self.terms:
            y = t.backward(y)
        return y

    def dense(self):
        a = self.terms[-1].dense() * self.scalar
        for t in reversed(self.terms[:-1]):
            a = t.dense() @ a
        return a


class Sum(Op):
    """fastmat/Sum.pyx:73-186."""

    def __init__(self, *terms):
        flat = []
        for t in terms:
            flat.extend(t.terms if isinstance(t, Sum) else [t])
        self.terms = flat
        self.shape = flat[0].shape
        dtype = np.int8
        for t in flat:
            dtype = promote(dtype, t.dtype)
        self.dtype = dtype
        self.widen_input = True

    def _fwd(self, x):
        out = self.terms[0].forward(x).astype(self.out_dtype(x.dtype))
        for t in self.terms[1:]:
            out += t.forward(x)
        return out

    def _bwd(self, x):
        out = self.terms[0].backward(x).astype(self.out_dtype(x.dtype))
        for t in self.terms[1:]:
            out += t.backward(x)
        return out

    def dense(self):
        return sum(t.dense().astype(np.complex128) for t in self.terms)


class Blocks(Op):
    """fastmat/Blocks.pyx:65-312: a grid of operators; output block row r
    is the sum over c of block (r, c) applied to input segment c."""

    def __init__(self, rows):
        self.rows = [list(r) for r in rows]
        self.heights = [r[0].shape[0] for r in self.rows]
        self.widths = [t.shape[1] for t in self.rows[0]]
        for r in self.rows:
            if len(r) != len(self.widths):
                raise ValueError("Blocks: incompatible number of entries")
            for c, t in enumerate(r):
                if t.shape != (r[0].shape[0], self.widths[c]):
                    raise ValueError("Blocks: block shapes do not match")
        dtype = np.int8
        for r in self.rows:
            for t in r:
                dtype = promote(dtype, t.dtype)
        self.dtype = dtype
        self.shape = (sum(self.heights), sum(self.widths))
        self.widen_input = True

    @staticmethod
    def _cuts(sizes):
        return np.concatenate([[0], np.cumsum(sizes)]).astype(int)

    def _fwd(self, x):
        ro, ci = self._cuts(self.heights), self._cuts(self.widths)
        y = np.zeros((self.shape[0], x.shape[1]), self.out_dtype(x.dtype))
        for r, row in enumerate(self.rows):
            for c, t in enumerate(row):
                y[ro[r]:ro[r + 1]] += t.forward(x[ci[c]:ci[c + 1]])
        return y

    def _bwd(self, x):
        ro, ci = self._cuts(self.heights), self._cuts(self.widths)
        y = np.zeros((self.shape[1], x.shape[1]), self.out_dtype(x.dtype))
        for r, row in enumerate(self.rows):
            for c, t in enumerate(row):
                y[ci[c]:ci[c + 1]] += t.backward(x[ro[r]:ro[r + 1]])
        return y

    def dense(self):
        return np.block([[t.dense().astype(np.complex128) for t in r]
                         for r in self.rows])


class Sparse(Op):
    """fastmat/Sparse.pyx:25-185: a CSR matrix; forward S x, backward
    S^H x.  Restated with the CSR arrays (row of every nonzero from the row
    pointers, products scattered into the rows with np.add.at) rather than
    scipy's product."""

    def __init__(self, mat):
        a = mat.tocsr()
        self.shape = a.shape
        self.dtype = np.dtype(a.dtype).type
        self.val = np.asarray(a.data)
        self.col = np.asarray(a.indices, dtype=np.int64)
        self.row = np.repeat(np.arange(a.shape[0], dtype=np.int64),
                             np.diff(np.asarray(a.indptr, dtype=np.int64)))

    def _fwd(self, x):
        dt = self.out_dtype(x.dtype)
        y = np.zeros((self.shape[0], x.shape[1]), dt)
        np.add.at(y, self.row, self.val[:, None].astype(dt) *
                  x[self.col].astype(dt))
        return y

    def _bwd(self, x):
        dt = self.out_dtype(x.dtype)
        y = np.zeros((self.shape[1], x.shape[1]), dt)
        np.add.at(y, self.col, np.conj(self.val)[:, None].astype(dt) *
                  x[self.row].astype(dt))
        return y

    def dense(self):
        a = np.zeros(self.shape, np.complex128)
        np.add.at(a, (self.row, self.col), self.val)
        return a


class BlockDiag(Op):
    """fastmat/BlockDiag.pyx:95-200: operators along the block diagonal."""

    def __init__(self, *terms):
        if len(terms) < 1:
            raise ValueError("You must specify at least one matrix.")
        self.terms = terms
        dtype = np.int8
        for t in terms:
            dtype = promote(dtype, t.dtype)
        self.dtype = dtype
        self.shape = (sum(t.shape[0] for t in terms),
                      sum(t.shape[1] for t in terms))
        self.widen_input = True

    def _apply(self, x, fwd):
        n_out = self.shape[0] if fwd else self.shape[1]
        y = np.zeros((n_out, x.shape[1]), self.out_dtype(x.dtype))
        i = o = 0
        for t in self.terms:
            n_i, n_o = (t.shape[1], t.shape[0]) if fwd else t.shape
            y[o:o + n_o] = (t.forward if fwd else t.backward)(x[i:i + n_i])
            i += n_i
            o += n_o
        return y

    def _fwd(self, x):
        return self._apply(x, True)

    def _bwd(self, x):
        return self._apply(x, False)

    def dense(self):
        a = np.zeros(self.shape, np.complex128)
        r = c = 0
        for t in self.terms:
            a[r:r + t.shape[0], c:c + t.shape[1]] = t.dense()
            r += t.shape[0]
            c += t.shape[1]
        return a


class Kron(Op):
    """fastmat/Kron.pyx:79-353: mode-wise application, np.kron ordering
    (factor 0 is the most significant index)."""

    def __init__(self, *factors):
        if len(factors) < 2:
            raise ValueError("Kronecker: Product must have at least two terms")
        self.factors = factors
        dtype = np.int8
        for f in factors:
            if f.shape[0] != f.shape[1]:
                raise ValueError("Kronecker: Product terms must be symmetric")
            dtype = promote(dtype, f.dtype)
        self.dtype = promote(dtype, safe_type_expansion(dtype))
        n = int(np.prod([f.shape[0] for f in factors]))
        self.shape = (n, n)
        self.widen_input = True

    def _apply(self, x, fwd):
        dims = [f.shape[0] for f in self.factors]
        m = x.shape[1]
        y = x.astype(self.out_dtype(x.dtype))
        for k, f in enumerate(self.factors):
            hi = int(np.prod(dims[:k]))
            lo = int(np.prod(dims[k + 1:]))
            t = y.reshape(hi, dims[k], lo, m).transpose(1, 0, 2, 3)
            t = t.reshape(dims[k], -1)
            r = f.forward(t) if fwd else f.backward(t)
            y = r.reshape(dims[k], hi, lo, m).transpose(1, 0, 2, 3)
            y = y.reshape(-1, m).astype(self.out_dtype(x.dtype))
        return y

    def _fwd(self, x):
        return self._apply(x, True)

    def _bwd(self, x):
        return self._apply(x, False)

    def dense(self):
        a = self.factors[0].dense().astype(np.complex128)
        for f in self.factors[1:]:
            a = np.kron(a, f.dense())
        return a


class Hermitian(Op):
    """fastmat/Matrix.pyx:2224-2321: swaps forward and backward."""

    def __init__(self, mat):
        self.mat = mat
        self.shape = (mat.shape[1], mat.shape[0])
        self.dtype = mat.dtype

    def _fwd(self, x):
        return self.mat._bwd(x)

    def _bwd(self, x):
        return self.mat._fwd(x)

    def dense(self):
        return self.mat.dense().T.conj()


class Conjugate(Op):
    """fastmat/Matrix.pyx:2326-2412: conj o op o conj."""

    def __init__(self, mat):
        self.mat = mat
        self.shape = mat.shape
        self.dtype = mat.dtype

    def _fwd(self, x):
        return np.conj(self.mat._fwd(np.conj(x)))

    def _bwd(self, x):
        return np.conj(self.mat._bwd(np.conj(x)))

    def dense(self):
        return self.mat.dense().conj()


def Transpose(mat):
    """fastmat/Matrix.pyx:2417-2482: Hermitian of the Conjugate."""
    return Hermitian(Conjugate(mat))


class Circulant(Op):
    """Circulant; a multi-dimensional c gives the multi-level CirculantML.

    1-level circulant (fastmat/Circulant.pyx:63-137, 217-227, 344-425).

    C[i, j] = c[(i - j) mod n].  Forward pads to the embedding length L when
    that is cheaper, convolves via FFT with spectrum fft(c_pad) / L and
    truncates back to n rows.
    """

    def __new__(cls, c, *args, **kw):
        if np.ndim(np.squeeze(np.asarray(c))) > 1:
            return CirculantML(np.squeeze(np.asarray(c)))
        return super().__new__(cls)

    def __init__(self, c, optimize=True, max_stage=4):
        self.c = np.array(c).reshape(-1)
        n = self.c.size
        self.n = n
        self.L = circulant_length(n, optimize, max_stage)
        cp = self.c
        if self.L != n:
            cp = np.concatenate([self.c, np.zeros(self.L - (2 * n - 1),
                                                  self.c.dtype), self.c[1:]])
        self.spectrum = np.fft.fft(cp.astype(np.complex128)) / self.L
        self.shape = (n, n)
        self.dtype = np.complex128

    def _conv(self, x, spec):
        m = x.shape[1]
        buf = np.zeros((self.L, m), np.complex128)
        buf[:self.n] = x
        # F.H (Diag (F x)) with unnormalised F.H = L * ifft
        y = np.fft.ifft(spec[:, None] * np.fft.fft(buf, axis=0), axis=0)
        return y[:self.n] * self.L

    def _fwd(self, x):
        return self._conv(x, self.spectrum)

    def _bwd(self, x):
        return self._conv(x, np.conj(self.spectrum))

    def dense(self):
        n = self.n
        i = np.arange(n)
        return self.c[(i[:, None] - i[None, :]) % n].astype(np.complex128)


class Toeplitz(Op):
    """1-level Toeplitz (fastmat/Toeplitz.pyx:79-322, 628-734).

    Defined by the column vector vecC (n_r entries) and the row vector vecR
    (n_c - 1 entries, indexed backwards: T[0, j] = vecR[-j]).  Embedded into
    a circulant of length L >= n_r + n_c - 1 with zeros inserted at the split.
    """

    def __new__(cls, vecC, vecR=None, *args, split=None, **kw):
        if vecR is None and np.ndim(vecC) > 1:
            return ToeplitzML(vecC, split)
        return super().__new__(cls)

    def __init__(self, vecC, vecR=None, optimize=True, max_stage=4,
                 split=None):
        if vecR is None:
            # one-level tensor form: tenT = [vecC, vecR] split at `split`
            t = np.asarray(vecC).reshape(-1)
            sp = (t.size + 1) // 2 if split is None else int(
                np.atleast_1d(split)[0])
            vecC, vecR = t[:sp], t[sp:]
        dt = np.promote_types(np.asarray(vecC).dtype, np.asarray(vecR).dtype)
        self.vecC = np.asarray(vecC).astype(dt).reshape(-1)
        self.vecR = np.asarray(vecR).astype(dt).reshape(-1)
        self.nr = self.vecC.size
        self.nc = self.vecR.size + 1
        dd = self.nr + self.nc - 1
        self.L = toeplitz_length(dd, optimize, max_stage)
        t = np.concatenate([self.vecC, np.zeros(self.L - dd, dt), self.vecR])
        self.spectrum = np.fft.fft(t.astype(np.complex128)) / self.L
        self.shape = (self.nr, self.nc)
        self.dtype = np.complex128

    def _fwd(self, x):
        buf = np.zeros((self.L, x.shape[1]), np.complex128)
        buf[:self.nc] = x
        y = np.fft.ifft(self.spectrum[:, None] * np.fft.fft(buf, axis=0),
                        axis=0)
        return y[:self.nr] * self.L

    def _bwd(self, x):
        buf = np.zeros((self.L, x.shape[1]), np.complex128)
        buf[:self.nr] = x
        y = np.fft.ifft(np.conj(self.spectrum)[:, None] *
                        np.fft.fft(buf, axis=0), axis=0)
        return y[:self.nc] * self.L

    def dense(self):
        i = np.arange(self.nr)[:, None]
        j = np.arange(self.nc)[None, :]
        d = i - j
        full = np.concatenate([self.vecR, self.vecC])  # index d + nc - 1
        return full[d + self.nc - 1].astype(np.complex128)


class CirculantML(Op):
    """Multi-level circulant (fastmat/Circulant.pyx:138-215, 344-425):
    C[i, j] = c[((i_k - j_k) mod n_k)_k] with row / column indices in C
    order.  fastmat applies Kron(F_n1, ..., F_nd)^H diag(fftn(c) / N)
    Kron(F_n1, ..., F_nd) (its per-level zero padding only changes the FFT
    lengths, not the result); restated with numpy's fftn over the level
    axes of every column."""

    def __init__(self, c):
        self.c = np.asarray(c)
        self.dims = self.c.shape
        n = int(np.prod(self.dims))
        self.spectrum = np.fft.fftn(self.c.astype(np.complex128))
        self.shape = (n, n)
        self.dtype = np.complex128

    def _apply(self, x, spec):
        m = x.shape[1]
        axes = tuple(range(1, len(self.dims) + 1))
        X = x.T.reshape((m,) + self.dims).astype(np.complex128)
        Y = np.fft.ifftn(spec[None] * np.fft.fftn(X, axes=axes), axes=axes)
        return Y.reshape(m, -1).T

    def _fwd(self, x):
        return self._apply(x, self.spectrum)

    def _bwd(self, x):
        return self._apply(x, np.conj(self.spectrum))

    def dense(self):
        return level_diff(self.c, self.dims, self.dims).astype(np.complex128)


class ToeplitzML(Op):
    """Multi-level Toeplitz (fastmat/Toeplitz.pyx:180-322, 628-734): level
    k has split[k] rows and shape[k] - split[k] + 1 columns and
    T[i, j] = t[((i_k - j_k) mod shape[k])_k]; fastmat applies it as the
    matching rows and columns of the multi-level circulant of t."""

    def __init__(self, t, split=None):
        self.t = np.asarray(t)
        dims = np.array(self.t.shape)
        sp = (dims + 1) // 2 if split is None else np.asarray(split)
        self.rows = tuple(int(v) for v in sp)
        self.cols = tuple(int(d - v + 1) for d, v in zip(dims, sp))
        self.circ = CirculantML(self.t)
        n = int(np.prod(dims))
        idx = np.unravel_index(np.arange(n), self.t.shape)
        keep_r = np.ones(n, bool)
        keep_c = np.ones(n, bool)
        for k in range(len(dims)):
            keep_r &= idx[k] < self.rows[k]
            keep_c &= idx[k] < self.cols[k]
        self.sel_r = np.arange(n)[keep_r]
        self.sel_c = np.arange(n)[keep_c]
        self.n = n
        self.shape = (self.sel_r.size, self.sel_c.size)
        self.dtype = np.complex128

    def _fwd(self, x):
        buf = np.zeros((self.n, x.shape[1]), np.complex128)
        buf[self.sel_c] = x
        return self.circ._fwd(buf)[self.sel_r]

    def _bwd(self, x):
        buf = np.zeros((self.n, x.shape[1]), np.complex128)
        buf[self.sel_r] = x
        return self.circ._bwd(buf)[self.sel_c]

    def dense(self):
        return level_diff(self.t, self.rows, self.cols).astype(np.complex128)


def level_diff(ten, rows, cols):
    """M[i, j] = ten[((i_k - j_k) mod ten.shape[k])_k] for multi-indices
    i < rows, j < cols in C order (fastmat/Circulant.pyx:349-425)."""
    ri = np.unravel_index(np.arange(int(np.prod(rows))), rows)
    ci = np.unravel_index(np.arange(int(np.prod(cols))), cols)
    return ten[tuple((r[:, None] - c[None, :]) % n
                     for r, c, n in zip(ri, ci, ten.shape))]


class Dense(Op):
    """fastmat/Matrix.pyx:1831-1842 / 1924-1935: a dense ``Matrix(array)``."""

    def __init__(self, a):
        self.a = np.asarray(a)
        self.shape = self.a.shape
        self.dtype = supported_dtype(self.a.dtype)

    def _fwd(self, x):
        return self.a.dot(x)

    def _bwd(self, x):
        return np.conj(self.a.T).dot(x)

    def dense(self):
        return self.a


class Eye(Op):
    """fastmat/Eye.pyx: identity."""

    def __init__(self, n):
        self.shape = (n, n)
        self.dtype = np.int8

    def _fwd(self, x):
        return x.copy()

    _bwd = _fwd

    def dense(self):
        return np.eye(self.shape[0], dtype=np.int8)


# ----------------------------------------------------------------------------
# exact-phase DFT (accuracy anchor for large N)
# ----------------------------------------------------------------------------

def exact_dft_rows(x, rows, sign=-1):
    """DFT of the columns of ``x`` evaluated only at output ``rows`` with the
    phase (n * k) mod N reduced exactly in integers before the float64
    sin/cos, so the only rounding is in the final sum."""
    x = np.asarray(x, np.complex128)
    if x.ndim == 1:
        x = x[:, None]
    n = x.shape[0]
    idx = np.arange(n, dtype=np.int64)
    out = np.empty((len(rows), x.shape[1]), np.complex128)
    for r, k in enumerate(rows):
        ph = (idx * int(k)) % n
        w = np.exp(sign * 2j * np.pi * ph / n)
        out[r] = w @ x
    return out


def rel_err(out, ref):
    """fastmat's error metric (fastmat/inspect/test.py:186-188):
    max |out - ref| / max |ref|."""
    ref = np.asarray(ref)
    out = np.asarray(out)
    mx = float(np.max(np.abs(ref))) if ref.size else 0.0
    diff = float(np.max(np.abs(out.astype(np.complex128) -
                               ref.astype(np.complex128)))) if ref.size else 0.0
    return diff / mx if mx != 0 else diff


def fastmat_tolerance(eps, max_dim, tol_power=1.0):
    """fastmat/inspect/test.py:176-189: 5 * 2 * eps * (2 sqrt(maxDim))^p."""
    return 5 * 2.0 * eps * (2.0 * math.sqrt(max_dim)) ** tol_power
