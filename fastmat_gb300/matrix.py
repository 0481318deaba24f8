"""The Matrix base class: fastmat's public operator API on the GB300 engine.

``forward``/``backward`` follow fastmat/Matrix.pyx:1844-2007: the input is a
1-D or 2-D array whose first axis matches the operator, its type is promoted
by fastmat's rule (fastmat/Matrix.pyx:1799-1808) and the result is a
Fortran-ordered array (1-D for 1-D input).  Host (numpy) inputs are copied to
the GPU, transformed there by the native engine and copied back; CUDA torch
tensors are transformed in place on the device and a CUDA tensor is
returned.  There is no CPU fallback: without the native library or a CUDA
device the transforms raise.
"""

import numpy as np

from . import _native
from . import types as T


class _Builder:
    """Collects the fm_node records of an operator tree."""

    def __init__(self):
        self.nodes = []
        self.children = []
        self.keep = []

    def vec(self, arr, integer=False):
        if arr is None:
            return None, 0, 0
        a = np.asarray(arr)
        if integer:
            a = a.astype(np.int64)
        else:
            a = a.astype(T.supported(a.dtype), copy=False)
        a = np.ascontiguousarray(a.reshape(-1, order='F') if a.ndim > 1
                                 else a)
        self.keep.append(a)
        return a.ctypes.data, a.size, _native.DTYPE_CODE[a.dtype]

    def add(self, kind, mat, children=(), n=0, vec0=None, vec1=None,
            int0=False, int1=False, scalar=1.0):
        node = _native.FmNode()
        node.kind = kind
        node.dtype = _native.DTYPE_CODE[np.dtype(mat.dtype)]
        node.rows, node.cols = mat.shape
        node.n = n
        p, ln, t = self.vec(vec0, int0)
        node.vec0, node.len0, node.type0 = p, ln, t
        p, ln, t = self.vec(vec1, int1)
        node.vec1, node.len1, node.type1 = p, ln, t
        s = complex(scalar)
        node.scalar_re, node.scalar_im = s.real, s.imag
        idx = [c._emit(self) for c in children]
        node.first_child = len(self.children)
        node.num_children = len(idx)
        self.children.extend(idx)
        self.nodes.append(node)
        return len(self.nodes) - 1


_TORCH_DTYPES = None


def _torch():
    import torch
    return torch


def _torch_dtype(dt):
    global _TORCH_DTYPES
    torch = _torch()
    if _TORCH_DTYPES is None:
        _TORCH_DTYPES = {
            np.dtype(np.int8): torch.int8, np.dtype(np.int16): torch.int16,
            np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
            np.dtype(np.float32): torch.float32,
            np.dtype(np.float64): torch.float64,
            np.dtype(np.complex64): torch.complex64,
            np.dtype(np.complex128): torch.complex128}
    return _TORCH_DTYPES[np.dtype(dt)]


def _numpy_dtype(tdt):
    torch = _torch()
    for k, v in {np.int8: torch.int8, np.int16: torch.int16,
                 np.int32: torch.int32, np.int64: torch.int64,
                 np.float32: torch.float32, np.float64: torch.float64,
                 np.complex64: torch.complex64,
                 np.complex128: torch.complex128}.items():
        if v == tdt:
            return np.dtype(k)
    raise TypeError("unsupported tensor dtype %s" % tdt)


def _compute_code(out_dtype, precision='native'):
    """Element type a plan computes in for a given output type.

    float64 / complex128 results are computed in double-float arithmetic
    (pairs of float32, ~2^-48 relative precision) unless
    ``precision='fp64'`` asks for the FP64 pipe; integer results in int64.
    """
    dt = np.dtype(out_dtype)
    if dt.kind in 'iub':
        return _native.FM_I64
    if precision == 'bf16' and dt == np.float32:
        return _native.FM_F32_TC
    if precision != 'fp64':
        if dt == np.complex128:
            return _native.FM_C128_DF
        if dt == np.float64:
            return _native.FM_F64_DF
    return _native.DTYPE_CODE[dt]


class Matrix:
    """A linear operator with fastmat's interface.

    ``Matrix(array)`` wraps a dense 2-D array (fastmat/Matrix.pyx:1468);
    subclasses define structured operators.  Options (keyword arguments)
    follow fastmat: ``minType`` (minimum internal type) and
    ``widenInputDatatype``.  ``precision`` selects how floating-point work
    is done: ``'native'`` (default: float64 / complex128 results computed in
    double-float arithmetic on the FP32 pipes), ``'fp64'`` (the FP64 pipe)
    or ``'fp32'`` (opt-in reduced precision: float32 / complex64 arithmetic
    and output) or ``'bf16'`` (as 'fp32', and the 16-point groups of
    Hadamard transforms on float32 data run on the tensor cores as BF16
    matrix products with FP32 accumulation, the operand split exactly into
    three BF16 terms).
    """

    _array = None

    def __init__(self, arrMatrix, **options):
        if not isinstance(arrMatrix, np.ndarray):
            raise TypeError("Matrix: Matrix is not a numpy ndarray")
        if arrMatrix.ndim != 2:
            raise ValueError("Matrix: array must be 2-D")
        self._array = np.array(arrMatrix, dtype=T.supported(arrMatrix.dtype))
        self._init_properties(arrMatrix.shape[0], arrMatrix.shape[1],
                              self._array.dtype.type, **options)

    # ------------------------------------------------------------ properties
    def _init_properties(self, rows, cols, dtype, **options):
        self._shape = (int(rows), int(cols))
        self._dtype = T.supported(dtype)
        self._minType = T.supported(options.get('minType', np.int8))
        self._widenInputDatatype = options.get('widenInputDatatype', False)
        prec = options.get('precision', 'native')
        if prec not in ('native', 'fp32', 'fp64', 'bf16'):
            raise ValueError(
                "precision must be 'native', 'fp64', 'fp32' or 'bf16'")
        self._precision = prec
        self._plans = {}

    def _getProperties(self):
        return {'minType': self._minType, 'precision': self._precision}

    @property
    def shape(self):
        return self._shape

    @property
    def numRows(self):
        return self._shape[0]

    @property
    def numCols(self):
        return self._shape[1]

    @property
    def dtype(self):
        return self._dtype

    @property
    def numpyType(self):
        return np.dtype(self._dtype)

    @property
    def content(self):
        return getattr(self, '_content', ())

    @property
    def precision(self):
        return self._precision

    @property
    def H(self):
        return Hermitian(self)

    @property
    def T(self):
        return Transpose(self)

    @property
    def conj(self):
        return _conjugate_of(self)

    def __len__(self):
        return self._shape[0]

    def __iter__(self):
        return iter(self.content)

    def __repr__(self):
        return "<%s[%dx%d]:0x%12x>" % (self.__class__.__name__,
                                       self.numRows, self.numCols, id(self))

    # ------------------------------------------------------------ operators
    __array_priority__ = 20.0

    def __add__(self, other):
        if isinstance(other, Matrix):
            from .operators import Sum
            return Sum(self, other)
        raise TypeError("Not an addition of fastmat matrices.")

    __radd__ = __add__

    def __sub__(self, other):
        if isinstance(other, Matrix):
            from .operators import Product, Sum
            return Sum(self, Product(other, np.int8(-1),
                                     typeExpansion=np.int8))
        raise TypeError("Not a subtraction of fastmat matrices.")

    def __rsub__(self, other):
        if isinstance(other, Matrix):
            from .operators import Product, Sum
            return Sum(other, Product(self, np.int8(-1),
                                      typeExpansion=np.int8))
        raise TypeError("Not a subtraction of fastmat matrices.")

    def __mul__(self, factor):
        if isinstance(factor, np.ndarray) or _is_tensor(factor):
            return self.forward(factor)
        from .operators import Product
        return Product(self, factor, typeExpansion=np.int8)

    def __rmul__(self, factor):
        if np.isscalar(factor) or isinstance(factor, Matrix):
            from .operators import Product
            return Product(factor, self, typeExpansion=np.int8)
        raise TypeError("Invalid product term for fastmat Matrix.")

    def __truediv__(self, divisor):
        if np.isscalar(divisor):
            if divisor == 0:
                raise ZeroDivisionError("Division by Zero.")
            from .operators import Product
            return Product(self, 1. / divisor)
        raise TypeError("Only scalars allowed as divisors.")

    def __floordiv__(self, divisor):
        raise NotImplementedError("Matrix Floor division not allowed.")

    # ------------------------------------------------------------ engine
    def _emit(self, b):
        """Append this operator's node(s) to a builder; return the index."""
        if self._array is None:
            raise NotImplementedError(
                "%s has no GPU form" % self.__class__.__name__)
        return b.add(_native.NODE_DENSE, self, vec0=self._array)

    def _output_dtype(self, x_dtype):
        internal = T.promote(x_dtype, self._minType)
        out = T.promote(internal, self._dtype)
        if self._precision in ('fp32', 'bf16'):
            out = T.single(out)
        return out

    def plan(self, out_dtype=np.complex128):
        """The native plan computing in the type of ``out_dtype``."""
        code = _compute_code(out_dtype, self._precision)
        p = self._plans.get(code)
        if p is None:
            b = _Builder()
            root = self._emit(b)
            p = _native.Plan(b.nodes, b.children, root, code, b.keep)
            self._plans[code] = p
        return p

    def autotune(self, num_cols=1, out_dtype=None, cache=True):
        """Pick the tile shape of every GPU launch of this operator by
        timing the candidates (see fm_plan_autotune) for `num_cols`
        columns; the choice is cached on disk per device and plan."""
        from . import tuning
        if out_dtype is None:
            out_dtype = self._output_dtype(np.complex128 if T.is_complex(
                self.dtype) else np.float64)
        return tuning.autotune(self.plan(out_dtype), num_cols, cache)

    def forward(self, arrX):
        """y = A x.  1-D or 2-D numpy arrays or CUDA torch tensors."""
        return self._transform(arrX, _native.FORWARD)

    def backward(self, arrX):
        """y = A^H x."""
        return self._transform(arrX, _native.BACKWARD)

    def _transform(self, x, direction):
        if _is_tensor(x):
            return self._transform_device(x, direction)
        if not isinstance(x, np.ndarray):
            x = np.asarray(x)
        n_req = self.numCols if direction == _native.FORWARD else self.numRows
        n_out = self.numRows if direction == _native.FORWARD else self.numCols
        if x.ndim < 1 or x.ndim > 2:
            raise ValueError("Input data array must be 1D or 2D")
        if x.shape[0] != n_req:
            raise ValueError(
                "Mismatch of vector size %d to relevant matrix axis %d" % (
                    x.shape[0], n_req))
        flat = x.ndim == 1
        x2 = x.reshape(n_req, 1) if flat else x
        sdt = T.supported(x2.dtype)
        if x2.dtype != sdt:
            x2 = x2.astype(sdt)
        out_dt = np.dtype(self._output_dtype(sdt))
        M = x2.shape[1]
        if M == 0:
            y = np.empty((n_out, 0), dtype=out_dt, order='F')
            return y
        plan = self.plan(out_dt)
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("fastmat_gb300 needs a CUDA device")
        xf = np.asfortranarray(x2)
        xt = torch.from_numpy(xf.T).to('cuda')
        yt = torch.empty((M, n_out), dtype=_torch_dtype(out_dt),
                         device='cuda')
        stream = torch.cuda.current_stream().cuda_stream
        plan.execute(direction, xt.data_ptr(), _native.DTYPE_CODE[xf.dtype],
                     n_req, yt.data_ptr(), _native.DTYPE_CODE[out_dt], n_out,
                     M, stream)
        y = yt.cpu().numpy().T
        plan.check()
        return y.reshape(n_out) if flat else y

    def _transform_device(self, x, direction):
        torch = _torch()
        n_req = self.numCols if direction == _native.FORWARD else self.numRows
        n_out = self.numRows if direction == _native.FORWARD else self.numCols
        if not x.is_cuda:
            return torch.from_numpy(np.ascontiguousarray(
                self._transform(x.numpy(), direction)))
        if x.dim() < 1 or x.dim() > 2:
            raise ValueError("Input data array must be 1D or 2D")
        if x.shape[0] != n_req:
            raise ValueError(
                "Mismatch of vector size %d to relevant matrix axis %d" % (
                    x.shape[0], n_req))
        flat = x.dim() == 1
        M = 1 if flat else x.shape[1]
        in_dt = _numpy_dtype(x.dtype)
        out_dt = np.dtype(self._output_dtype(in_dt))
        if flat:
            xc = x.contiguous()
        elif x.stride(0) == 1 and (M == 1 or x.stride(1) >= n_req):
            xc = x
        else:
            xc = x.t().contiguous().t()
        # one column: its stride along the (size-1) column axis is irrelevant
        ld_x = n_req if (flat or M == 1) else xc.stride(1)
        yt = torch.empty((M, n_out), dtype=_torch_dtype(out_dt),
                         device=x.device)
        if M > 0:
            plan = self.plan(out_dt)
            with torch.cuda.device(x.device):
                stream = torch.cuda.current_stream().cuda_stream
                plan.execute(direction, xc.data_ptr(),
                             _native.DTYPE_CODE[in_dt], ld_x, yt.data_ptr(),
                             _native.DTYPE_CODE[out_dt], n_out, M, stream)
        return yt.reshape(n_out) if flat else yt.t()

    # ------------------------------------------------------------ callers
    @property
    def largestSingularValue(self):
        """sigma_max of the operator, as fastmat computes it
        (fastmat/Matrix.pyx:826-921): scipy's svds (ARPACK) on the
        LinearOperator, whose matvecs run on the GPU; a dense SVD for
        operators with at most two rows or columns.  Cached."""
        v = getattr(self, '_largestSingularValue', None)
        if v is None:
            if self.numRows > 2 and self.numCols > 2:
                from scipy.sparse.linalg import LinearOperator, svds
                op = LinearOperator(
                    shape=self.shape, matvec=self.forward,
                    rmatvec=self.backward, matmat=self.forward,
                    dtype=np.promote_types(np.float64, self.dtype))
                v = float(svds(op, 1, return_singular_vectors=False)[0])
            else:
                v = float(np.linalg.svd(np.atleast_2d(self.array),
                                        compute_uv=False)[0])
            self._largestSingularValue = v
        return v

    @property
    def scipyLinearOperator(self):
        """scipy.sparse.linalg.LinearOperator whose matvec / rmatvec /
        matmat are this operator's forward / backward
        (fastmat/Matrix.pyx:985-1006)."""
        op = getattr(self, '_scipyLinearOperator', None)
        if op is None:
            from scipy.sparse.linalg import LinearOperator
            op = LinearOperator(shape=self.shape, matvec=self.forward,
                                rmatvec=self.backward, matmat=self.forward,
                                dtype=self.dtype)
            self._scipyLinearOperator = op
        return op

    # ------------------------------------------------------------ dense
    def reference(self):
        """Dense ground truth built without the fast transforms."""
        return self._reference()

    def _reference(self):
        if self._array is not None:
            return self._array.copy()
        raise NotImplementedError

    @property
    def array(self):
        """Dense array of the operator, computed with the fast transform
        (forward applied to identity columns on the GPU)."""
        if self._array is not None:
            return self._array
        eye = np.eye(self.numCols, dtype=np.int8)
        return self.forward(eye)

    def getCol(self, idx):
        e = np.zeros(self.numCols, dtype=np.int8)
        e[idx] = 1
        return self.forward(e)

    def getRow(self, idx):
        e = np.zeros(self.numRows, dtype=np.int8)
        e[idx] = 1
        return np.conj(self.backward(e))


def _fcontig_tensor(t):
    """2-D column-major view (n, M) of a tensor (copies if needed)."""
    if t.dim() == 1:
        t = t.unsqueeze(1)
    if t.stride(0) == 1 and (t.shape[1] <= 1 or t.stride(1) >= t.shape[0]):
        return t
    return t.t().contiguous().t()


def _is_tensor(x):
    t = type(x)
    return t.__module__.startswith('torch') and t.__name__ == 'Tensor'


class Hermitian(Matrix):
    """Hermitian transpose (fastmat/Matrix.pyx:2224-2321)."""

    def __init__(self, matrix):
        if not isinstance(matrix, Matrix):
            raise TypeError("Hermitian: Not a fastmat Matrix")
        self._nested = matrix
        self._content = (matrix,)
        self._init_properties(matrix.numCols, matrix.numRows, matrix.dtype,
                              **matrix._getProperties())

    def __repr__(self):
        return "<%s.H>" % self._nested.__repr__()

    @property
    def H(self):
        return self._nested

    def _emit(self, b):
        return b.add(_native.NODE_HERMITIAN, self, children=(self._nested,))

    def _reference(self):
        return self._nested.reference().T.conj()


class Conjugate(Matrix):
    """Complex conjugate (fastmat/Matrix.pyx:2326-2412)."""

    def __init__(self, matrix):
        if not isinstance(matrix, Matrix):
            raise TypeError("Conjugate: Not a fastmat Matrix")
        self._nested = matrix
        self._content = (matrix,)
        self._init_properties(matrix.numRows, matrix.numCols, matrix.dtype,
                              **matrix._getProperties())

    def __repr__(self):
        return "<conj(%s)>" % self._nested.__repr__()

    @property
    def conj(self):
        return self._nested

    def _emit(self, b):
        return b.add(_native.NODE_CONJUGATE, self, children=(self._nested,))

    def _reference(self):
        return self._nested.reference().conj()


def _conjugate_of(matrix):
    """fastmat/Matrix.pyx:2305-2323 (getConjugate): real operators are their
    own conjugate."""
    return Conjugate(matrix) if T.is_complex(matrix.dtype) else matrix


class Transpose(Hermitian):
    """Transpose = Hermitian of the Conjugate (fastmat/Matrix.pyx:2417)."""

    def __init__(self, matrix):
        if not isinstance(matrix, Matrix):
            raise TypeError("Transpose: Not a fastmat Matrix")
        self._nestedConj = matrix
        inner = _conjugate_of(matrix)
        self._nested = inner
        self._content = (inner,)
        self._init_properties(inner.numCols, inner.numRows, inner.dtype,
                              **inner._getProperties())

    def __repr__(self):
        return "<%s.T>" % self._nestedConj.__repr__()

    @property
    def T(self):
        return self._nestedConj

    def _reference(self):
        return self._nestedConj.reference().T
