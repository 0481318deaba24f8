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
        # None: an empty (zero) block of a Blocks node
        idx = [-1 if c is None else c._emit(self) for c in children]
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


#: outputs at least this large come from page-locked host memory
_PINNED_MIN_BYTES = 1 << 20


def _host_output(rows, cols, dt):
    """Fortran-ordered (rows x cols) result array.  Large ones live in
    page-locked memory from torch's caching host allocator (reused across
    calls once freed), so the device-to-host copies of fm_execute_host run
    asynchronously, overlapped with the transform of the next column
    chunk; the array keeps its torch storage alive."""
    dt = np.dtype(dt)
    if rows * cols * dt.itemsize >= _PINNED_MIN_BYTES:
        torch = _torch()
        t = torch.empty((cols, rows), dtype=_torch_dtype(dt),
                        pin_memory=True)
        return t.numpy().T
    return np.empty((rows, cols), dtype=dt, order='F')


def _device_index(device=None):
    """Index of a CUDA device (torch.device, int or None = current); -1
    when no CUDA device is visible."""
    torch = _torch()
    if device is None:
        return torch.cuda.current_device() if torch.cuda.is_available() else -1
    if isinstance(device, int):
        return device
    d = torch.device(device)
    if d.type != 'cuda':
        raise ValueError("not a CUDA device: %s" % (device,))
    return d.index if d.index is not None else torch.cuda.current_device()


class _device_scope:
    """Make device `dev` current inside the block (no-op for dev < 0)."""

    def __init__(self, dev):
        self.dev = dev
        self.ctx = None

    def __enter__(self):
        if self.dev >= 0:
            self.ctx = _torch().cuda.device(self.dev)
            self.ctx.__enter__()
        return self

    def __exit__(self, *exc):
        if self.ctx is not None:
            return self.ctx.__exit__(*exc)
        return False


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

    def plan(self, out_dtype=np.complex128, device=None):
        """The native plan computing in the type of ``out_dtype`` on a CUDA
        device (default: the current one).  A plan's constants live on the
        device it was built on, so plans are kept per device; the plan is
        built with that device current."""
        code = _compute_code(out_dtype, self._precision)
        dev = _device_index(device)
        p = self._plans.get((dev, code))
        if p is None:
            b = _Builder()
            root = self._emit(b)
            with _device_scope(dev):
                p = _native.Plan(b.nodes, b.children, root, code, b.keep)
            self._plans[(dev, code)] = p
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
        """y = A x.  1-D or 2-D numpy arrays or CUDA torch tensors.

        numpy inputs are transformed synchronously and a failure the kernels
        record on the device (a bounded wait that gave up) raises here.  CUDA
        tensors are transformed asynchronously on the current stream, like
        any torch operation; ``check()`` synchronises and raises such a
        failure."""
        return self._transform(arrX, _native.FORWARD)

    def check(self):
        """Synchronise with the device and raise RuntimeError if a kernel of
        one of this operator's plans recorded a failure since the last
        check (results of the affected calls are incomplete)."""
        for p in list(self._plans.values()):
            p.check()

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
        # (an operator without a GPU form raises NotImplementedError here)
        plan = self.plan(out_dt)
        if not _torch().cuda.is_available():
            raise RuntimeError("fastmat_gb300 needs a CUDA device")
        xf = np.asfortranarray(x2)
        y = _host_output(n_out, M, out_dt)
        # fm_execute_host: column chunks pipelined over copy-in, compute and
        # copy-out streams, synchronous, device status checked
        plan.execute_host(direction, xf, y)
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
            # the plan of the tensor's device, launched with it current
            plan = self.plan(out_dt, device=x.device)
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

    @property
    def largestEigenValue(self):
        """Eigenvalue of largest magnitude of a square operator
        (fastmat/Matrix.pyx:680-765): scipy's eigs (ARPACK) on the
        LinearOperator whose matvecs run on the GPU; numpy's eigvals of the
        dense array for a 1 x 1 operator.  Cached."""
        v = getattr(self, '_largestEigenValue', None)
        if v is None:
            if self.numRows != self.numCols:
                raise ValueError("largestEigenValue: Matrix must be square.")
            if self.numRows > 1:
                from scipy.sparse.linalg import eigs
                v = eigs(self._promoted_operator(), 1,
                         return_eigenvectors=False)[0]
            else:
                v = np.linalg.eigvals(self.array)[0]
            self._largestEigenValue = v
        return v

    @property
    def largestEigenVec(self):
        """Eigenvector of the largest-magnitude eigenvalue
        (fastmat/Matrix.pyx:771-811).  Cached with the eigenvalue."""
        v = getattr(self, '_largestEigenVec', None)
        if v is None:
            if self.numRows != self.numCols:
                raise ValueError("largestEigenVec: Matrix must be square.")
            dt = np.promote_types(np.float64, self.dtype)
            if self.numRows > 2:
                from scipy.sparse.linalg import eigs
                S, V = eigs(self._promoted_operator(), 1,
                            return_eigenvectors=True)
                S, v = S[0], V[:, 0]
            else:
                S, V = np.linalg.eig(self.array)
                S, v = S.astype(dt)[0], V[:, 0].astype(dt)
            self._largestEigenValue = S
            self._largestEigenVec = v
        return v

    @property
    def largestSingularVectors(self):
        """(u, v) leading left and right singular vectors
        (fastmat/Matrix.pyx:925-983): scipy's svds over GPU matvecs; a dense
        SVD for a single row or column.  Cached with the singular value.
        Real vectors are returned as float64; complex ones stay complex
        (fastmat casts both to float64, dropping imaginary parts)."""
        v = getattr(self, '_largestSingularVectors', None)
        if v is None:
            if self.numRows > 1 and self.numCols > 1:
                from scipy.sparse.linalg import svds
                U, S, V = svds(self._promoted_operator(), 1,
                               return_singular_vectors=True)
            else:
                U, S, V = np.linalg.svd(np.atleast_2d(self.array))
            self._largestSingularValue = float(np.asarray(S)[0])
            v = (U.astype(np.float64) if not np.iscomplexobj(U) else U,
                 V.astype(np.float64) if not np.iscomplexobj(V) else V)
            self._largestSingularVectors = v
        return v

    def _promoted_operator(self):
        from scipy.sparse.linalg import LinearOperator
        return LinearOperator(shape=self.shape, matvec=self.forward,
                              rmatvec=self.backward, matmat=self.forward,
                              dtype=np.promote_types(np.float64, self.dtype))

    @property
    def gram(self):
        """A^H A as a fastmat operator (fastmat/Matrix.pyx:1026-1028)."""
        g = getattr(self, '_gram', None)
        if g is None:
            from .operators import Product
            g = self._gram = Product(self.H, self)
        return g

    @property
    def inverse(self):
        """The inverse, applied by an iterative solver
        (fastmat/Matrix.pyx:1290-1291)."""
        inv = getattr(self, '_inverse', None)
        if inv is None:
            inv = self._inverse = Inverse(self)
        return inv

    @property
    def pseudoInverse(self):
        """The Moore-Penrose pseudo-inverse, applied by least squares
        (fastmat/Matrix.pyx:1313-1314)."""
        inv = getattr(self, '_pseudoInverse', None)
        if inv is None:
            inv = self._pseudoInverse = PseudoInverse(self)
        return inv

    # ------------------------------------------------------------ dense
    def reference(self):
        """Dense ground truth built without the fast transforms."""
        return self._reference()

    def _reference(self):
        if self._array is not None:
            return self._array.copy()
        raise NotImplementedError

    #: bytes of unit vectors plus results per engine call when columns or
    #: rows of the operator are formed on the GPU
    _UNIT_BLOCK_BYTES = 1 << 28

    def _unit_blocks(self, idx, direction, in_dtype):
        """Yield (start, stop, Y) for consecutive blocks of the indices idx,
        Y a CUDA tensor (n_out, stop - start) holding A e_i (forward) or
        A^H e_i (backward) for i in idx[start:stop].  The unit vectors of a
        block are written on the device and the whole block is one engine
        call (as many columns as fit _UNIT_BLOCK_BYTES)."""
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("fastmat_gb300 needs a CUDA device")
        n_in = self.numCols if direction == _native.FORWARD else self.numRows
        n_out = self.numRows if direction == _native.FORWARD else self.numCols
        in_dtype = np.dtype(in_dtype)
        out_dtype = np.dtype(self._output_dtype(in_dtype))
        per_col = n_in * in_dtype.itemsize + n_out * out_dtype.itemsize
        k = int(max(1, min(len(idx), self._UNIT_BLOCK_BYTES // per_col)))
        tdt = _torch_dtype(in_dtype)
        idx_dev = torch.as_tensor(np.asarray(idx, dtype=np.int64),
                                  device='cuda')
        for a in range(0, len(idx), k):
            b = min(a + k, len(idx))
            e = torch.zeros((b - a, n_in), dtype=tdt, device='cuda')
            e[torch.arange(b - a, device='cuda'), idx_dev[a:b]] = 1
            yield a, b, self._transform_device(e.t(), direction)

    def _unit_matrix(self, idx, direction, in_dtype):
        """numpy (n_out, len(idx)) Fortran array of A e_i / A^H e_i."""
        n_out = self.numRows if direction == _native.FORWARD else self.numCols
        out = np.empty((n_out, len(idx)),
                       dtype=self._output_dtype(np.dtype(in_dtype)),
                       order='F')
        for a, b, y in self._unit_blocks(idx, direction, in_dtype):
            out[:, a:b] = y.t().cpu().numpy().T
        return out

    def _check_index(self, idx, size, what):
        arr = np.asarray(idx)
        if arr.size and (arr.min() < 0 or arr.max() >= size):
            raise IndexError("%s index exceeds matrix dimensions." % what)

    @property
    def array(self):
        """Dense array of the operator (fastmat/Matrix.pyx:360-387),
        computed with the fast transform: the forward applied to identity
        columns on the GPU, a block of columns per engine call.  Cached."""
        if self._array is not None:
            return self._array
        a = getattr(self, '_arrayCache', None)
        if a is None:
            a = self.getArray()
        return a

    def getArray(self):
        if self._array is not None:
            return self._array
        self._arrayCache = self._unit_matrix(
            np.arange(self.numCols), _native.FORWARD, self.numpyType)
        return self._arrayCache

    def _dense_if_known(self):
        return (self._array if self._array is not None
                else getattr(self, '_arrayCache', None))

    def getCol(self, idx):
        """Column idx (fastmat/Matrix.pyx:429-458)."""
        if not np.isscalar(idx):
            raise TypeError("Scalar index required.")
        if idx < 0 or idx >= self.numCols:
            raise IndexError("Column index exceeds matrix dimensions.")
        d = self._dense_if_known()
        if d is not None:
            return np.squeeze(d[:, idx])
        return self._getCol(idx)

    def _getCol(self, idx):
        return self._unit_matrix([idx], _native.FORWARD,
                                 self.numpyType)[:, 0]

    def getRow(self, idx):
        """Row idx (fastmat/Matrix.pyx:501-530): the conjugate of A^H e_idx."""
        if not np.isscalar(idx):
            raise TypeError("Scalar index required.")
        if idx < 0 or idx >= self.numRows:
            raise IndexError("Row index exceeds matrix dimensions.")
        d = self._dense_if_known()
        if d is not None:
            return np.squeeze(d[idx, :])
        return self._getRow(idx)

    def _getRow(self, idx):
        return np.conj(self._unit_matrix([idx], _native.BACKWARD,
                                         self.numpyType)[:, 0])

    def _selection(self, indices, size):
        if isinstance(indices, slice):
            return np.arange(*indices.indices(size))
        arr = np.array(indices)
        if arr.ndim > 1:
            raise IndexError("Index array must have at most one dimension.")
        return arr.astype(np.int64)

    def getCols(self, indices):
        """Columns by index, slice or index vector
        (fastmat/Matrix.pyx:389-427); all selected columns are formed by
        one engine call per block of columns."""
        if np.isscalar(indices):
            return self.getCol(indices)
        d = self._dense_if_known()
        if d is not None:
            return d[:, indices]
        idx = self._selection(indices, self.numCols)
        self._check_index(idx, self.numCols, "Column")
        out = self._unit_matrix(idx, _native.FORWARD, self.numpyType)
        return out.astype(self.numpyType, copy=False)

    def getRows(self, indices):
        """Rows by index, slice or index vector
        (fastmat/Matrix.pyx:460-499)."""
        if np.isscalar(indices):
            return self.getRow(indices)
        d = self._dense_if_known()
        if d is not None:
            return d[indices, :]
        idx = self._selection(indices, self.numRows)
        self._check_index(idx, self.numRows, "Row")
        out = np.conj(self._unit_matrix(idx, _native.BACKWARD,
                                        self.numpyType)).T
        return np.ascontiguousarray(out).astype(self.numpyType, copy=False)

    def _getItem(self, idxRow, idxCol):
        d = self._dense_if_known()
        if d is not None:
            return d[idxRow, idxCol]
        if self.numRows < self.numCols:
            return self._getCol(idxCol)[idxRow]
        return self._getRow(idxRow)[idxCol]

    def __getitem__(self, tplIdx):
        """Element, row, column or sub-array access
        (fastmat/Matrix.pyx:532-658)."""
        def selector(index, size):
            if isinstance(index, (list, tuple, np.ndarray)):
                arr = np.squeeze(np.asarray(index))
                if arr.ndim == 0:
                    arr = arr.reshape(1)
                if not np.issubdtype(arr.dtype, np.integer):
                    raise TypeError("Group indexing only allows int vectors.")
                if arr.ndim != 1:
                    raise IndexError("Group indexing vector must be 1D.")
                return (arr[0] if arr.size == 1 else arr), arr.size
            if index is Ellipsis:
                return Ellipsis, size
            if isinstance(index, slice):
                slc = slice(*index.indices(size))
                if slc.start == 0 and slc.stop == size and slc.step == 1:
                    return Ellipsis, size
                return slc, len(range(slc.start, slc.stop, slc.step))
            if np.isscalar(index):
                return index, 1
            raise TypeError("Axis index is neither iterable, slice or int.")

        rowSel, colSel = Ellipsis, Ellipsis
        rowCount, colCount = self.numRows, self.numCols
        if tplIdx is not Ellipsis:
            if not isinstance(tplIdx, tuple):
                raise IndexError("Invalid type of indexing tuple.")
            if len(tplIdx) < 1 or len(tplIdx) > 2:
                raise IndexError("None or too many indices given.")
            rowSel, rowCount = selector(tplIdx[0], self.numRows)
            if len(tplIdx) > 1:
                colSel, colCount = selector(tplIdx[1], self.numCols)
        if np.isscalar(rowSel):
            if np.isscalar(colSel):
                return self._getItem(rowSel, colSel)
            return self._getRow(rowSel)[colSel]
        if np.isscalar(colSel):
            return self._getCol(colSel)[rowSel]
        if rowSel is Ellipsis:
            if colSel is Ellipsis:
                return self.array
            return self.getCols(colSel)
        if colSel is Ellipsis:
            return self.getRows(rowSel)
        if rowCount <= 0 or colCount <= 0:
            return None
        if rowCount < colCount:
            return self.getRows(rowSel)[:, colSel]
        return self.getCols(colSel)[rowSel]

    # ------------------------------------------------------------ norms
    def _unit_norms(self, direction, size):
        """Euclidean norms of A e_i (forward) or A^H e_i (backward) for every
        i < size, float64, reduced on the GPU block by block (only the norms
        come back to the host)."""
        torch = _torch()
        out = np.empty(size, dtype=np.float64)
        for a, b, y in self._unit_blocks(np.arange(size), direction,
                                          np.float64):
            out[a:b] = torch.linalg.vector_norm(
                y, dim=0).to(torch.float64).cpu().numpy()
        return out

    def _getColNorms(self):
        return self._unit_norms(_native.FORWARD, self.numCols)

    def _getRowNorms(self):
        return self._unit_norms(_native.BACKWARD, self.numRows)

    def _getColNormalized(self):
        norms = self.colNorms
        if np.any(norms == 0):
            raise ValueError("Normalization: Matrix has zero-norm column.")
        from .operators import Diag
        return self * Diag(1. / norms)

    def _getRowNormalized(self):
        norms = self.rowNorms
        if np.any(norms == 0):
            raise ValueError("Normalization: Matrix has zero-norm row.")
        from .operators import Diag
        return Diag(1. / norms) * self

    @property
    def colNorms(self):
        """Column norms, float64 (fastmat/Matrix.pyx:1035-1088).  Cached."""
        v = getattr(self, '_colNorms', None)
        if v is None:
            v = self._colNorms = self._getColNorms()
        return v

    def getColNorms(self):
        self._colNorms = self._getColNorms()
        return self._colNorms

    @property
    def rowNorms(self):
        """Row norms, float64 (fastmat/Matrix.pyx:1095-1148).  Cached."""
        v = getattr(self, '_rowNorms', None)
        if v is None:
            v = self._rowNorms = self._getRowNorms()
        return v

    def getRowNorms(self):
        self._rowNorms = self._getRowNorms()
        return self._rowNorms

    @property
    def colNormalized(self):
        """A diag(1 / colNorms) (fastmat/Matrix.pyx:1168-1177)."""
        v = getattr(self, '_colNormalized', None)
        if v is None:
            v = self._colNormalized = self._getColNormalized()
        return v

    @property
    def rowNormalized(self):
        """diag(1 / rowNorms) A (fastmat/Matrix.pyx:1197-1206)."""
        v = getattr(self, '_rowNormalized', None)
        if v is None:
            v = self._rowNormalized = self._getRowNormalized()
        return v


class _Solved(Matrix):
    """An operator applied by solving with another: each column of the
    input is one call of a scipy iterative solver whose matvecs are the
    nested operator's GPU transforms (fastmat/Matrix.pyx:2490-2600)."""

    def __init__(self, matrix, rows, cols, solver):
        if not isinstance(matrix, Matrix):
            raise TypeError("Inverse: Not a fastmat Matrix")
        self._nested = matrix
        self._content = (matrix, )
        self._init_properties(rows, cols,
                              np.promote_types(matrix.dtype, np.float32),
                              **matrix._getProperties())
        self._solver = solver

    def _emit(self, b):
        raise NotImplementedError(
            "%s is applied by an iterative solver and cannot be fused into "
            "a GPU plan" % self.__class__.__name__)

    def _operator(self, direction):
        op = self._nested.scipyLinearOperator
        return op if direction == _native.FORWARD else op.H

    def _transform(self, x, direction):
        if _is_tensor(x):
            # the solver iterates on the host; a tensor comes back as a
            # (column-major) tensor on its device
            y = self._transform(x.detach().cpu().numpy(), direction)
            torch = _torch()
            if y.ndim == 1:
                return torch.from_numpy(y).to(x.device)
            return torch.from_numpy(np.ascontiguousarray(y.T)).to(x.device).t()
        x = np.asarray(x)
        if x.ndim < 1 or x.ndim > 2:
            raise ValueError("Input data array must be 1D or 2D")
        n_req = self.numCols if direction == _native.FORWARD else self.numRows
        if x.shape[0] != n_req:
            raise ValueError(
                "Mismatch of vector size %d to relevant matrix axis %d" % (
                    x.shape[0], n_req))
        op = self._operator(direction)
        flat = x.ndim == 1
        x2 = x.reshape(n_req, 1) if flat else x
        cols = [self._solver(op, x2[:, m], atol=1e-12)[0]
                for m in range(x2.shape[1])]
        n_out = self.numRows if direction == _native.FORWARD else self.numCols
        y = (np.asfortranarray(np.stack(cols, axis=1)) if cols else
             np.empty((n_out, 0), dtype=self.dtype, order='F'))
        return y.reshape(n_out) if flat else y


class Inverse(_Solved):
    """A^-1 of a square operator, applied by scipy's lgmres
    (fastmat/Matrix.pyx:2490-2541)."""

    def __init__(self, matrix):
        from scipy.sparse.linalg import lgmres
        if not isinstance(matrix, Matrix):
            raise TypeError("Inverse: Not a fastmat Matrix")
        if matrix.shape[0] != matrix.shape[1]:
            raise ValueError("Inverse: Matrix not square, so not invertible.")
        super().__init__(matrix, matrix.shape[0], matrix.shape[0], lgmres)

    def __repr__(self):
        return "<%s.(^-1)>" % self._nested.__repr__()

    def _reference(self):
        return np.linalg.inv(self._nested.reference())


class PseudoInverse(_Solved):
    """A^+ applied by scipy's lsqr (fastmat/Matrix.pyx:2544-2600)."""

    def __init__(self, matrix):
        from scipy.sparse.linalg import lsqr
        if not isinstance(matrix, Matrix):
            raise TypeError("Inverse: Not a fastmat Matrix")
        super().__init__(matrix, matrix.shape[1], matrix.shape[0], lsqr)

    def __repr__(self):
        return "<%s.(^+)>" % self._nested.__repr__()

    def _reference(self):
        return np.linalg.pinv(self._nested.reference())


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
