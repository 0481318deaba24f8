"""ctypes binding of the native engine's C ABI (include/fmgpu.h).

The library is loaded lazily on first use.  If it is missing, or no CUDA
device is present, every transform raises RuntimeError: there is no CPU
fallback for the matvec path.
"""

import ctypes
import os
import threading

import numpy as np

from . import _build

FM_OK = 0
FM_ERR_VALUE = 1
FM_ERR_TYPE = 2
FM_ERR_UNSUPPORTED = 3
FM_ERR_CUDA = 4
FM_ERR_NOMEM = 5
FM_ERR_TIMEOUT = 6

# element types: fastmat's ftype numbering (fastmat/core/types.pxd:45-55)
FM_I8, FM_I16, FM_I32, FM_I64, FM_F32, FM_F64, FM_C64, FM_C128 = range(8)
DTYPE_CODE = {
    np.dtype(np.int8): FM_I8, np.dtype(np.int16): FM_I16,
    np.dtype(np.int32): FM_I32, np.dtype(np.int64): FM_I64,
    np.dtype(np.float32): FM_F32, np.dtype(np.float64): FM_F64,
    np.dtype(np.complex64): FM_C64, np.dtype(np.complex128): FM_C128,
}
CODE_DTYPE = {v: k for k, v in DTYPE_CODE.items()}

# compute types: float64 / complex128 in double-float arithmetic
FM_F64_DF = 16
FM_C128_DF = 17
FM_F32_TC = 18   # float32, Hadamard 16-point groups on the tensor cores

(NODE_FOURIER, NODE_CIRCULANT, NODE_TOEPLITZ, NODE_HADAMARD, NODE_DIAG,
 NODE_PARTIAL, NODE_PERMUTATION, NODE_PRODUCT, NODE_SUM, NODE_KRON,
 NODE_HERMITIAN, NODE_CONJUGATE, NODE_EYE, NODE_DENSE,
 NODE_BLOCKS, NODE_SPARSE) = range(1, 17)

FORWARD = 0
BACKWARD = 1


class FmNode(ctypes.Structure):
    _fields_ = [
        ('kind', ctypes.c_int32), ('dtype', ctypes.c_int32),
        ('rows', ctypes.c_int64), ('cols', ctypes.c_int64),
        ('first_child', ctypes.c_int32), ('num_children', ctypes.c_int32),
        ('n', ctypes.c_int64),
        ('vec0', ctypes.c_void_p), ('len0', ctypes.c_int64),
        ('type0', ctypes.c_int32), ('pad0', ctypes.c_int32),
        ('vec1', ctypes.c_void_p), ('len1', ctypes.c_int64),
        ('type1', ctypes.c_int32), ('pad1', ctypes.c_int32),
        ('scalar_re', ctypes.c_double), ('scalar_im', ctypes.c_double),
    ]


class FmPlanInfo(ctypes.Structure):
    _fields_ = [
        ('rows', ctypes.c_int64), ('cols', ctypes.c_int64),
        ('num_launches_fwd', ctypes.c_int32),
        ('num_launches_bwd', ctypes.c_int32),
        ('scratch_bytes_per_col', ctypes.c_int64),
        ('const_bytes', ctypes.c_int64),
        ('compute_type', ctypes.c_int32), ('pad', ctypes.c_int32),
    ]


#: every entry point include/fmgpu.h declares
EXPORTS = ('fm_plan_create', 'fm_execute', 'fm_execute_profiled',
           'fm_execute_static', 'fm_execute_host', 'fm_release_host_staging',
           'fm_plan_check',
           'fm_plan_set_tile', 'fm_plan_set_tile_layout', 'fm_plan_get_tile',
           'fm_plan_autotune', 'fm_plan_set_wait_limit',
           'fm_plan_destroy', 'fm_plan_get_info', 'fm_plan_describe',
           'fm_batch_create', 'fm_batch_execute', 'fm_batch_execute_graph',
           'fm_batch_check', 'fm_batch_set_wait_limit', 'fm_batch_get_info',
           'fm_batch_destroy', 'fm_reduce_mulconj',
           'fm_debug_fail_allocation', 'fm_last_error', 'fm_version')

_lib = None
_lock = threading.Lock()


def library_path():
    """The engine library: FASTMAT_GB300_LIB if set (a custom build),
    else the in-tree libfmgpu.so."""
    return os.environ.get('FASTMAT_GB300_LIB') or _build.LIB


def load(build_if_missing=True):
    """Load libfmgpu.so (building it first if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError('fastmat_gb300 native library is not '
                                   'built: %s' % path)
            _build.build()
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        I32, I64 = ctypes.c_int32, ctypes.c_int64
        lib.fm_plan_create.argtypes = [ctypes.POINTER(FmNode), I32,
                                       ctypes.POINTER(I32), I32, I32, I32,
                                       ctypes.POINTER(P)]
        lib.fm_plan_create.restype = ctypes.c_int
        lib.fm_execute.argtypes = [P, I32, P, I32, I64, P, I32, I64, I64, P]
        lib.fm_execute.restype = ctypes.c_int
        lib.fm_execute_profiled.argtypes = [
            P, I32, P, I32, I64, P, I32, I64, I64, P,
            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(I32)]
        lib.fm_execute_profiled.restype = ctypes.c_int
        lib.fm_execute_static.argtypes = [P, I32, P, I32, I64, P, I32, I64,
                                          I64, P]
        lib.fm_execute_static.restype = ctypes.c_int
        lib.fm_execute_host.argtypes = [P, I32, P, I32, I64, P, I32, I64, I64]
        lib.fm_execute_host.restype = ctypes.c_int
        lib.fm_plan_set_tile.argtypes = [P, I32, I32, I32, I32]
        lib.fm_plan_set_tile.restype = ctypes.c_int
        lib.fm_plan_set_tile_layout.argtypes = [P, I32, I32, I32, I32, I32]
        lib.fm_plan_set_tile_layout.restype = ctypes.c_int
        lib.fm_plan_get_tile.argtypes = [P, I32, I32, ctypes.POINTER(I32),
                                         ctypes.POINTER(I32),
                                         ctypes.POINTER(I32)]
        lib.fm_plan_get_tile.restype = ctypes.c_int
        lib.fm_plan_autotune.argtypes = [P, I32, I64, P]
        lib.fm_plan_autotune.restype = ctypes.c_int
        lib.fm_plan_check.argtypes = [P]
        lib.fm_plan_check.restype = ctypes.c_int
        lib.fm_plan_set_wait_limit.argtypes = [P, I64]
        lib.fm_plan_set_wait_limit.restype = ctypes.c_int
        lib.fm_batch_set_wait_limit.argtypes = [P, I64]
        lib.fm_batch_set_wait_limit.restype = ctypes.c_int
        lib.fm_release_host_staging.argtypes = []
        lib.fm_release_host_staging.restype = ctypes.c_int
        lib.fm_debug_fail_allocation.argtypes = [I32]
        lib.fm_debug_fail_allocation.restype = ctypes.c_int
        lib.fm_plan_destroy.argtypes = [P]
        lib.fm_plan_destroy.restype = ctypes.c_int
        lib.fm_plan_get_info.argtypes = [P, ctypes.POINTER(FmPlanInfo)]
        lib.fm_plan_get_info.restype = ctypes.c_int
        lib.fm_plan_describe.argtypes = [P, I32, ctypes.c_char_p, I64]
        lib.fm_plan_describe.restype = ctypes.c_int
        PP = ctypes.POINTER(P)
        PI32 = ctypes.POINTER(I32)
        PI64 = ctypes.POINTER(I64)
        lib.fm_batch_create.argtypes = [I32, PP, PI32, PP, PI32, PI64, PP,
                                        PI32, PI64, PI64, PP]
        lib.fm_batch_create.restype = ctypes.c_int
        lib.fm_batch_execute.argtypes = [P, P]
        lib.fm_batch_execute.restype = ctypes.c_int
        lib.fm_batch_execute_graph.argtypes = [P, P]
        lib.fm_batch_execute_graph.restype = ctypes.c_int
        lib.fm_batch_check.argtypes = [P]
        lib.fm_batch_check.restype = ctypes.c_int
        lib.fm_batch_get_info.argtypes = [P, PI64, PI64, PI64]
        lib.fm_batch_get_info.restype = ctypes.c_int
        lib.fm_batch_destroy.argtypes = [P]
        lib.fm_batch_destroy.restype = ctypes.c_int
        lib.fm_reduce_mulconj.argtypes = [I64, I64, I64, I64, I32, P, I64,
                                          P, I64, P, ctypes.c_double, P, P,
                                          I64, P]
        lib.fm_reduce_mulconj.restype = ctypes.c_int
        lib.fm_last_error.argtypes = []
        lib.fm_last_error.restype = ctypes.c_char_p
        lib.fm_version.argtypes = []
        lib.fm_version.restype = I32
        _lib = lib
        return lib


def check(status):
    """Map a C ABI status to the exception fastmat raises for that case."""
    if status == FM_OK:
        return
    msg = _lib.fm_last_error().decode(errors='replace') if _lib else ''
    if status == FM_ERR_VALUE:
        raise ValueError(msg)
    if status == FM_ERR_TYPE:
        raise TypeError(msg)
    if status == FM_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status == FM_ERR_NOMEM:
        raise MemoryError(msg)
    raise RuntimeError('fmgpu error %d: %s' % (status, msg))


class Plan:
    """Owns one native plan (an operator tree compiled for one compute
    type)."""

    def __init__(self, nodes, children, root, compute_type, keepalive):
        lib = load()
        n = len(nodes)
        arr = (FmNode * n)(*nodes)
        ch = (ctypes.c_int32 * max(1, len(children)))(*children)
        handle = ctypes.c_void_p()
        self._keep = keepalive
        check(lib.fm_plan_create(arr, n, ch, len(children), root,
                                 compute_type, ctypes.byref(handle)))
        self.handle = handle
        self.compute_type = compute_type
        self._lib = lib

    def execute(self, direction, x_ptr, x_type, ld_x, y_ptr, y_type, ld_y,
                num_cols, stream):
        check(self._lib.fm_execute(self.handle, direction, x_ptr, x_type,
                                   ld_x, y_ptr, y_type, ld_y, num_cols,
                                   stream))

    def execute_profiled(self, direction, x_ptr, x_type, ld_x, y_ptr, y_type,
                         ld_y, num_cols, stream):
        """Run once, returning each launch's elapsed milliseconds."""
        cap = 64
        ms = (ctypes.c_float * cap)()
        n = ctypes.c_int32(cap)
        check(self._lib.fm_execute_profiled(
            self.handle, direction, x_ptr, x_type, ld_x, y_ptr, y_type, ld_y,
            num_cols, stream, ms, ctypes.byref(n)))
        return [ms[i] for i in range(n.value)]

    def execute_host(self, direction, x, y):
        """x, y: Fortran-ordered 2-D numpy arrays (host memory)."""
        check(self._lib.fm_execute_host(
            self.handle, direction, x.ctypes.data, DTYPE_CODE[x.dtype],
            x.shape[0], y.ctypes.data, DTYPE_CODE[y.dtype], y.shape[0],
            x.shape[1]))

    def tiles(self, direction):
        """[(vectors_per_tile, nbuf, layout)] of every launch."""
        out = []
        for k in range(self.num_launches(direction)):
            b, n, lay = (ctypes.c_int32(), ctypes.c_int32(),
                         ctypes.c_int32())
            check(self._lib.fm_plan_get_tile(self.handle, direction, k,
                                             ctypes.byref(b), ctypes.byref(n),
                                             ctypes.byref(lay)))
            out.append((b.value, n.value, lay.value))
        return out

    def set_tiles(self, direction, tiles):
        """Replay [(vectors_per_tile, nbuf, layout)] (as tiles() returns)."""
        for k, (b, n, lay) in enumerate(tiles):
            check(self._lib.fm_plan_set_tile_layout(self.handle, direction, k,
                                                    b, n, lay))

    def num_launches(self, direction):
        inf = self.info()
        return (inf.num_launches_fwd if direction == FORWARD
                else inf.num_launches_bwd)

    def autotune(self, direction, num_cols, stream=None):
        check(self._lib.fm_plan_autotune(self.handle, direction, num_cols,
                                         stream))

    def check(self):
        """Raise if a kernel of this plan reported a failure (syncs)."""
        check(self._lib.fm_plan_check(self.handle))

    def set_wait_limit(self, polls):
        """Polls of a bounded device wait before it gives up (see
        fm_plan_set_wait_limit; default 2^22)."""
        check(self._lib.fm_plan_set_wait_limit(self.handle, polls))

    def info(self):
        inf = FmPlanInfo()
        check(self._lib.fm_plan_get_info(self.handle, ctypes.byref(inf)))
        return inf

    def describe(self, direction=FORWARD):
        buf = ctypes.create_string_buffer(1 << 16)
        check(self._lib.fm_plan_describe(self.handle, direction, buf,
                                         len(buf)))
        return buf.value.decode()

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                self._lib.fm_plan_destroy(h)
            except Exception:
                pass
            self.handle = None


def release_host_staging():
    """Free the device buffers the host entry point keeps for the current
    device (fm_release_host_staging)."""
    check(load().fm_release_host_staging())


def fail_allocation(after):
    """Test hook: make the device allocation after `after` more successful
    ones fail (fm_debug_fail_allocation); after < 0 disarms."""
    check(load().fm_debug_fail_allocation(after))


def reduce_mulconj(A, n, Cc, num_cols, type_code, u, ld_u, v, ld_v, out,
                   scale=1.0, d=None, w=None, ld_w=0, stream=None):
    """fm_reduce_mulconj on device pointers (see include/fmgpu.h)."""
    lib = load()
    check(lib.fm_reduce_mulconj(A, n, Cc, num_cols, type_code, u, ld_u, v,
                                ld_v, out, scale, d, w, ld_w, stream))


class BatchHandle:
    """Owns one native batch (see fm_batch_create)."""

    def __init__(self, plans, directions, xs, x_types, ld_x, ys, y_types,
                 ld_y, num_cols):
        lib = load()
        n = len(plans)
        P = ctypes.c_void_p
        arr = lambda t, v: (t * n)(*v)  # noqa: E731
        handle = ctypes.c_void_p()
        self._plans = list(plans)   # the batch reads their constants
        check(lib.fm_batch_create(
            n, arr(P, [p.handle.value for p in plans]),
            arr(ctypes.c_int32, directions), arr(P, xs),
            arr(ctypes.c_int32, x_types), arr(ctypes.c_int64, ld_x),
            arr(P, ys), arr(ctypes.c_int32, y_types),
            arr(ctypes.c_int64, ld_y), arr(ctypes.c_int64, num_cols),
            ctypes.byref(handle)))
        self.handle = handle
        self._lib = lib

    def execute(self, stream=None, graph=False):
        fn = (self._lib.fm_batch_execute_graph if graph
              else self._lib.fm_batch_execute)
        check(fn(self.handle, stream))

    def check(self):
        check(self._lib.fm_batch_check(self.handle))

    def set_wait_limit(self, polls):
        """Polls of a grid-barrier wait (fm_batch_set_wait_limit)."""
        check(self._lib.fm_batch_set_wait_limit(self.handle, polls))

    def info(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(self._lib.fm_batch_get_info(self.handle, ctypes.byref(a),
                                          ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                self._lib.fm_batch_destroy(h)
            except Exception:
                pass
            self.handle = None
