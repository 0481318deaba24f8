"""fastmat's element types and binary promotion rule.

fastmat supports eight element types (fastmat/core/types.pxd:45-55) and
promotes with numpy's ``promote_types`` over them
(fastmat/core/types.pyx:443-453); unsupported numpy types are first mapped
onto the closest supported one (fastmat/core/types.pyx:423-426).
"""

import numpy as np

SUPPORTED = (np.int8, np.int16, np.int32, np.int64,
             np.float32, np.float64, np.complex64, np.complex128)


def supported(dtype):
    """The fastmat type a numpy dtype is handled as."""
    dt = np.dtype(dtype)
    if dt.type in SUPPORTED:
        return dt.type
    if dt.kind == 'b':
        return np.int8
    if dt.kind == 'u':
        return {1: np.int16, 2: np.int32, 4: np.int64}.get(dt.itemsize,
                                                             np.int64)
    raise TypeError("unsupported data type %s" % dt)


def promote(a, b):
    return supported(np.promote_types(supported(a), supported(b)))


def safe_type_expansion(dtype):
    """fastmat/core/types.pyx:378-394."""
    dt = np.dtype(dtype).type
    if dt in (np.int8, np.int16):
        return np.float32
    if dt in (np.int32, np.int64):
        return np.float64
    return dt


def is_integer(dtype):
    return np.dtype(dtype).kind in 'iub'


def is_complex(dtype):
    return np.dtype(dtype).kind == 'c'


def single(dtype):
    """The single-precision form of a floating type (ints unchanged)."""
    dt = np.dtype(dtype).type
    if dt == np.complex128:
        return np.complex64
    if dt == np.float64:
        return np.float32
    return dt
