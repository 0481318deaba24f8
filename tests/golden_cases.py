"""Loader for the golden fixtures in tests/golden/ (written by
tests/golden/make_golden.py from the reference fastmat)."""

import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


class Case:
    def __init__(self, meta, data):
        self.name = meta['name']
        self.expr = meta['expr']
        self.shape = tuple(meta['shape'])
        self.dtype = np.dtype(meta['dtype'])
        self.params = {k: data['%s__p_%s' % (self.name, k)]
                       for k in meta['params']}
        self.x = data['%s__x' % self.name]
        self.g = data['%s__g' % self.name]
        self.fwd = data['%s__fwd' % self.name]
        self.bwd = data['%s__bwd' % self.name]
        self.dense = (data['%s__dense' % self.name] if meta['dense']
                      else None)

    def build(self, namespace):
        env = dict(namespace)
        env.update(self.params)
        return eval(self.expr, env)  # noqa: S307 (fixture expressions)

    def __repr__(self):
        return self.name


def load_cases():
    with open(os.path.join(HERE, 'operators.json')) as f:
        meta = json.load(f)
    data = np.load(os.path.join(HERE, 'operators.npz'))
    return [Case(m, data) for m in meta]


def load_accessors():
    """name -> {key: array} of the reference's dense accessors
    (tests/golden/accessors.npz)."""
    data = np.load(os.path.join(HERE, 'accessors.npz'))
    out = {}
    for k in data.files:
        name, key = k.split('__', 1)
        out.setdefault(name, {})[key] = data[k]
    return out


def load_fftsizes():
    return np.load(os.path.join(HERE, 'fftsizes.npz'))


def load_circulant1024():
    return np.load(os.path.join(HERE, 'circulant1024.npz'))


#: cases where the reference itself is less accurate than 1e-12: fastmat's
#: Bluestein chirp forms the phase n^2 pi / N in float64
#: (fastmat/Fourier.pyx:130-146), which costs ~1e-12 at N = 4099; these are
#: held to the exact DFT separately.
REFERENCE_ERROR = {'fourier_4099': 5e-12}


def tolerance(ref, x, case_dtype=None, name=None):
    """Accuracy bound for a result against a reference output.

    Double-precision results are held to 1e-12 relative error (fastmat's
    metric, max|out-ref|/max|ref|).  Where the reference itself computed in
    single precision (numpy 2's FFT keeps complex64 for single-precision
    input) the bound is the single-precision one of fastmat's test harness
    (fastmat/inspect/test.py:176-189 with TOL_POWER 1 and eps(float32)).
    """
    single = (np.dtype(ref.dtype) in (np.float32, np.complex64) or
              np.dtype(x.dtype) in (np.float32, np.complex64))
    if single:
        n = max(ref.shape[0], x.shape[0])
        return 5 * 2.0 * np.finfo(np.float32).eps * 2.0 * np.sqrt(n)
    return REFERENCE_ERROR.get(name, 1e-12)
