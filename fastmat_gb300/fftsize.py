"""fastmat's FFT-size heuristics.

These decide the observable structure of the reference's operators (the
Bluestein length ``Fourier._numL`` and the embedding length of a padded
Circulant/Toeplitz), so the drop-in classes expose the same values.  The
GPU engine picks its own transform lengths independently.

Restated from fastmat/core/cmath.pyx:35-214, fastmat/Fourier.pyx:109-122,
fastmat/Circulant.pyx:107-124 and fastmat/Toeplitz.pyx:225-237.
"""

import math

import numpy as np


def _search(target, max_factor, state, best):
    # state = (complexity << 16) + length: one comparison orders by
    # complexity first (fastmat/core/cmath.pyx:35-82)
    for ff in range(max_factor, 0, -1):
        length = (state & 0xFFFF) * ff
        complexity = (state >> 16) + ff + 1
        packed = (complexity << 16) + length
        if packed <= best and length < target:
            best = _search(target, ff, packed, best)
        elif packed < best:
            best = packed
    return best


def find_optimal_fft_size(order, max_stage=4):
    """fastmat/core/cmath.pyx:85-153; ``remaining`` is a C float there."""
    padded = 1
    remaining = np.float32(order)
    while remaining > 64:
        padded *= 4
        remaining = np.float32(remaining / np.float32(4))
    x = int(math.ceil(float(remaining)))
    if x != 1:
        padded *= _search(x, max_stage, 1, (15 << 16) + 64) & 0xFFFF
    return padded


def fft_complexity(n):
    """fastmat/core/cmath.pyx:156-209 (float32 result)."""
    nn = int(n)
    c = 0
    while nn > 0 and nn % 4 == 0:
        c += 5
        nn //= 4
    if nn > 1 and nn % 2 == 0:
        c += 3
        nn //= 2
    ii = 3
    while nn > 1 and ii * ii < nn:
        if nn % ii == 0:
            c += ii + 1
            nn //= ii
        else:
            ii += 2
    if nn > 1:
        c += nn + 1
    return float(np.float32(n) * np.float32(c + 1))


def bluestein_length(order, optimize=True, max_stage=4):
    if not optimize:
        return 0
    padded = find_optimal_fft_size(order * 2 - 1, max_stage)
    direct = fft_complexity(order)
    conv = 2 * fft_complexity(padded) + 2 * padded + 2 * order
    return 0 if direct < conv else padded


def circulant_length(n, optimize=True, max_stage=4):
    if not optimize:
        return n
    padded = find_optimal_fft_size(2 * n - 1, max_stage)
    return padded if fft_complexity(n) > fft_complexity(padded) else n


def toeplitz_length(dd, optimize=True, max_stage=4):
    if not optimize:
        return dd
    opt = find_optimal_fft_size(dd, max_stage)
    return opt if fft_complexity(opt) < fft_complexity(dd) else dd
