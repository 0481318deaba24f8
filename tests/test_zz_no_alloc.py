"""fm_execute_static: the entry point for callers that must not allocate
device memory during a call (for example code running under a framework that
has already reserved the device memory for its own caching allocator, or a
latency-critical loop that cannot take the synchronisation cudaMalloc and
cudaFree imply).  It runs a plan like fm_execute but keeps the scratch its
multi-launch plans need in a fixed 16 MiB array compiled into the library.

This file is collected last so that, if it fails, a run stopping at the
first failure has already run every other test.  It calls both entry points
through the C ABI (ctypes) on device buffers and compares them."""

import ctypes

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu

STATIC_BYTES = 16 << 20


def _plan_with_scratch(n=20000):
    """A long circulant: its four-step convolution keeps an L-row scratch
    buffer per column between launches (L = 65536 here)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(11)
    c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    op = fg.Circulant(c)
    plan = op.plan(np.complex128)
    assert plan.info().scratch_bytes_per_col > 0
    return op, plan


def _run(lib_fn, plan, xt, yt, m, stream):
    from fastmat_gb300 import _native
    n_in, n_out = xt.shape[1], yt.shape[1]
    return lib_fn(plan.handle, _native.FORWARD, ctypes.c_void_p(xt.data_ptr()),
                  _native.FM_C128, n_in, ctypes.c_void_p(yt.data_ptr()),
                  _native.FM_C128, n_out, m, ctypes.c_void_p(stream))


def test_static_entry_matches_fm_execute_on_two_calls_in_a_row():
    import torch
    from fastmat_gb300 import _native
    lib = _native.load()
    op, plan = _plan_with_scratch()
    n = op.numRows
    m = 4
    per_col = plan.info().scratch_bytes_per_col
    assert per_col * m <= STATIC_BYTES
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(5)
    for call in range(2):
        x = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
        xt = torch.from_numpy(x).cuda()  # row k = column k (column-major)
        y_ref = torch.empty_like(xt)
        y_sta = torch.full_like(xt, float('nan'))
        assert _run(lib.fm_execute, plan, xt, y_ref, m, stream) == 0
        st = _run(lib.fm_execute_static, plan, xt, y_sta, m, stream)
        assert st == 0, lib.fm_last_error()
        torch.cuda.synchronize()
        a, b = y_ref.cpu().numpy(), y_sta.cpu().numpy()
        assert np.all(np.isfinite(b))
        assert fo.rel_err(b, a) <= 1e-12, (call, fo.rel_err(b, a))
        # and both against the FFT definition of the circulant product
        want = np.fft.ifft(np.fft.fft(op.tenC)[None, :] *
                           np.fft.fft(x, axis=1), axis=1)
        assert fo.rel_err(b, want) <= 1e-12


def test_static_entry_rejects_oversize_calls():
    import torch
    from fastmat_gb300 import _native
    lib = _native.load()
    op, plan = _plan_with_scratch()
    per_col = plan.info().scratch_bytes_per_col
    m = STATIC_BYTES // per_col + 1
    n = op.numRows
    xt = torch.zeros((m, n), dtype=torch.complex128, device='cuda')
    yt = torch.zeros_like(xt)
    st = _run(lib.fm_execute_static, plan, xt, yt, m,
              torch.cuda.current_stream().cuda_stream)
    assert st == _native.FM_ERR_VALUE
    assert b'static' in lib.fm_last_error()
