"""fm_execute_static: the entry point for callers that must not allocate
device memory during a call (for example code running under a framework that
has already reserved the device memory for its own caching allocator, or a
latency-critical loop that cannot take the synchronisation cudaMalloc and
cudaFree imply).  It runs a plan like fm_execute but keeps the scratch its
multi-launch plans need in a fixed 16 MiB array compiled into the library.

This file is collected last so that, if it fails, a run stopping at the
first failure has already run every other test.  It calls both entry points
through the C ABI (ctypes) on device buffers and compares them.  Each case
runs the static entry point on a FRESH plan before that plan has ever run
through fm_execute (so the plan owns no scratch buffer the static path could
borrow) and checks that the device's free memory does not change across the
two static calls."""

import ctypes

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu

STATIC_BYTES = 16 << 20


def _cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _operator(kind):
    """Operators whose plans keep scratch between launches: a long circulant
    (four-step convolution, an L-row buffer per column, L = 65536) and a Sum
    of two of them (also the accumulating copy that reads its destination
    first)."""
    import fastmat_gb300 as fg
    rng = np.random.default_rng(11)
    n = 20000
    c1, c2 = _cplx(rng, n), _cplx(rng, n)
    if kind == 'circulant':
        return fg.Circulant(c1), fo.Circulant(c1)
    return (fg.Sum(fg.Circulant(c1), fg.Circulant(c2)),
            fo.Sum(fo.Circulant(c1), fo.Circulant(c2)))


def _run(lib_fn, plan, direction, xt, yt, m, stream):
    from fastmat_gb300 import _native
    n_in, n_out = xt.shape[1], yt.shape[1]
    return lib_fn(plan.handle, direction, ctypes.c_void_p(xt.data_ptr()),
                  _native.FM_C128, n_in, ctypes.c_void_p(yt.data_ptr()),
                  _native.FM_C128, n_out, m, ctypes.c_void_p(stream))


@pytest.mark.parametrize('direction', [0, 1], ids=['forward', 'backward'])
@pytest.mark.parametrize('kind', ['circulant', 'sum'])
def test_static_entry_matches_fm_execute_on_two_calls_in_a_row(kind,
                                                               direction):
    import torch
    from fastmat_gb300 import _native
    lib = _native.load()
    m = 4
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(5 + direction)
    op, oop = _operator(kind)
    n = op.numRows
    xs = [torch.from_numpy(_cplx(rng, m, n)).cuda() for _ in range(2)]
    y_sta = [torch.full_like(x, float('nan')) for x in xs]
    y_ref = [torch.empty_like(x) for x in xs]
    # warm-up on another plan of the same operator: loads the kernels and the
    # static array's module, so only the calls under test remain
    warm = op.plan(np.complex128)
    assert _run(lib.fm_execute_static, warm, direction, xs[0], y_ref[0], m,
                stream) == 0
    # a fresh plan: it has never run, so it owns no scratch buffer
    op.__dict__.pop('_plans', None)
    op._plans = {}
    plan = op.plan(np.complex128)
    assert plan is not warm
    per_col = plan.info().scratch_bytes_per_col
    assert per_col > 0 and per_col * m <= STATIC_BYTES
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2):
        st = _run(lib.fm_execute_static, plan, direction, xs[call],
                  y_sta[call], m, stream)
        assert st == 0, lib.fm_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, \
        "fm_execute_static allocated device memory"
    # the allocating entry point on the same plan, afterwards
    for call in range(2):
        assert _run(lib.fm_execute, plan, direction, xs[call], y_ref[call], m,
                    stream) == 0
    plan.check()
    for call in range(2):
        a, b = y_ref[call].cpu().numpy(), y_sta[call].cpu().numpy()
        assert np.all(np.isfinite(b))
        assert fo.rel_err(b, a) <= 1e-12, (call, fo.rel_err(b, a))
        x = xs[call].cpu().numpy().T
        want = (oop.forward(x) if direction == 0 else oop.backward(x)).T
        assert fo.rel_err(b, want) <= 1e-12


def test_static_entry_rejects_oversize_calls():
    import torch
    from fastmat_gb300 import _native
    lib = _native.load()
    op, _ = _operator('circulant')
    plan = op.plan(np.complex128)
    per_col = plan.info().scratch_bytes_per_col
    m = STATIC_BYTES // per_col + 1
    n = op.numRows
    xt = torch.zeros((m, n), dtype=torch.complex128, device='cuda')
    yt = torch.zeros_like(xt)
    st = _run(lib.fm_execute_static, plan, 0, xt, yt, m,
              torch.cuda.current_stream().cuda_stream)
    assert st == _native.FM_ERR_VALUE
    assert b'static' in lib.fm_last_error()
