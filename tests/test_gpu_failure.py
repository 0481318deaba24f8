"""Failure paths, exercised without faulting the GPU.

* A bounded device wait that gives up: every wait of the kernels for a tile
  copy (an mbarrier) and the batch's grid barrier polls at most a set number
  of times.  With the limit set to 0 the first wait gives up at once; the
  kernel records FM_ERR_TIMEOUT in the plan's (batch's) status word, waits
  with the default limit for the copies it has in flight and returns.  The
  host sees the status through fm_plan_check / fm_batch_check (RuntimeError
  here), the context stays usable, and with the default limit restored the
  next call is correct.
* A device allocation that fails: the library's one-shot test hook makes a
  chosen cudaMalloc report "out of memory".  The call raises MemoryError
  (fastmat's exception for an allocation failure), frees what it had
  allocated, and the same call succeeds afterwards."""

import numpy as np
import pytest

from oracle import fm_oracle as fo

pytestmark = pytest.mark.gpu


def cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize('expr', ['fourier', 'kron_strided', 'hadamard'])
def test_wait_limit_zero_reports_timeout_then_recovers(expr):
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(5)
    if expr == 'fourier':   # contiguous vectors: bulk copies + mbarrier
        op, oop = fg.Fourier(1024), fo.Fourier(1024)
        dt = np.complex128
        x = cplx(rng, 1024, 64)
    elif expr == 'kron_strided':   # strided mode: TMA boxes + mbarrier
        # complex64 throughout: the loads need no type conversion; 1024
        # points, above the strided register FFT's lengths (which has no
        # spin waits), so the mode runs on element-major TMA tiles
        op = fg.Kron(fg.Fourier(1024), fg.Eye(64), precision='fp32')
        oop = fo.Kron(fo.Fourier(1024), fo.Eye(64))
        dt = np.complex64
        x = cplx(rng, op.numCols, 8).astype(np.complex64)
        assert 'rsfft' not in op.plan(np.complex64).describe(0)
    else:
        # (the register-resident FWHT, which takes orders 10 to 13 on
        # float32, has no spin waits: its copies complete in hardware)
        op, oop = fg.Hadamard(9), fo.Hadamard(9)
        dt = np.float32
        x = rng.standard_normal((512, 64)).astype(np.float32)
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    plan = op.plan(op._output_dtype(x.dtype))
    plan.set_wait_limit(0)
    try:
        op.forward(xt)
        with pytest.raises(RuntimeError, match='bounded wait'):
            plan.check()
    finally:
        plan.set_wait_limit(1 << 22)
    # the status was cleared by the check; the context is usable
    plan.check()
    y = op.forward(xt).cpu().numpy()
    plan.check()
    tol = 1e-12 if np.dtype(dt).itemsize >= 8 and dt != np.complex64 else 1e-5
    assert fo.rel_err(y, oop.forward(x.astype(
        np.complex128 if np.iscomplexobj(x) else np.float64))) <= tol
    with pytest.raises(ValueError):
        plan.set_wait_limit(-1)


def test_fused_fwht_pass_wait_timeout_then_recovers():
    """The fused two-pass FWHT (one launch, second-pass items wait for
    their column's first-pass items): with the poll limit 0 a second-pass
    item that finds its column unfinished gives up at once.  With one
    column the second-pass items are handed out while the last first-pass
    items still run, so a timeout is all but certain within three calls;
    the kernel returns, check() reports it, and with the default limit the
    result is bit-exact again."""
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(8)
    x = rng.standard_normal((1 << 22, 1)).astype(np.float32)
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    op = fg.Hadamard(22)
    plan = op.plan(np.float32)
    assert 'fused-with-next' in plan.describe(0)
    plan.set_wait_limit(0)
    timed_out = False
    try:
        for _ in range(3):
            op.forward(xt)
            try:
                plan.check()
            except RuntimeError as e:
                assert 'bounded wait' in str(e)
                timed_out = True
                break
    finally:
        plan.set_wait_limit(1 << 22)
    assert timed_out
    plan.check()
    y = op.forward(xt).cpu().numpy()
    plan.check()
    ref = fo.Hadamard(22).forward(x)
    assert np.array_equal(y.view(np.uint32), ref.view(np.uint32))


def test_batch_grid_barrier_timeout_then_recovers():
    import torch
    import fastmat_gb300 as fg
    rng = np.random.default_rng(6)
    # long circulants: three launch levels, so two grid barriers
    specs = [(fg.Circulant(cplx(rng, n)), n) for n in (20000, 9000, 300)]
    xs = [torch.from_numpy(cplx(rng, n, 2).astype(np.complex64)).cuda()
          for _, n in specs]
    batch = fg.Batch([(op, x) for (op, _), x in zip(specs, xs)])
    assert batch.info()[1] >= 3
    batch.set_wait_limit(0)
    batch.run()
    with pytest.raises(RuntimeError, match='bounded'):
        batch.check()
    batch.set_wait_limit(1 << 22)
    batch.run()
    batch.check()
    for (op, n), x, y in zip(specs, xs, batch.outputs):
        ref = fo.Circulant(op.tenC).forward(x.cpu().numpy().astype(
            np.complex128))
        assert fo.rel_err(y.cpu().numpy(), ref) <= 1e-12


def test_allocation_failure_during_plan_creation():
    """Every device allocation of a plan's construction (spectrum, twiddles,
    index maps, temporaries of the nested FFT, status word) failing in turn:
    MemoryError each time, no device memory left behind, and the plan builds
    and computes correctly afterwards."""
    import fastmat_gb300 as fg
    from fastmat_gb300 import _native
    _native.load()
    rng = np.random.default_rng(7)
    c = cplx(rng, 20000)
    x = cplx(rng, 20000, 3)
    fg.Circulant(c).forward(x)   # warm: kernels loaded, staging allocated
    before = _free_bytes()
    failed = 0
    for k in range(400):
        op = fg.Circulant(c)
        _native.fail_allocation(k)
        try:
            op.plan(np.complex128)
        except MemoryError as e:
            failed += 1
            assert 'cudaMalloc' in str(e) or 'memory' in str(e).lower()
            continue
        finally:
            _native.fail_allocation(-1)
        break
    else:
        raise AssertionError('plan creation never succeeded')
    assert failed >= 3   # spectrum temporaries, constants, status word
    del op
    import gc
    gc.collect()
    assert _free_bytes() == before
    y = fg.Circulant(c).forward(x)
    assert fo.rel_err(y, fo.Circulant(c).forward(x)) <= 1e-12


def test_allocation_failure_during_execution():
    """The scratch a multi-launch plan grows on its first call with more
    columns fails: MemoryError, then the same call succeeds."""
    import torch
    import fastmat_gb300 as fg
    from fastmat_gb300 import _native
    rng = np.random.default_rng(8)
    c = cplx(rng, 20000)
    op = fg.Circulant(c)
    x = torch.from_numpy(cplx(rng, 3, 20000)).cuda().t()
    op.forward(x[:, :1])          # plan built, scratch for one column
    _native.fail_allocation(0)
    try:
        with pytest.raises(MemoryError):
            op.forward(x)          # needs scratch for three columns
    finally:
        _native.fail_allocation(-1)
    y = op.forward(x).cpu().numpy()
    assert fo.rel_err(y, fo.Circulant(c).forward(x.cpu().numpy())) <= 1e-12


def test_allocation_failure_in_host_staging():
    """fm_execute_host's device staging grows for a larger call and fails:
    MemoryError through the numpy path, then the call succeeds."""
    import fastmat_gb300 as fg
    from fastmat_gb300 import _native
    rng = np.random.default_rng(9)
    n = 1 << 16
    op = fg.Fourier(n)
    op.forward(cplx(rng, n, 1))
    big = cplx(rng, n, 40)
    _native.release_host_staging()   # the next host call allocates it
    _native.fail_allocation(0)
    try:
        with pytest.raises(MemoryError):
            op.forward(big)
    finally:
        _native.fail_allocation(-1)
    y = op.forward(big)
    assert fo.rel_err(y[:, :4], np.fft.fft(big[:, :4], axis=0)) <= 1e-12
