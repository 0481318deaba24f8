"""Benchmark of the structured-operator matvec path on GB300.

Workload (default): y = Kron(Fourier(256), Hadamard(8), Circulant(c)) x with
c complex128 of length 128 (N = 8,388,608) on X of 8 columns, seeded
synthetic data (iid N(0,1) real and imaginary parts).  A step is one forward
matvec of the 8 columns.

Metric: matvec GB/s = algorithmic bytes (X read once + Y written once) / time
per step.  ``value`` is the FP64 (complex128) drop-in path with inputs
resident in HBM; the FP32 (complex64) form is reported beside it together
with its speedup over FP64 and its relative error against FP64.  ``e2e`` is
the same metric through the host C ABI (fm_execute_host) with pinned host
buffers, so every step includes the host->device copy of X and the
device->host copy of Y.

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W]
                        [--impl gb300|reference] [--workload kron|...]
For N > 1 launch under torch.distributed.run: every rank runs its own
replica on its own 8 columns (the columns are independent, no collective on
the data path); timing is the max over ranks.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GIB = float(1 << 30)
SEED = 1


# ---------------------------------------------------------------- workloads
def workload_kron(fg, precision):
    rng = np.random.default_rng(SEED)
    c = rng.standard_normal(128) + 1j * rng.standard_normal(128)
    op = fg.Kron(fg.Fourier(256), fg.Hadamard(8), fg.Circulant(c),
                 precision=precision)
    return op, 8, c


def workload_hadamard(fg, precision):
    op = fg.Hadamard(22, precision=precision)
    return op, 64, None


def workload_circulant(fg, precision):
    rng = np.random.default_rng(0)
    c = rng.standard_normal(1024) + 1j * rng.standard_normal(1024)
    return fg.Circulant(c, precision=precision), 16, c


def workload_chain(fg, precision):
    rng = np.random.default_rng(3)
    n = 1 << 18
    c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    d = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    rows = np.sort(rng.choice(n, n // 4, replace=False))
    op = fg.Partial(fg.Product(fg.Circulant(c), fg.Diag(d)), rows=rows,
                    precision=precision)
    return op, 32, (c, d, rows)


def _prime_at_most(n):
    def prime(k):
        if k < 2:
            return False
        i = 2
        while i * i <= k:
            if k % i == 0:
                return False
            i += 1
        return True
    while not prime(n):
        n -= 1
    return n


def batched_specs(seed=0, count=512):
    """512 operators: Circulant / Toeplitz / Fourier uniformly, sizes
    log-uniform in [64, 65536], 30% replaced by a prime or a
    non-power-of-two size, the rest rounded to a power of two; 1-32
    right-hand sides each."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        kind = int(rng.integers(0, 3))
        n = int(round(np.exp(rng.uniform(np.log(64), np.log(65536)))))
        if rng.uniform() < 0.3:
            n = (_prime_at_most(n) if rng.uniform() < 0.5
                 else (n | 1) * 3 // 2)
        else:
            n = 1 << int(round(np.log2(n)))
        n = min(max(n, 64), 65536)
        m = int(rng.integers(1, 33))
        if kind == 0:
            vec = (rng.standard_normal(n) + 1j * rng.standard_normal(n),)
        elif kind == 1:
            vec = (rng.standard_normal(n) + 1j * rng.standard_normal(n),
                   rng.standard_normal(n - 1) +
                   1j * rng.standard_normal(n - 1))
        else:
            vec = ()
        specs.append((kind, n, m, vec))
    return specs


def batched_ops(ns, specs, precision=None):
    kw = {} if precision is None else {'precision': precision}
    ops = []
    for kind, n, m, vec in specs:
        if kind == 0:
            ops.append((ns.Circulant(vec[0], **kw), m))
        elif kind == 1:
            ops.append((ns.Toeplitz(vec[0], vec[1], **kw), m))
        else:
            ops.append((ns.Fourier(n, **kw), m))
    return ops


WORKLOADS = {
    'kron': (workload_kron, np.complex128, np.complex64,
             'Kron(Fourier(256), Hadamard(8), Circulant(128)), N=8388608, '
             '8 columns'),
    'hadamard': (workload_hadamard, np.float64, np.float32,
                 'Hadamard(22), N=4194304, 64 columns'),
    'circulant': (workload_circulant, np.complex128, np.complex64,
                  'Circulant(1024), 16 columns'),
    'chain': (workload_chain, np.complex128, np.complex64,
              'Partial(rows N/4) Circulant(c) Diag(d), N=262144, '
              '32 columns'),
    'batched': (None, np.complex128, np.complex64,
                '512 Circulant/Toeplitz/Fourier operators, sizes '
                'log-uniform 64..65536 (30% prime or non-power-of-two), '
                '1-32 columns each'),
}


def input_dtype(name, fp32):
    return WORKLOADS[name][2] if fp32 else WORKLOADS[name][1]


# ---------------------------------------------------------------- helpers
def dist_info():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed
    region."""

    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,'
             'clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index),
                 '--query-gpu=' + self.QUERY, '--format=csv,noheader,nounits',
                 '-lms', '100'], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def ncu_traffic(workload, form, launch):
    """DRAM bytes (read + write) of one launch from the committed ncu
    summary profiles/dram_traffic.txt (lines: workload form launch bytes),
    or None when that launch was not captured."""
    try:
        with open(os.path.join(ROOT, 'profiles', 'dram_traffic.txt')) as f:
            for ln in f:
                t = ln.split()
                if (len(t) >= 4 and not ln.startswith('#') and
                        t[0] == workload and t[1] == form and
                        t[2] == str(launch)):
                    return float(t[3])
    except OSError:
        pass
    return None


def make_input(n, m, dtype, seed):
    rng = np.random.default_rng(seed)
    if np.dtype(dtype).kind == 'c':
        x = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
    else:
        x = rng.standard_normal((n, m))
    return np.asfortranarray(x.astype(dtype))


# ---------------------------------------------------------------- GPU arm
def time_device(torch, op, xt, steps, warmup, barrier):
    """Time `steps` forward matvecs on device-resident data."""
    for _ in range(warmup):
        yt = op.forward(xt)
    torch.cuda.synchronize()
    barrier()
    s = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        yt = op.forward(xt)
    e1.record(s)
    torch.cuda.synchronize()
    barrier()
    return e0.elapsed_time(e1) / steps, yt


def _dist_setup(torch, world, local, backend=None):
    """(barrier, max-over-ranks) for N replicas, no-ops for one.  The
    replicas exchange no data; the process group only times them together
    (NCCL on GPUs, gloo where there is none)."""
    cuda = torch.cuda.is_available()
    if world > 1:
        import torch.distributed as dist
        if cuda:
            torch.cuda.set_device(local)
        dist.init_process_group(backend or ('nccl' if cuda else 'gloo'))
        dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'

        def barrier():
            dist.barrier()

        def allmax(v):
            t = torch.tensor([v], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return barrier, allmax
    if cuda:
        torch.cuda.set_device(0)
    return (lambda: None), (lambda v: v)


_LAUNCH_RE = None


def launch_bytes(plan, n_in, n_out, M, esz_x, esz_y):
    """Algorithmic bytes of every launch of a forward call: the rows of its
    input view read once and the rows of its output view written once, at
    the element size of the buffer each lives in (x, y or scratch in the
    plan's I/O type), times the columns."""
    import re
    global _LAUNCH_RE
    if _LAUNCH_RE is None:
        _LAUNCH_RE = re.compile(
            r'launch src=(\d+) dst=(\d+)(?: in=\((\d+),(\d+),(\d+)\) '
            r'out=\((\d+),(\d+),(\d+)\))?')
    esz_io = {16: 8, 17: 16, 18: 4}.get(plan.compute_type)
    if esz_io is None:
        esz_io = np.dtype(fg_dtype(plan.compute_type)).itemsize
    out = []
    for ln in plan.describe(0).splitlines():
        m = _LAUNCH_RE.match(ln)
        if not m:
            continue
        src, dst = int(m.group(1)), int(m.group(2))
        if m.group(3) is not None:
            rin = int(m.group(3)) * int(m.group(4)) * int(m.group(5))
            rout = int(m.group(6)) * int(m.group(7)) * int(m.group(8))
        else:  # sparse product: its operands' shapes
            rin, rout = n_in, n_out
        rin = min(rin, n_in) if src == 0 else rin
        rout = min(rout, n_out) if dst == 1 else rout
        b_in = rin * (esz_x if src == 0 else esz_y if src == 1 else esz_io)
        b_out = rout * (esz_y if dst == 1 else esz_io)
        out.append(M * (b_in + b_out))
    return out


def fg_dtype(code):
    import fastmat_gb300 as fg
    return fg._native.CODE_DTYPE[code]


def _per_launch(fg, torch, op, xt, yt, dt, out_dt, reps=5):
    plan = op.plan(out_dt)
    code = fg._native.DTYPE_CODE
    runs = [plan.execute_profiled(
        fg._native.FORWARD, xt.data_ptr(), code[np.dtype(dt)], op.numCols,
        yt.data_ptr(), code[out_dt], op.numRows, xt.shape[1],
        torch.cuda.current_stream().cuda_stream) for _ in range(reps)]
    plan.check()
    return plan, np.mean(np.array(runs), axis=0)


def roofline_of(fg, plan, per_launch, n_in, n_out, M, dt, out_dt, peak,
                peak_kind, workload, form, what='vprog'):
    """Roofline of the dominant launch: its algorithmic bytes over its
    CUDA-event time, against the measured copy bandwidth."""
    lb = launch_bytes(plan, n_in, n_out, M, np.dtype(dt).itemsize,
                      np.dtype(out_dt).itemsize)
    if len(lb) != len(per_launch):
        lb = [(n_in * np.dtype(dt).itemsize +
               n_out * np.dtype(out_dt).itemsize) * M] * len(per_launch)
    k = int(np.argmax(per_launch))
    ach = lb[k] / (per_launch[k] * 1e-3) / 1e9
    line = [ln for ln in plan.describe(0).splitlines()
            if ln.startswith('launch')][k]
    if 'rconv' in line and 'fused-with-next' in line:
        kernel = 'rkch (circulant and Hadamard modes, one launch)'
    elif 'rconv' in line:
        kernel = 'rconv'
    elif 'fused-with-next' in line:
        kernel = 'rfwht2 (both FWHT passes, one launch)'
    elif 'rfwht' in line:
        kernel = 'rfwht' if 'stride=1 ' in line else 'rsfwht'
    elif 'rsfft' in line:
        kernel = 'rsfft'
    else:
        kernel = what
    return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind,
            "traffic": ncu_traffic(workload, form, k + 1),
            "kernel": "%s launch %d of %d" % (kernel, k + 1,
                                              len(per_launch)),
            "kernel_ms": float(per_launch[k]),
            "kernel_bytes": int(lb[k]),
            "launch_ms": [round(float(v), 4) for v in per_launch]}


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a.astype(np.complex128) - b)) /
                 np.max(np.abs(b)))


def measure_form(torch, fg, name, prec, dt, M, args, barrier, allmax, peak,
                 peak_kind, seed, form, clocks=None, x=None):
    """One form of one workload: CUDA-event step time on device-resident
    data, per-launch times, roofline of the dominant launch."""
    build_fn = WORKLOADS[name][0]
    op, _, _ = build_fn(fg, prec)
    out_dt = np.dtype(op._output_dtype(np.dtype(dt)))
    if not args.no_autotune:
        op.autotune(M, out_dtype=out_dt)
    if x is None:
        x = make_input(op.numCols, M, dt, seed)
    xt = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().t()
    if clocks is not None:
        clocks.start()
    ms, yt = time_device(torch, op, xt, args.steps, args.warmup, barrier)
    clk = clocks.stop() if clocks is not None else None
    ms = allmax(ms)
    nbytes = (op.numCols * np.dtype(dt).itemsize +
              op.numRows * out_dt.itemsize) * M
    plan, per_launch = _per_launch(fg, torch, op, xt, yt, dt, out_dt)
    return dict(op=op, x=x, xt=xt, y=yt, ms=ms, bytes=nbytes, clk=clk,
                plan=plan, per_launch=per_launch, out_dt=out_dt,
                n_launch=len(per_launch),
                roofline=roofline_of(fg, plan, per_launch, op.numCols,
                                     op.numRows, M, dt, out_dt, peak,
                                     peak_kind, name, form))


def _oracle_columns(name, x, cols):
    """The oracle's forward on selected columns of x (float64 / complex128
    unless the input is single precision)."""
    op, _ = _oracle_workload(name)
    return op.forward(np.asfortranarray(x[:, cols]))


def summarize(r, world):
    return {"ms_per_step": r['ms'],
            "value": world * r['bytes'] / (r['ms'] * 1e-3) / 1e9,
            "unit": "GB/s", "roofline": r['roofline']}


def config_circulant(torch, fg, args, ctx):
    """cfg: Circulant(1024) on 16 columns, FP64 drop-in and FP32 form."""
    M = 16
    r64 = measure_form(torch, fg, 'circulant', 'native', np.complex128, M,
                       args, *ctx, seed=0, form='fp64')
    r32 = measure_form(torch, fg, 'circulant', 'fp32', np.complex64, M,
                       args, *ctx, seed=0, form='fp32')
    ref = _oracle_columns('circulant', r64['x'], list(range(M)))
    out = summarize(r64, 1)
    out.update({
        "workload": WORKLOADS['circulant'][3], "dtype": "c128 I/O, "
        "double-float arithmetic (~2^-48)",
        "note": "launch-bound (0.5 MiB of operands per step)",
        "rel_err_vs_oracle": rel_err(r64['y'].cpu().numpy(), ref),
        "oracle_sample": "all %d columns" % M,
        "fp32_form": dict(summarize(r32, 1),
                          rel_err_vs_oracle=rel_err(r32['y'].cpu().numpy(),
                                                    ref))})
    out["gpu_launches_per_step"] = r64['n_launch']
    return out


def config_hadamard(torch, fg, args, ctx):
    """cfg: Hadamard(22) on 64 float32 columns: FP64 (double-float), FP32
    (butterflies in fastmat's order: bit-exact to its float32 result) and
    BF16 tensor-core forms."""
    from oracle import fm_oracle as fo
    M = 64
    x32 = make_input(1 << 22, M, np.float32, 3)
    r32 = measure_form(torch, fg, 'hadamard', 'fp32', np.float32, M, args,
                       *ctx, seed=3, form='fp32', x=x32)
    rbf = measure_form(torch, fg, 'hadamard', 'bf16', np.float32, M, args,
                       *ctx, seed=3, form='bf16', x=x32)
    y32 = r32.pop('y').cpu().numpy()
    ybf = rbf.pop('y').cpu().numpy()
    for r in (r32, rbf):
        del r['xt']
    torch.cuda.empty_cache()
    r64 = measure_form(torch, fg, 'hadamard', 'native', np.float64, M, args,
                       *ctx, seed=3, form='fp64', x=x32.astype(np.float64))
    y64 = r64['y'].cpu().numpy()
    cols = [0, M - 1]
    H = fo.Hadamard(22)
    ref = H.forward(x32[:, cols].astype(np.float64))
    ref32 = H.forward(np.asfortranarray(x32[:, cols]))
    out = summarize(r64, 1)
    out.update({
        "workload": WORKLOADS['hadamard'][3],
        "dtype": "f64 I/O, double-float arithmetic (~2^-48)",
        "rel_err_vs_oracle": rel_err(y64[:, cols], ref),
        "oracle_sample": "columns %s" % cols,
        "fp32_form": dict(summarize(r32, 1), dtype="f32",
                          speedup_vs_fp64=r64['ms'] / r32['ms'],
                          rel_err_vs_oracle=rel_err(y32[:, cols], ref),
                          bit_exact_vs_float32_oracle=bool(
                              np.array_equal(y32[:, cols], ref32))),
        "bf16_form": dict(summarize(rbf, 1),
                          dtype="f32 data, bf16 x3 MMA, f32 accumulation",
                          rel_err_vs_oracle=rel_err(ybf[:, cols], ref))})
    del r64, y64
    torch.cuda.empty_cache()
    return out


def config_chain(torch, fg, args, ctx):
    """cfg: Partial(rows) Circulant Diag, N = 2^18, 32 columns: fused
    forward (FP64 and FP32) and the differentiable form (complex64)."""
    M = 32
    r64 = measure_form(torch, fg, 'chain', 'native', np.complex128, M,
                       args, *ctx, seed=4, form='fp64')
    r32 = measure_form(torch, fg, 'chain', 'fp32', np.complex64, M, args,
                       *ctx, seed=4, form='fp32')
    cols = [0, 1]
    ref = _oracle_columns('chain', r64['x'], cols)
    out = summarize(r64, 1)
    out.update({
        "workload": WORKLOADS['chain'][3],
        "dtype": "c128 I/O, double-float arithmetic (~2^-48)",
        "rel_err_vs_oracle": rel_err(r64['y'].cpu().numpy()[:, cols], ref),
        "oracle_sample": "columns %s" % cols,
        "fp32_form": dict(summarize(r32, 1),
                          rel_err_vs_oracle=rel_err(
                              r32['y'].cpu().numpy()[:, cols], ref)),
        "differentiable": measure_grad(torch, fg, args)})
    return out


def config_batched(torch, fg, args, ctx):
    """cfg: 512 operators in one persistent launch (complex64, CUDA graph)
    against the FP64 path applied operator by operator."""
    from oracle import fm_oracle as fo
    _, _, peak, peak_kind = ctx
    specs = batched_specs(seed=0)
    ops32 = batched_ops(fg, specs, 'fp32')
    rng = np.random.default_rng(100)
    xs = []
    for op, m in ops32:
        x = (rng.standard_normal((m, op.numCols)) +
             1j * rng.standard_normal((m, op.numCols))).astype(np.complex64)
        xs.append(torch.from_numpy(x).cuda().t())
    nbytes = sum((op.numCols + op.numRows) * m * 8 for op, m in ops32)
    batch = fg.Batch([(op, x) for (op, _), x in zip(ops32, xs)])
    launches, levels, tiles = batch.info()
    ms = _time_events(torch, lambda: batch.run(graph=True), args.steps,
                      args.warmup)
    batch.check()
    ys = batch.outputs
    ops64 = batched_ops(fg, specs)

    def per_op64():
        for (op, _), x in zip(ops64, xs):
            op.forward(x)

    ms64 = _time_events(torch, per_op64, 2, 1)
    # oracle on a sample: every 16th operator with all its columns
    sample = list(range(0, len(specs), 16))
    oops = batched_ops(fo, specs)
    err = 0.0
    for i in sample:
        x = xs[i].cpu().numpy().astype(np.complex128)
        err = max(err, rel_err(ys[i].cpu().numpy(), oops[i][0].forward(x)))
    ach = nbytes / (ms * 1e-3) / 1e9
    return {"workload": WORKLOADS['batched'][3], "dtype": "c64",
            "ms_per_step": ms, "value": ach, "unit": "GB/s",
            "operators": len(ops32), "plan_launches_replaced": launches,
            "levels": levels, "tiles": tiles,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak,
                         "unit": "GB/s", "frac": ach / peak,
                         "peak_kind": peak_kind,
                         "traffic": ncu_traffic('batched', 'fp32', 1),
                         "kernel": "batch_kernel (one cooperative launch)"},
            "rel_err_vs_oracle": err,
            "oracle_sample": "%d of %d operators (every 16th), all their "
                             "columns" % (len(sample), len(specs)),
            "fp64_per_operator": {"ms_per_step": ms64,
                                  "speedup_of_batch": ms64 / ms}}


def e2e_class_api(torch, fg, op, dt, M, args, barrier, allmax, seed):
    """The drop-in call a user makes, op.forward(ndarray), on a page-locked
    host input: every step copies X to the device and Y back (the pipelined
    host entry point fm_execute_host); the result array is page-locked
    memory reused from torch's caching host allocator after warm-up."""
    n_in = op.numCols
    xh = torch.empty((M, n_in), dtype=fg.matrix._torch_dtype(dt)) \
        .pin_memory()
    xh.numpy()[:] = make_input(n_in, M, dt, seed).T
    xa = xh.numpy().T
    for _ in range(args.warmup):
        y = op.forward(xa)
    del y
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        y = op.forward(xa)
    t1 = time.perf_counter()
    barrier()
    return allmax((t1 - t0) * 1e3 / args.steps), xa, y


def run_gpu(args):
    import torch
    rank, world, local = dist_info()
    barrier, allmax = _dist_setup(torch, world, local)
    import fastmat_gb300 as fg
    name = args.workload
    build_fn, dt64, dt32, desc = WORKLOADS[name]
    _, M, _ = build_fn(fg, 'native')
    peak, peak_kind = measured_peak()
    ctx = (barrier, allmax, peak, peak_kind)
    dev = torch.cuda.current_device()
    uuid = getattr(torch.cuda.get_device_properties(dev), 'uuid', None)
    clocks = ClockSampler('GPU-%s' % uuid if uuid is not None else dev)
    seed = 1000 + rank
    r64 = measure_form(torch, fg, name, 'native', dt64, M, args, *ctx,
                       seed=seed, form='fp64', clocks=clocks)
    r32 = measure_form(torch, fg, name, 'fp32', dt32, M, args, *ctx,
                       seed=seed, form='fp32')
    # accuracy: both forms against the oracle on column 0 (the FP32 form's
    # input is the same data rounded to single precision)
    y64 = r64['y'][:, 0].cpu().numpy()
    y32 = r32['y'][:, 0].cpu().numpy()
    ref = _oracle_columns(name, r64['x'], [0])[:, 0]
    rel64, rel32 = rel_err(y64, ref), rel_err(y32, ref)
    rel32_64 = rel_err(y32, y64)
    for r in (r64, r32):
        del r['xt'], r['y']
    torch.cuda.empty_cache()

    # e2e through the class API and through the C ABI, pinned host buffers
    op64 = r64['op']
    e2e_ms, xa, ya = e2e_class_api(torch, fg, op64, dt64, M, args, barrier,
                                   allmax, seed)
    yc = torch.empty((M, op64.numRows),
                     dtype=fg.matrix._torch_dtype(r64['out_dt'])) \
        .pin_memory().numpy().T
    for _ in range(args.warmup):
        r64['plan'].execute_host(fg._native.FORWARD, xa, yc)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r64['plan'].execute_host(fg._native.FORWARD, xa, yc)
    cabi_ms = allmax((time.perf_counter() - t0) * 1e3 / args.steps)
    assert np.array_equal(ya, yc)
    del xa, ya, yc
    e2e = {"value": world * r64['bytes'] / (e2e_ms * 1e-3) / 1e9,
           "unit": "GB/s", "ms_per_step": e2e_ms,
           "h2d_bytes_per_step": int(op64.numCols * M *
                                     np.dtype(dt64).itemsize),
           "d2h_bytes_per_step": int(op64.numRows * M *
                                     r64['out_dt'].itemsize),
           "path": "class API %s.forward(ndarray) on a page-locked input "
                   "(fm_execute_host pipeline: column chunks over copy-in, "
                   "compute and copy-out streams)" % type(op64).__name__,
           "c_abi_fm_execute_host": {
               "ms_per_step": cabi_ms,
               "value": world * r64['bytes'] / (cabi_ms * 1e-3) / 1e9}}

    line = {
        "metric": "matvec GB/s vs HBM roofline; FP32 vs FP64 GPU speedup at "
                  "rel err <=1e-5",
        "value": world * r64['bytes'] / (r64['ms'] * 1e-3) / 1e9,
        "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r64['ms'],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("c128" if np.dtype(dt64).kind == 'c' else "f64") +
                 " (I/O; double-float arithmetic on the FP32 pipes, "
                 "~2^-48 relative)",
        "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": desc, "columns_per_gpu": M,
                   "parallelism": "replicas over columns (no collective)",
                   "l2": "inputs larger than L2 (%.0f MiB per operand)" %
                         (r64['bytes'] / 2 / 2 ** 20)},
        "rel_err_vs_oracle": rel64,
        "oracle_sample": "column 0",
        "fp32_form": {
            "value": world * r32['bytes'] / (r32['ms'] * 1e-3) / 1e9,
            "unit": "GB/s", "ms_per_step": r32['ms'],
            "speedup_vs_fp64": r64['ms'] / r32['ms'],
            "rel_err_vs_oracle": rel32, "rel_err_vs_fp64": rel32_64,
            "dtype": "c64" if np.dtype(dt64).kind == 'c' else "f32",
            "roofline": r32['roofline']},
        "roofline": r64['roofline'],
        "e2e": e2e,
        "gpu_launches": int(args.steps * r64['n_launch']),
        "clocks": r64['clk'],
    }
    if name == 'chain':
        line["differentiable"] = measure_grad(torch, fg, args)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(name)
    if name == 'kron' and not args.only and world == 1:
        del r64, r32
        torch.cuda.empty_cache()
        configs = {}
        for key, fn, cpu in (('circulant', config_circulant, 'circulant'),
                             ('hadamard', config_hadamard, 'hadamard'),
                             ('chain', config_chain, 'chain'),
                             ('batched', config_batched, 'batched')):
            configs[key] = fn(torch, fg, args, ctx)
            if not args.no_cpu_baseline:
                configs[key]["cpu_baseline"] = cpu_baseline(cpu,
                                                            budget_s=3.0)
            torch.cuda.empty_cache()
        line["configs"] = configs
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _time_events(torch, fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def measure_grad(torch, fg, args):
    """The differentiable form of the chain (complex64): forward, and
    forward + backward of ||y - b||^2 with gradients for x, c and d."""
    from fastmat_gb300 import autograd as fa
    op, M, _ = workload_chain(fg, 'fp32')
    n = op.numCols
    x = torch.from_numpy(make_input(n, M, np.complex64, 11).T).cuda().t()
    b = torch.from_numpy(make_input(op.numRows, M, np.complex64, 12).T) \
        .cuda().t()
    mod = fa.Operator(op)
    xg = x.clone().requires_grad_(True)

    def fwd():
        with torch.no_grad():
            mod(x)

    def fwd_bwd():
        loss = (mod(xg) - b).abs().pow(2).sum()
        loss.backward()

    def fused():
        op.forward(x)

    t_fused = _time_events(torch, fused, args.steps, args.warmup)
    t_fwd = _time_events(torch, fwd, args.steps, args.warmup)
    t_fb = _time_events(torch, fwd_bwd, args.steps, args.warmup)
    return {"dtype": "c64", "grads": ["x", "c", "d"],
            "fused_forward_ms": t_fused, "forward_ms": t_fwd,
            "forward_backward_ms": t_fb,
            "ratio_vs_forward": t_fb / t_fwd,
            "ratio_vs_fused_forward": t_fb / t_fused}


def run_batched(args):
    """The batched configuration alone (its own JSON line)."""
    import torch
    rank, world, local = dist_info()
    barrier, allmax = _dist_setup(torch, world, local)
    import fastmat_gb300 as fg
    peak, peak_kind = measured_peak()
    dev = torch.cuda.current_device()
    uuid = getattr(torch.cuda.get_device_properties(dev), 'uuid', None)
    clocks = ClockSampler('GPU-%s' % uuid if uuid is not None else dev)
    clocks.start()
    r = config_batched(torch, fg, args, (barrier, allmax, peak, peak_kind))
    clk = clocks.stop()
    line = {
        "metric": "matvec GB/s vs HBM roofline; FP32 vs FP64 GPU speedup at "
                  "rel err <=1e-5",
        "value": world * r['value'], "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r['ms_per_step'], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": r['workload'], "operators": r['operators']},
        "roofline": r['roofline'], "gpu_launches": int(args.steps),
        "clocks": clk, "batched": r}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline('batched')
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------- CPU arms
def _oracle_workload(name):
    from oracle import fm_oracle as fo
    if name == 'kron':
        rng = np.random.default_rng(SEED)
        c = rng.standard_normal(128) + 1j * rng.standard_normal(128)
        return fo.Kron(fo.Fourier(256), fo.Hadamard(8), fo.Circulant(c)), 8
    if name == 'hadamard':
        return fo.Hadamard(22), 64
    if name == 'circulant':
        rng = np.random.default_rng(0)
        c = rng.standard_normal(1024) + 1j * rng.standard_normal(1024)
        return fo.Circulant(c), 16
    rng = np.random.default_rng(3)
    n = 1 << 18
    c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    d = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    rows = np.sort(rng.choice(n, n // 4, replace=False))
    return fo.Partial(fo.Product(fo.Circulant(c), fo.Diag(d)), rows=rows), 32


def _column_bytes(op, dt_in, dt_out):
    return (op.shape[1] * np.dtype(dt_in).itemsize +
            op.shape[0] * np.dtype(dt_out).itemsize)


def cpu_baseline(name, columns=1, budget_s=10.0):
    """The oracle (numpy restatement of fastmat's CPU path) on a bounded
    sample of the workload, single thread: `columns` columns, repeated for
    about `budget_s` seconds (batched: the operators in order, all their
    columns, until the budget is used)."""
    if name == 'batched':
        from oracle import fm_oracle as fo
        ops = batched_ops(fo, batched_specs(seed=0))
        rng = np.random.default_rng(7)
        t0 = time.perf_counter()
        nbytes, done = 0, 0
        for op, m in ops:
            x = (rng.standard_normal((op.shape[1], m)) +
                 1j * rng.standard_normal((op.shape[1], m)))
            x = x.astype(np.complex64)
            y = op.forward(x)
            nbytes += x.nbytes + m * op.shape[0] * 8
            done += 1
            if time.perf_counter() - t0 > budget_s:
                break
        dt = time.perf_counter() - t0
        return {"value": nbytes / dt / 1e9, "unit": "GB/s", "cores": 1,
                "kind": "port",
                "sample": "first %d of %d operators of the batch with all "
                          "their columns, one at a time, %.1f s" % (
                              done, len(ops), dt)}
    op, M = _oracle_workload(name)
    dt_in = WORKLOADS[name][1]
    x = make_input(op.shape[1], columns, dt_in, 7)
    op.forward(x)  # warm-up
    t0 = time.perf_counter()
    reps = 0
    while True:
        y = op.forward(x)
        reps += 1
        if time.perf_counter() - t0 > budget_s or reps >= 50:
            break
    dt = (time.perf_counter() - t0) / reps
    nbytes = columns * _column_bytes(op, dt_in, y.dtype)
    return {"value": nbytes / dt / 1e9, "unit": "GB/s", "cores": 1,
            "kind": "port",
            "sample": "%d of %d columns of the workload, %d rep(s), "
                      "%.3f s per call" % (columns, M, reps, dt)}


_REF = {}


def _ref_init(name):
    """Pool initializer: build the oracle operator and one seeded input
    column per worker process (outside the timed region)."""
    op, _ = _oracle_workload(name)
    _REF['op'] = op
    _REF['x'] = make_input(op.shape[1], 1, WORKLOADS[name][1], 100)
    op.forward(_REF['x'])


def _ref_init_batched():
    from oracle import fm_oracle as fo
    ops = batched_ops(fo, batched_specs(seed=0))
    rng = np.random.default_rng(100)
    _REF['ops'] = [(op, (rng.standard_normal((op.shape[1], m)) +
                         1j * rng.standard_normal((op.shape[1], m)))
                    .astype(np.complex64)) for op, m in ops]


def _ref_worker_batched(i):
    op, x = _REF['ops'][i]
    op.forward(x)
    return i


def _run_reference_batched(args):
    import multiprocessing as mp
    specs = batched_specs(seed=0)
    cores = os.cpu_count() or 1
    ctx = mp.get_context('spawn')
    # largest operators first so that the pool's tail stays short
    order = sorted(range(len(specs)), key=lambda i: -specs[i][1] *
                   specs[i][2])
    with ctx.Pool(cores, initializer=_ref_init_batched) as pool:
        times = []
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_ref_worker_batched, order, chunksize=1)
            if step >= args.warmup:
                times.append(time.perf_counter() - t0)
    nbytes = sum(2 * n * m * 8 for _, n, m, _ in specs)
    ms = 1e3 * statistics.mean(times)
    value = nbytes / (ms * 1e-3) / 1e9
    print(json.dumps({
        "impl": "reference",
        "metric": "matvec GB/s vs HBM roofline; FP32 vs FP64 GPU speedup at "
                  "rel err <=1e-5",
        "value": value, "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": WORKLOADS['batched'][3],
                   "operators": len(specs)},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": cores,
                         "kind": "port",
                         "sample": "all %d operators per step, one operator "
                                   "per pool task" % len(specs)},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


def _ref_worker(reps):
    op, x = _REF['op'], _REF['x']
    for _ in range(reps):
        op.forward(x)
    return reps


def run_reference(args):
    """Reference arm: the oracle port of fastmat's CPU path on the host
    cores, columns processed in parallel by a spawn-started process pool."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    if args.workload == 'batched':
        return _run_reference_batched(args)
    import multiprocessing as mp
    op, M = _oracle_workload(args.workload)
    dt_in = WORKLOADS[args.workload][1]
    cores = min(M, os.cpu_count() or 1)
    ctx = mp.get_context('spawn')
    with ctx.Pool(cores, initializer=_ref_init,
                  initargs=(args.workload,)) as pool:
        times = []
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_ref_worker, [1] * M, chunksize=1)
            if step >= args.warmup:
                times.append(time.perf_counter() - t0)
    out_dt = np.complex128 if np.dtype(dt_in).kind == 'c' else np.float64
    nbytes = M * _column_bytes(op, dt_in, out_dt)
    ms = 1e3 * statistics.mean(times)
    value = nbytes / (ms * 1e-3) / 1e9
    desc = WORKLOADS[args.workload][3]
    print(json.dumps({
        "impl": "reference",
        "metric": "matvec GB/s vs HBM roofline; FP32 vs FP64 GPU speedup at "
                  "rel err <=1e-5",
        "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128" if np.dtype(dt_in).kind == 'c' else "f64",
        "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": desc, "columns_per_gpu": M},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": cores,
                         "kind": "port",
                         "sample": "all %d columns per step, one column per "
                                   "worker process (step time includes "
                                   "process-pool dispatch)" % M},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


def profile_target(args):
    """Small case of a workload for profilers: forward twice on a few
    columns (inputs still larger than L2 for the long workloads)."""
    import torch
    import fastmat_gb300 as fg
    torch.cuda.set_device(0)
    if args.workload == 'batched':
        # the first COLS operators of the batch, complex64, one launch
        ops = batched_ops(fg, batched_specs(seed=0)[:args.profile_target],
                          'fp32')
        xs = [torch.randn(m, op.numCols, dtype=torch.complex64,
                          device='cuda').t() for op, m in ops]
        b = fg.Batch([(op, x) for (op, _), x in zip(ops, xs)])
        for _ in range(2):
            b.run()
        b.check()
        print(json.dumps({"profile_target": "batched",
                          "operators": len(ops), "info": b.info()}))
        return
    build_fn, dt64, dt32, _ = WORKLOADS[args.workload]
    prec = {'fp32': 'fp32', 'bf16': 'bf16'}.get(args.form, 'native')
    op, M, _ = build_fn(fg, prec)
    dt = dt64 if args.form == 'fp64' else dt32
    if not args.no_autotune:
        op.autotune(M, out_dtype=op._output_dtype(np.dtype(dt)))
    x = make_input(op.numCols, args.profile_target, dt, 5)
    xt = torch.from_numpy(x.T).cuda().t()
    for _ in range(2):
        y = op.forward(xt)
    torch.cuda.synchronize()
    op.plan(np.dtype(op._output_dtype(np.dtype(dt)))).check()
    print(json.dumps({"profile_target": args.workload, "form": args.form,
                      "columns": args.profile_target,
                      "launches_per_call": op.plan(np.dtype(
                          op._output_dtype(np.dtype(dt)))).num_launches(0),
                      "shape": list(y.shape)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default='kron', choices=sorted(WORKLOADS))
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-autotune', action='store_true')
    ap.add_argument('--only', action='store_true',
                    help='the chosen workload alone (the default kron run '
                         'also measures the other configurations)')
    ap.add_argument('--profile-target', type=int, default=0, metavar='COLS',
                    help='no timing: run the workload forward twice on COLS '
                         'columns with the tile shapes tuned for the full '
                         'column count (a small case for ncu captures)')
    ap.add_argument('--form', default='fp64',
                    choices=['fp64', 'fp32', 'bf16'],
                    help='form run by --profile-target')
    args = ap.parse_args()
    if args.profile_target:
        return profile_target(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == 'reference':
        run_reference(args)
    elif args.workload == 'batched':
        run_batched(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
