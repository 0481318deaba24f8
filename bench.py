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


def run_gpu(args):
    import torch
    rank, world, local = dist_info()
    barrier, allmax = _dist_setup(torch, world, local)
    import fastmat_gb300 as fg
    build_fn, dt64, dt32, desc = WORKLOADS[args.workload]
    op64, M, _ = build_fn(fg, 'native')
    op32, _, _ = build_fn(fg, 'fp32')
    n_in, n_out = op64.numCols, op64.numRows

    peak, peak_kind = measured_peak()
    results = {}
    dev = torch.cuda.current_device()
    uuid = getattr(torch.cuda.get_device_properties(dev), 'uuid', None)
    clocks = ClockSampler('GPU-%s' % uuid if uuid is not None else dev)
    ref_y = None
    for name, op, dt in (('fp64', op64, dt64), ('fp32', op32, dt32)):
        # plan creation includes the autotuner's choice of tile shapes
        if not args.no_autotune:
            op.autotune(M, out_dtype=op._output_dtype(np.dtype(dt)))
        x = make_input(n_in, M, dt, 1000 + rank)
        xt = torch.from_numpy(x.T).cuda().t()  # column-major device tensor
        if name == 'fp64':
            clocks.start()
        ms, yt = time_device(torch, op, xt, args.steps, args.warmup, barrier)
        if name == 'fp64':
            clk = clocks.stop()
        ms = allmax(ms)
        out_dt = np.dtype(op._output_dtype(np.dtype(dt)))
        nbytes = (n_in * M * np.dtype(dt).itemsize +
                  n_out * M * out_dt.itemsize)
        # per-launch timing of the same call (CUDA events between launches)
        plan = op.plan(out_dt)
        code = fg._native.DTYPE_CODE
        launches = []
        for _ in range(max(1, min(args.steps, 5))):
            launches.append(plan.execute_profiled(
                fg._native.FORWARD, xt.data_ptr(), code[np.dtype(dt)], n_in,
                yt.data_ptr(), code[out_dt], n_out, M,
                torch.cuda.current_stream().cuda_stream))
        per_launch = np.mean(np.array(launches), axis=0)
        results[name] = dict(ms=ms, bytes=nbytes, launches=per_launch,
                             n_launch=len(per_launch), out_dt=out_dt, dt=dt,
                             plan=plan, y=yt)
        if name == 'fp64':
            ref_y = yt
    # relative error of the FP32 form against FP64: fresh calls on the same
    # seeded input (rounded to single precision for the FP32 form)
    xe = make_input(n_in, M, dt64, 1000 + rank)
    y64 = op64.forward(torch.from_numpy(xe.T).cuda().t()).cpu().numpy()
    y32 = op32.forward(torch.from_numpy(
        xe.astype(dt32).T).cuda().t()).cpu().numpy()
    rel = float(np.max(np.abs(y32.astype(y64.dtype) - y64)) /
                np.max(np.abs(y64)))
    del y32

    # e2e: host C ABI with pinned host buffers, copies inside the timed region
    e2e = None
    r64 = results['fp64']
    xh = torch.empty((M, n_in), dtype=fg.matrix._torch_dtype(dt64)) \
        .pin_memory()
    xh.numpy()[:] = make_input(n_in, M, dt64, 1000 + rank).T
    yh = torch.empty((M, n_out), dtype=fg.matrix._torch_dtype(
        r64['out_dt'])).pin_memory()
    xa = xh.numpy().T
    ya = yh.numpy().T
    plan64 = r64['plan']
    for _ in range(args.warmup):
        plan64.execute_host(fg._native.FORWARD, xa, ya)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plan64.execute_host(fg._native.FORWARD, xa, ya)
    t1 = time.perf_counter()
    barrier()
    e2e_ms = allmax((t1 - t0) * 1e3 / args.steps)
    e2e = {"value": world * r64['bytes'] / (e2e_ms * 1e-3) / 1e9,
           "unit": "GB/s", "ms_per_step": e2e_ms,
           "h2d_bytes_per_step": int(n_in * M * np.dtype(dt64).itemsize),
           "d2h_bytes_per_step": int(n_out * M * r64['out_dt'].itemsize),
           "path": "fm_execute_host (C ABI), pinned host buffers"}

    def roofline(r, form):
        shares = r['launches'] / r['launches'].sum()
        k = int(np.argmax(r['launches']))
        kern_ms = float(r['launches'][k])
        # every launch of this workload reads X-sized data and writes
        # Y-sized data once; its algorithmic bytes are the step's bytes
        achieved = r['bytes'] / (kern_ms * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic(args.workload, form, k + 1),
                "peak_kind": peak_kind,
                "kernel": "vprog launch %d of %d" % (k + 1, len(shares)),
                "kernel_ms": kern_ms,
                "launch_ms": [round(float(v), 4) for v in r['launches']]}

    r32 = results['fp32']
    line = {
        "metric": "matvec GB/s vs HBM roofline; FP32 vs FP64 GPU speedup at "
                  "rel err <=1e-5",
        "value": world * r64['bytes'] / (r64['ms'] * 1e-3) / 1e9,
        "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r64['ms'],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128" if np.dtype(dt64).kind == 'c' else "f64",
        "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": desc, "columns_per_gpu": M,
                   "parallelism": "replicas over columns (no collective)",
                   "l2": "inputs larger than L2 (%.0f MiB per operand)" %
                         (r64['bytes'] / 2 / 2 ** 20)},
        "fp32_form": {
            "value": world * r32['bytes'] / (r32['ms'] * 1e-3) / 1e9,
            "unit": "GB/s", "ms_per_step": r32['ms'],
            "speedup_vs_fp64": r64['ms'] / r32['ms'],
            "rel_err_vs_fp64": rel, "dtype": "c64",
            "roofline": roofline(r32, 'fp32')},
        "roofline": roofline(r64, 'fp64'),
        "e2e": e2e,
        "gpu_launches": int(args.steps * r64['n_launch']),
        "clocks": clk,
    }
    if args.workload == 'chain':
        line["differentiable"] = measure_grad(torch, fg, args)
    if args.workload == 'hadamard':
        line["bf16_form"] = measure_bf16(torch, fg, args, build_fn, n_in, M,
                                         xe, op64, peak, peak_kind)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def measure_bf16(torch, fg, args, build_fn, n_in, M, xe, op64, peak,
                 peak_kind):
    """The tensor-core form of the Hadamard workload: float32 data, the
    16-point groups as BF16 MMA with FP32 accumulation (three-term split)."""
    op, _, _ = build_fn(fg, 'bf16')
    dt = np.float32
    if not args.no_autotune:
        op.autotune(M, out_dtype=np.float32)
    xt = torch.from_numpy(xe.astype(dt).T).cuda().t()
    ms, yt = time_device(torch, op, xt, args.steps, args.warmup,
                         lambda: None)
    y64 = op64.forward(torch.from_numpy(xe.T).cuda().t()).cpu().numpy()
    rel = float(np.max(np.abs(yt.cpu().numpy().astype(np.float64) - y64)) /
                np.max(np.abs(y64)))
    plan = op.plan(np.float32)
    code = fg._native.DTYPE_CODE
    n_out = op.numRows
    launches = np.mean(np.array([plan.execute_profiled(
        fg._native.FORWARD, xt.data_ptr(), code[np.dtype(dt)], n_in,
        yt.data_ptr(), code[np.dtype(dt)], n_out, M,
        torch.cuda.current_stream().cuda_stream) for _ in range(3)]), axis=0)
    nbytes = (n_in + n_out) * M * 4
    k = int(np.argmax(launches))
    ach = nbytes / (launches[k] * 1e-3) / 1e9
    return {"value": nbytes / (ms * 1e-3) / 1e9, "unit": "GB/s",
            "ms_per_step": ms, "dtype": "f32 data, bf16 x3 MMA, f32 accum",
            "rel_err_vs_fp64": rel,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak,
                         "unit": "GB/s", "frac": ach / peak,
                         "traffic": ncu_traffic(args.workload, 'bf16', k + 1),
                         "peak_kind": peak_kind,
                         "kernel": "vprog launch %d of %d (tensor-core "
                                   "FWHT groups)" % (k + 1, len(launches)),
                         "launch_ms": [round(float(v), 4) for v in launches]}}


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
    """Many operators in one persistent launch (complex64), replayed as a
    CUDA graph, against the plain FP64 path applying them one by one."""
    import torch
    rank, world, local = dist_info()
    barrier, allmax = _dist_setup(torch, world, local)
    import fastmat_gb300 as fg
    specs = batched_specs(seed=rank)
    ops32 = batched_ops(fg, specs, 'fp32')
    ops64 = batched_ops(fg, specs)
    rng = np.random.default_rng(100 + rank)
    xs, xs64 = [], []
    for op, m in ops32:
        x = (rng.standard_normal((m, op.numCols)) +
             1j * rng.standard_normal((m, op.numCols))).astype(np.complex64)
        xs.append(torch.from_numpy(x).cuda().t())
        xs64.append(xs[-1].to(torch.complex128))
    nbytes = sum((op.numCols + op.numRows) * m * 8 for op, m in ops32)
    batch = fg.Batch([(op, x) for (op, _), x in zip(ops32, xs)])
    launches, levels, tiles = batch.info()
    dev = torch.cuda.current_device()
    uuid = getattr(torch.cuda.get_device_properties(dev), 'uuid', None)
    clocks = ClockSampler('GPU-%s' % uuid if uuid is not None else dev)
    for _ in range(args.warmup):
        batch.run(graph=True)
    torch.cuda.synchronize()
    barrier()
    clocks.start()
    ms = _time_events(torch, lambda: batch.run(graph=True), args.steps, 0)
    clk = clocks.stop()
    batch.check()
    ms = allmax(ms)
    ys = [y.clone() for y in batch.outputs]

    def per_op64():
        for (op, _), x in zip(ops64, xs64):
            op.forward(x)

    ms64 = allmax(_time_events(torch, per_op64, 2, 1))
    rel = 0.0
    for (op, _), x, y in zip(ops64, xs64, ys):
        r = op.forward(x)
        rel = max(rel, float((y.to(torch.complex128) - r).abs().max() /
                             r.abs().max()))
    # e2e: pinned host inputs / outputs, copies inside the timed region
    hx = [x.t().contiguous().cpu().pin_memory() for x in xs]
    hy = [torch.empty(tuple(y.t().shape), dtype=y.dtype).pin_memory()
          for y in ys]
    dx = [x.t() for x in xs]            # row-major (M, n) views of the inputs
    dy = [y.t() for y in batch.outputs]

    def e2e_step():
        for h, d in zip(hx, dx):
            d.copy_(h, non_blocking=True)
        batch.run(graph=True)
        for h, d in zip(hy, dy):
            h.copy_(d, non_blocking=True)
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_ms = allmax((time.perf_counter() - t0) * 1e3 / args.steps)
    peak, peak_kind = measured_peak()
    achieved = nbytes / (ms * 1e-3) / 1e9
    h2d = sum(op.numCols * m * 8 for op, m in ops32)
    line = {
        "metric": "matvec GB/s vs HBM roofline; FP32 vs FP64 GPU speedup at "
                  "rel err <=1e-5",
        "value": world * achieved, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": WORKLOADS['batched'][3],
                   "operators": len(ops32),
                   "plan_launches_replaced": launches, "levels": levels,
                   "tiles": tiles,
                   "parallelism": "replicas (each rank its own batch)",
                   "l2": "working set %.0f MiB (larger than L2)" %
                         (nbytes / 2 ** 20)},
        "fp64_per_operator": {"ms_per_step": ms64,
                              "value": world * nbytes * 2 / (ms64 * 1e-3) /
                              1e9,
                              "unit": "GB/s", "dtype": "c128",
                              "speedup_of_batch": ms64 / ms,
                              "rel_err_batch_vs_fp64": rel},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": ncu_traffic('batched', 'fp32', 1),
                     "peak_kind": peak_kind,
                     "kernel": "batch_kernel (one cooperative launch)"},
        "e2e": {"value": world * nbytes / (e2e_ms * 1e-3) / 1e9,
                "unit": "GB/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(nbytes - h2d),
                "path": "pinned host buffers, one copy per operand, graph "
                        "replay of the batch"},
        "gpu_launches": int(args.steps),
        "clocks": clk,
    }
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
