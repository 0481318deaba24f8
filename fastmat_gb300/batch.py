"""Many operators in one persistent launch.

``Batch([(op, x), ...])`` binds operators of different kinds and sizes to
their right-hand sides (CUDA tensors of shape (n,) or (n, M)) and runs all
of them with ONE cooperative kernel launch (fm_batch_execute): the k-th
launch of every operator's plan forms level k, the CTAs meet at a grid
barrier between levels.  ``run(graph=True)`` captures that launch into a
CUDA graph once and replays it.  fastmat itself applies operators one call
at a time (fastmat/Matrix.pyx:1844-1910); each result here equals what
``op.forward(x)`` (or ``op.backward(x)``) returns.

The operators' plans must share one compute type: complex64 (operators
built with ``precision='fp32'``) or complex128 in double-float arithmetic
(the default precision with complex128 results).
"""

import numpy as np

from . import _native
from .matrix import _fcontig_tensor, _numpy_dtype, _torch_dtype


class Batch:
    """Operators bound to inputs, applied together (see module docstring).

    ``items``: sequence of ``(op, x)`` or ``(op, x, y)``; ``y`` (optional)
    is an output tensor of shape (rows, M) with the operator's output type.
    ``backward=True`` applies every operator's adjoint instead."""

    def __init__(self, items, backward=False):
        import torch
        self._ops, self._xs, self._ys, self._flat = [], [], [], []
        plans, dirs, xp, xt, ldx, yp, yt, ldy, cols = ([] for _ in range(9))
        direction = _native.BACKWARD if backward else _native.FORWARD
        for it in items:
            op, x = it[0], it[1]
            y = it[2] if len(it) > 2 else None
            if not (hasattr(x, 'is_cuda') and x.is_cuda):
                raise TypeError("Batch: inputs must be CUDA tensors")
            n_in = op.numRows if backward else op.numCols
            n_out = op.numCols if backward else op.numRows
            if x.dim() not in (1, 2) or x.shape[0] != n_in:
                raise ValueError("Batch: input shape does not match the "
                                 "operator")
            flat = x.dim() == 1
            xc = _fcontig_tensor(x)
            M = xc.shape[1]
            in_dt = _numpy_dtype(x.dtype)
            out_dt = np.dtype(op._output_dtype(in_dt))
            if y is None:
                y = torch.empty((M, n_out), dtype=_torch_dtype(out_dt),
                                device=x.device).t()
            elif (tuple(y.shape) != (n_out, M) or y.stride(0) != 1 or
                  y.dtype != _torch_dtype(out_dt)):
                raise ValueError("Batch: output must be a column-major "
                                 "(%d, %d) tensor of %s" % (n_out, M,
                                                            out_dt))
            p = op.plan(out_dt)
            plans.append(p)
            dirs.append(direction)
            xp.append(xc.data_ptr())
            xt.append(_native.DTYPE_CODE[in_dt])
            ldx.append(max(xc.stride(1), n_in) if M > 1 else n_in)
            yp.append(y.data_ptr())
            yt.append(_native.DTYPE_CODE[out_dt])
            ldy.append(max(y.stride(1), n_out) if M > 1 else n_out)
            cols.append(M)
            self._ops.append(op)
            self._xs.append(xc)
            self._ys.append(y)
            self._flat.append(flat)
        if not plans:
            raise ValueError("Batch: no operators")
        self._h = _native.BatchHandle(plans, dirs, xp, xt, ldx, yp, yt, ldy,
                                      cols)

    @property
    def outputs(self):
        """The result tensors, in the order of the items."""
        return [y.reshape(-1) if f else y
                for y, f in zip(self._ys, self._flat)]

    def run(self, graph=False, stream=None):
        """Apply every operator (one launch; graph=True: CUDA graph
        replay).  Asynchronous on the current stream."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        self._h.execute(stream, graph)
        return self.outputs

    def check(self):
        """Synchronise and raise if a bounded wait of the launch gave up."""
        self._h.check()

    def set_wait_limit(self, polls):
        """Polls of a grid-barrier wait before the launch gives up and
        reports a timeout (default 2^22; 0: at once).  Set it before the
        first ``run(graph=True)``."""
        self._h.set_wait_limit(polls)

    def info(self):
        """(launches of the separate plans, levels, tiles)."""
        return self._h.info()
