"""Sparse-recovery algorithms that call the matvec path in a loop, kept on
the GPU.

``ISTA`` and ``FISTA`` follow fastmat's (fastmat/algorithms/ISTA.py,
fastmat/algorithms/FISTA.py): the same constructor parameters (``numLambda``,
``numMaxSteps``, ``cbStep``), the same iteration and the same result (the
unthresholded values on the support of the final iterate).  Every
``forward`` / ``backward`` runs on device-resident torch tensors, so an
iteration moves no data between host and device; a numpy right-hand side is
copied to the GPU once and the result copied back once.  The step size
1 / sigma_max(A)^2 comes from ``Matrix.largestSingularValue`` (scipy's
svds over GPU matvecs, as fastmat/Matrix.pyx:895-921).
"""

import numpy as np

from .matrix import Matrix, _torch


class _Iterative:
    def __init__(self, fmatA, **kwargs):
        if not isinstance(fmatA, Matrix):
            raise TypeError("fmatA must be a fastmat matrix")
        self.fmatA = fmatA
        self.numLambda = 0.1
        self.numMaxSteps = 100
        self.cbStep = None
        self.cbTrace = None
        self.updateParameters(**kwargs)

    def updateParameters(self, **kwargs):
        for k, v in kwargs.items():
            setattr(self, k, v)

    def handleCallback(self, cb):
        if cb is not None:
            cb(self)

    @staticmethod
    def softThreshold(arrX, numAlpha):
        """Soft thresholding (fastmat/algorithms/ISTA.py:111-121) on a
        device tensor."""
        torch = _torch()
        arrM = torch.clamp(arrX.abs() - numAlpha, min=0)
        return (arrM / (arrM + numAlpha)) * arrX

    def process(self, arrB):
        """Solve for every column of arrB (numpy array or CUDA tensor; the
        result has the same kind)."""
        torch = _torch()
        host = not hasattr(arrB, 'is_cuda')
        if host:
            b = np.asarray(arrB)
            if b.ndim > 2 or b.ndim < 1:
                raise ValueError("Only n x m arrays are supported")
            dt = np.promote_types(np.float32, b.dtype)
            tb = torch.from_numpy(np.ascontiguousarray(
                b.reshape(b.shape[0], -1).astype(dt).T)).cuda().t()
        else:
            if arrB.dim() > 2 or arrB.dim() < 1:
                raise ValueError("Only n x m arrays are supported")
            tb = arrB if arrB.dim() == 2 else arrB.unsqueeze(1)
        if self.numMaxSteps <= 0:
            raise ValueError("the algorithm needs at least one step")
        flat = (np.ndim(arrB) if host else arrB.dim()) == 1
        res = self._process(tb)
        if flat:
            res = res.reshape(-1)
        if host:
            return np.asfortranarray(res.cpu().numpy())
        return res


class ISTA(_Iterative):
    """Iterative soft thresholding: min ||A x - b||^2 + lambda ||x||_1
    (fastmat/algorithms/ISTA.py:27-160)."""

    def _process(self, arrB):
        torch = _torch()
        A = self.fmatA
        self.numL = 1.0 / (A.largestSingularValue ** 2)
        dt = torch.promote_types(torch.float32, arrB.dtype)
        self.arrX = torch.zeros((arrB.shape[1], A.numCols), dtype=dt,
                                device=arrB.device).t()
        self.arrB = arrB
        for self.numStep in range(self.numMaxSteps):
            r = A.forward(self.arrX) - arrB
            self.arrStep = self.arrX - self.numL * A.backward(r)
            self.arrX = self.softThreshold(
                self.arrStep, self.numL * self.numLambda * 0.5)
            self.handleCallback(self.cbStep)
            self.handleCallback(self.cbTrace)
        self.arrResult = torch.where(self.arrX != 0, self.arrStep, self.arrX)
        return self.arrResult


class FISTA(_Iterative):
    """Fast iterative soft thresholding with Nesterov momentum
    (fastmat/algorithms/FISTA.py:27-180)."""

    def _process(self, arrB):
        torch = _torch()
        A = self.fmatA
        self.numL = 1.0 / (A.largestSingularValue ** 2)
        self.t = 1
        dt = torch.promote_types(torch.float32, arrB.dtype)
        self.arrX = torch.zeros((arrB.shape[1], A.numCols), dtype=dt,
                                device=arrB.device).t()
        self.arrY = self.arrX.clone()
        self.arrB = arrB
        for self.numStep in range(self.numMaxSteps):
            self.arrXold = self.arrX
            r = A.forward(self.arrY) - arrB
            self.arrStep = self.arrY - self.numL * A.backward(r)
            self.arrX = self.softThreshold(
                self.arrStep, self.numL * self.numLambda * 0.5)
            tOld = self.t
            self.t = (1 + np.sqrt(1 + 4 * self.t ** 2)) / 2
            self.arrY = self.arrX + ((tOld - 1) / self.t) * (
                self.arrX - self.arrXold)
            self.handleCallback(self.cbStep)
            self.handleCallback(self.cbTrace)
        return torch.where(self.arrX != 0, self.arrStep, self.arrX)
