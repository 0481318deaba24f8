"""Plans are cached per (device, compute type) and built with their device
current: a plan's constants live on the device it was built on, so a
tensor on another device must get a plan of its own (no GPU needed: the
native plan is replaced by a recorder)."""

import numpy as np

import fastmat_gb300 as fg
from fastmat_gb300 import _native, matrix


class _FakePlan:
    built_on = []

    def __init__(self, nodes, children, root, code, keep):
        self.code = code
        self.device = matrix._CURRENT[0]
        _FakePlan.built_on.append(self.device)


class _FakeScope:
    def __init__(self, dev):
        self.dev = dev

    def __enter__(self):
        self.prev = matrix._CURRENT[0]
        matrix._CURRENT[0] = self.dev

    def __exit__(self, *exc):
        matrix._CURRENT[0] = self.prev
        return False


def test_plans_are_kept_per_device(monkeypatch):
    monkeypatch.setattr(matrix, '_CURRENT', [0], raising=False)
    monkeypatch.setattr(_native, 'Plan', _FakePlan)
    monkeypatch.setattr(matrix, '_device_scope', _FakeScope)
    monkeypatch.setattr(matrix, '_device_index',
                        lambda d=None: matrix._CURRENT[0] if d is None
                        else int(d))
    _FakePlan.built_on = []
    op = fg.Fourier(16)
    p0 = op.plan(np.complex128)
    p1 = op.plan(np.complex128, device=1)
    p0b = op.plan(np.complex128, device=0)
    assert p0 is p0b and p1 is not p0
    # each plan was built while its own device was current
    assert p0.device == 0 and p1.device == 1
    assert _FakePlan.built_on == [0, 1]
    # the compute type is part of the key too
    p2 = op.plan(np.complex64, device=1)
    assert p2 is not p1 and p2.device == 1
    assert set(op._plans) == {(0, p0.code), (1, p1.code), (1, p2.code)}
