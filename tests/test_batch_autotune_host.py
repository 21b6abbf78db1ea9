"""Host logic of ``PropagatorBatch.autotune`` with fake plans (CPU only).

A kernel-shape pair whose setter fails (a column tile that would not divide
nx) is skipped, and every solve ends in its chosen or original shapes with
its saved psik, also when stepping a candidate raises.
"""
import types

import numpy as np
import pytest

from spinor_gpe import batch as batch_mod
from spinor_gpe.pspinor import _native


class FakeProp:
    """The attributes ``PropagatorBatch`` reads from a ``TensorPropagator``."""

    def __init__(self, shape, bad_pairs=()):
        self._device = 'cuda:0'
        self._bits = 64
        self._shape = shape
        self._plan = types.SimpleNamespace(_h=None)
        self.tensor_core_dft = False
        self._shapes = (0, 0)
        self._bad = set(bad_pairs)
        self._psik = [np.full(shape, 1 + 0j), np.full(shape, 2 + 0j)]
        self.set_calls = []

    @property
    def kernel_shapes(self):
        return self._shapes

    @kernel_shapes.setter
    def kernel_shapes(self, pair):
        pair = tuple(pair)
        self.set_calls.append(pair)
        if pair in self._bad:
            raise _native.SgpeError(_native.SGPE_ERR_ARG, 'column tile does not divide nx')
        self._shapes = pair

    @property
    def psik(self):
        return [FakeTensor(p) for p in self._psik]

    @psik.setter
    def psik(self, value):
        self._psik = [np.asarray(v.a) for v in value]


class FakeTensor:
    def __init__(self, a):
        self.a = np.array(a)

    def clone(self):
        return FakeTensor(self.a.copy())


class FakeEvent:
    clock = [0.0]

    def __init__(self, **_):
        self.t = 0.0

    def record(self, _stream=None):
        self.t = FakeEvent.clock[0]

    def synchronize(self):
        pass

    def elapsed_time(self, other):
        return other.t - self.t


def install_fakes(monkeypatch, cost, fail_on=None):
    """``cost[pair]``: ms a step of that pair takes on the fake clock;
    ``fail_on``: a pair whose stepping raises."""

    class FakeBatch:
        def __init__(self, plans):
            self.members = [p for p in PROPS if p._plan in plans]

        def steps(self, _torch, n, _device):
            pair = self.members[0].kernel_shapes
            if pair == fail_on:
                raise _native.SgpeError(_native.SGPE_ERR_CUDA, 'planted failure')
            for p in self.members:      # stepping changes the state
                p._psik = [x * 1.5 for x in p._psik]
            FakeEvent.clock[0] += cost[pair] * n

        def close(self):
            pass

    lib = types.SimpleNamespace(sgpe_shape_count=lambda bits, axis, n: 3)
    monkeypatch.setattr(_native, 'load', lambda: lib)
    monkeypatch.setattr(_native, 'Batch', FakeBatch)
    fake_cuda = types.SimpleNamespace(Event=FakeEvent, current_stream=lambda _d=None: None)
    monkeypatch.setattr(batch_mod, 'torch', types.SimpleNamespace(cuda=fake_cuda))


PROPS = []


def make_batch(props):
    PROPS[:] = props
    return batch_mod.PropagatorBatch(props)


def test_unusable_pairs_are_skipped_and_states_restored(monkeypatch):
    cost = {(r, c): 10.0 + r + c for r in range(3) for c in range(3)}
    cost[(2, 1)] = 1.0                      # fastest usable pair
    cost[(1, 2)] = 0.5                      # faster still, but its tile does not fit
    props = [FakeProp((32, 64), bad_pairs={(1, 2), (0, 2), (2, 2)}) for _ in range(3)]
    install_fakes(monkeypatch, cost)
    b = make_batch(props)
    before = [[t.a.copy() for t in p.psik] for p in props]
    out = b.autotune(n_steps=4, warmup=1)
    times = out[(64, 32, 64)]
    assert (1, 2) not in times and (0, 2) not in times
    assert set(times) == {(r, c) for r in range(3) for c in range(2)}
    for p, s in zip(props, before):
        assert p.kernel_shapes == (2, 1)
        for a, b0 in zip(p._psik, s):
            np.testing.assert_array_equal(a, b0)


def test_failure_while_stepping_restores_shapes_and_states(monkeypatch):
    cost = {(r, c): 5.0 for r in range(3) for c in range(3)}
    props = [FakeProp((64, 64)) for _ in range(2)]
    for p in props:
        p._shapes = (1, 0)
    install_fakes(monkeypatch, cost, fail_on=(0, 2))
    b = make_batch(props)
    before = [[t.a.copy() for t in p.psik] for p in props]
    with pytest.raises(_native.SgpeError):
        b.autotune(n_steps=2, warmup=1)
    for p, s in zip(props, before):
        assert p.kernel_shapes == (1, 0)     # its own shapes: nothing was chosen
        for a, b0 in zip(p._psik, s):
            np.testing.assert_array_equal(a, b0)
