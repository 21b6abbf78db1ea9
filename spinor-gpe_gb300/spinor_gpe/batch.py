"""Many independent solves stepped together on one GPU.

``PropagatorBatch`` takes ``TensorPropagator`` objects (any mix of grid sizes,
parameters, imaginary/real time and precision on one device) and advances
them all by ``n`` full steps with one native call (``sgpe_batch_steps``):
the solves' steps are captured once as independent branches of a CUDA graph,
so small solves that cannot fill the GPU alone run concurrently.  Each
propagator stays usable on its own (``psik``, ``energy()``, ...).
"""
import itertools

import torch

from .pspinor import _native


class PropagatorBatch:
    """A batch of ``TensorPropagator`` objects advanced together."""

    def __init__(self, propagators, queue=False):
        """``queue=True``: step the solves with one persistent launch fed
        from a device work queue (``sgpe_batch_set_queue``; complex64 solves
        with separable operators, sides 128-1024) instead of grouped
        launches in parallel graph branches."""
        self.propagators = list(propagators)
        if not self.propagators:
            raise ValueError('a batch needs at least one propagator')
        devs = {p._device for p in self.propagators}
        if len(devs) != 1:
            raise ValueError('all propagators of a batch must be on one device')
        self._device = devs.pop()
        self._batch = _native.Batch([p._plan for p in self.propagators])
        self.queue = bool(queue)
        if self.queue:
            self._batch.set_queue(True)

    def check_device(self):
        """Raise ``SgpeError`` if a work-queue wait gave up (synchronous)."""
        self._batch.check_device_status()

    def full_steps(self, n_steps):
        """Advance every solve by ``n_steps`` full Strang steps."""
        self._batch.steps(torch, n_steps, self._device)
        for p in self.propagators:
            p._psik_cache = None

    def autotune(self, n_steps=32, warmup=9, margin=0.02):
        """Kernel shapes for batched stepping, picked by measurement.

        Solves of one precision and grid form a class; each class is stepped
        as a batch of its own in every pair of kernel shapes
        (``sgpe_shape_count``) and its solves take the fastest pair (their
        current pair stays unless another is more than ``margin`` faster).
        A class that runs as one grouped launch can prefer other shapes than
        one solve alone (more blocks per launch favour more points per
        thread).  The states are restored afterwards by reloading each
        solve's psik, so stepping continues as from newly built propagators
        with these shapes.  Returns {(bits, ny, nx): {(row, col): us per
        class step}} for the classes that had a choice."""
        lib = _native.load()
        saved = [[t.clone() for t in p.psik] for p in self.propagators]
        own_shapes = [p.kernel_shapes for p in self.propagators]
        classes = {}
        for p in self.propagators:
            classes.setdefault((p._bits,) + tuple(p._shape), []).append(p)
        out = {}
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        chosen = {}
        try:
            for key, members in classes.items():
                bits, ny, nx = key
                pairs = list(itertools.product(range(lib.sgpe_shape_count(bits, 0, nx)),
                                               range(lib.sgpe_shape_count(bits, 1, ny))))
                if len(pairs) < 2 or any(p.tensor_core_dft for p in members):
                    continue
                own = members[0].kernel_shapes
                times = {}
                for pair in pairs:
                    try:
                        for p in members:
                            p.kernel_shapes = pair
                    except _native.SgpeError:
                        # a column tile of this shape does not divide nx
                        # (the per-plan autotuner skips such pairs too)
                        continue
                    sub = _native.Batch([p._plan for p in members])
                    try:
                        sub.steps(torch, warmup, self._device)
                        stream = torch.cuda.current_stream(self._device)
                        ev0.record(stream)
                        sub.steps(torch, n_steps, self._device)
                        ev1.record(stream)
                        ev1.synchronize()
                    finally:
                        sub.close()
                    times[pair] = 1e3 * ev0.elapsed_time(ev1) / n_steps
                if not times:
                    continue
                best = min(times, key=times.get)
                if own in times and times[own] <= (1.0 + margin) * times[best]:
                    best = own
                for p in members:
                    chosen[id(p)] = best
                out[key] = times
        finally:
            # every solve ends in its chosen (else its own) shapes, with the
            # state it had before tuning
            for p, own, s in zip(self.propagators, own_shapes, saved):
                p.kernel_shapes = chosen.get(id(p), own)
                p.psik = s
        return out

    def grid_points(self):
        """Total grid points of the batch (sum of Nx*Ny)."""
        return sum(p._shape[0] * p._shape[1] for p in self.propagators)

    def close(self):
        self._batch.close()
