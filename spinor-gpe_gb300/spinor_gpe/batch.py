"""Many independent solves stepped together on one GPU.

``PropagatorBatch`` takes ``TensorPropagator`` objects (any mix of grid sizes,
parameters, imaginary/real time and precision on one device) and advances
them all by ``n`` full steps with one native call (``sgpe_batch_steps``):
the solves' steps are captured once as independent branches of a CUDA graph,
so small solves that cannot fill the GPU alone run concurrently.  Each
propagator stays usable on its own (``psik``, ``energy()``, ...).
"""
import torch

from .pspinor import _native


class PropagatorBatch:
    """A batch of ``TensorPropagator`` objects advanced together."""

    def __init__(self, propagators):
        self.propagators = list(propagators)
        if not self.propagators:
            raise ValueError('a batch needs at least one propagator')
        devs = {p._device for p in self.propagators}
        if len(devs) != 1:
            raise ValueError('all propagators of a batch must be on one device')
        self._device = devs.pop()
        self._batch = _native.Batch([p._plan for p in self.propagators])

    def full_steps(self, n_steps):
        """Advance every solve by ``n_steps`` full Strang steps."""
        self._batch.steps(torch, n_steps, self._device)
        for p in self.propagators:
            p._psik_cache = None

    def grid_points(self):
        """Total grid points of the batch (sum of Nx*Ny)."""
        return sum(p._shape[0] * p._shape[1] for p in self.propagators)

    def close(self):
        self._batch.close()
