"""Kernel-shape wisdom: the shapes the autotuner picked, per grid.

Every pass of the solver (the row pass along x and the column pass along y)
can run in several kernel shapes (launch configurations with different
points per thread and radix plans; ``sgpe_shape_count`` in
``include/spinor_gb300.h``).  A new plan starts in built-in defaults
measured on GB300; ``TensorPropagator.autotune()`` times every pair of
shapes on the live state and keeps the fastest (``sgpe_autotune``).  The
choices are remembered here per (precision bits, ny, nx) for the rest of the
process, so later propagators of the same grid start in them, and can be
saved to and loaded from a JSON file (like FFTW's wisdom).  When the
environment variable ``SGPE_WISDOM`` names a readable file it is loaded at
import.

Shapes change the rounding of the transforms (every shape meets the parity
tolerances), so a run is reproducible bit for bit only with the same
shapes; the wisdom file records them.

``python -m spinor_gpe.tuning --sides 64 256 512 --dtype 64 --out w.json``
autotunes square grids of those sides on this GPU, prints the step time of
every pair and saves the choices.
"""
import json
import os

_WISDOM = {}


def _key(bits, ny, nx):
    return (int(bits), int(ny), int(nx))


def remember(bits, ny, nx, shapes):
    """Record the (row, column) shapes for a grid."""
    _WISDOM[_key(bits, ny, nx)] = (int(shapes[0]), int(shapes[1]))


def lookup(bits, ny, nx):
    """The remembered (row, column) shapes of a grid, or None."""
    return _WISDOM.get(_key(bits, ny, nx))


def forget():
    """Drop all remembered shapes (new plans take the built-in defaults)."""
    _WISDOM.clear()


def save(path):
    """Write the remembered shapes as JSON."""
    rows = [{'bits': k[0], 'ny': k[1], 'nx': k[2], 'row_shape': v[0],
             'col_shape': v[1]} for k, v in sorted(_WISDOM.items())]
    with open(path, 'w', encoding='utf-8') as f:
        json.dump({'kernel_shapes': rows}, f, indent=1)


def load(path):
    """Merge shapes from a JSON file written by ``save``."""
    with open(path, encoding='utf-8') as f:
        data = json.load(f)
    for r in data.get('kernel_shapes', []):
        remember(r['bits'], r['ny'], r['nx'], (r['row_shape'], r['col_shape']))


def default_steps(ny, nx):
    """Steps per candidate for ``autotune``: about 2e7 grid-point steps,
    between 16 and 256."""
    return int(max(16, min(256, 2e7 // (int(ny) * int(nx)))))


_ENV = os.environ.get('SGPE_WISDOM')
if _ENV and os.path.isfile(_ENV):
    load(_ENV)


def tune_grids(sides, bits=64, time='real', n_steps=None, device='cuda'):
    """Autotune square grids of the given sides on the Raman-dressed
    workload (harmonic trap, Omega = 1, k_L = 3, delta = 0.5; the set-up of
    ``workloads.raman_quench_1024`` scaled to each side) and remember the
    choices.  Returns {side: {(row, col): microseconds per step}}."""
    import tempfile

    from . import workloads
    from .pspinor import pspinor as spin
    from .pspinor import tensor_propagator as tprop
    from .pspinor import tensor_tools as ttools
    out = {}
    for n in sides:
        path = tempfile.mkdtemp(prefix='sgpe_tune_') + '/q/'
        ps = workloads.raman_quench_1024(spin.PSpinor, ttools.fft_2d, path, n=int(n), delta=0.5)
        dt = 1e-3 if time == 'real' else 0.02
        prop = tprop.TensorPropagator(ps, dt, 10, device, time=time, dtype=bits)
        prop.full_steps(2)
        out[int(n)] = prop.autotune(n_steps=n_steps or max(32, default_steps(n, n)))
    return out


def _main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(
        prog='python -m spinor_gpe.tuning',
        description='Autotune the kernel shapes of square grids on this GPU, print the '
                    'step times of every pair and optionally save the choices as wisdom.')
    ap.add_argument('--sides', type=int, nargs='+', default=[32, 64, 128, 256, 512])
    ap.add_argument('--dtype', type=int, choices=(64, 128), default=64)
    ap.add_argument('--time', choices=('real', 'imag'), default='real')
    ap.add_argument('--steps', type=int, default=None, help='steps per candidate')
    ap.add_argument('--out', default=None, help='write the wisdom JSON here')
    a = ap.parse_args(argv)
    # the propagators record their choices in the package's module (under
    # ``python -m`` this file also runs as ``__main__``, a second copy)
    from spinor_gpe import tuning as mod
    res = mod.tune_grids(a.sides, a.dtype, a.time, a.steps)
    for n, times in res.items():
        if not times:
            print(f'complex{a.dtype} {n}x{n} {a.time}: one kernel shape per pass at this side')
            continue
        cells = ', '.join(f'({r},{c}) {us:.1f}' for (r, c), us in sorted(times.items()))
        print(f'complex{a.dtype} {n}x{n} {a.time}: us/step {cells}; kept {mod.lookup(a.dtype, n, n)}')
    if a.out:
        mod.save(a.out)


if __name__ == '__main__':
    _main()
