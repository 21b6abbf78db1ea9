"""Host-side construction of the sub-step operators in FP64.

The original pre-computes full (Ny, Nx) complex operator arrays for the two
sub-step durations (``spinor_gpe/pspinor/tensor_propagator.py:138-149``,
built by ``tensor_tools.evolution_op`` ``:546-560`` and
``tensor_tools.coupling_op`` ``:563-591``).  Here each operator is computed in
FP64 and described compactly for the native library:

* an energy field E(x, y) whose FP64 values equal a(x) + b(y) to within a few
  ulps is split, and exp(-i E t) = exp(-i a t) * exp(-i b t) becomes an
  x-table times a y-table (the harmonic trap, the free-particle and
  momentum-shifted kinetic energies, uniform or gradient detunings);
* fields constant along an axis become 1-D tables, constant fields scalars;
* anything else is passed as a full field.

Tables are rounded once to the working precision by the library.  Kinetic
tables are emitted in natural (unshifted) FFT order: the original stores
k-space fields fftshift-centred (``pspinor.py:339-347, 380-381``).
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class FieldSpec:
    """Complex values with broadcast strides: value(x, y) = values[x*sx + y*sy]."""
    values: np.ndarray
    sx: int
    sy: int

    @property
    def kind(self):
        return {(0, 0): 'uniform', (1, 0): 'x', (0, 1): 'y'}.get(
            (self.sx, self.sy), 'full')

    def dense(self, ny, nx):
        """The full (ny, nx) array this spec represents (for tests)."""
        y, x = np.mgrid[0:ny, 0:nx]
        return self.values[x * self.sx + y * self.sy]


@dataclass
class SubstepSpec:
    """Operators of one sub-step, matching ``sgpe_substep_ops``."""
    kin_a: list = field(default_factory=list)
    kin_b: list = field(default_factory=list)
    pot_a: list = field(default_factory=list)
    pot_b: list = field(default_factory=list)
    cpl_c: FieldSpec = None
    cpl_s: FieldSpec = None
    cpl_e: FieldSpec = None
    int_z: complex = 0j


def one():
    return FieldSpec(np.ones(1, dtype=np.complex128), 0, 0)


def _axes_profile(f):
    """('uniform'|'x'|'y'|None, values) for exact constancy along axes."""
    if np.all(f == f.flat[0]):
        return 'uniform', np.array([f.flat[0]])
    if np.all(f == f[0:1, :]):
        return 'x', f[0, :].copy()
    if np.all(f == f[:, 0:1]):
        return 'y', f[:, 0].copy()
    return None, None


def split_separable(e, ulps=8):
    """Return (a, b) with e[y, x] == a[x] + b[y] to within ``ulps`` FP64 ulps
    of max|e|, or None when ``e`` is not separable."""
    e = np.asarray(e, dtype=np.float64)
    a = e[0, :].copy()
    b = e[:, 0] - e[0, 0]
    resid = np.abs(e - (a[None, :] + b[:, None]))
    scale = max(float(np.max(np.abs(e))), np.finfo(np.float64).tiny)
    if np.max(resid) <= ulps * np.finfo(np.float64).eps * scale:
        return a, b
    return None


def _spec(values, kind, nx):
    v = np.asarray(values, dtype=np.complex128).ravel()
    return FieldSpec(v, *{'uniform': (0, 0), 'x': (1, 0), 'y': (0, 1),
                          'full': (1, nx)}[kind])


class Decomposition:
    """A real FP64 field described compactly, found once and reused for
    every operator built from the field: ``kind`` 'uniform' / 'x' / 'y'
    with the values along that axis, 'sep' with tables a(x), b(y)
    (split_separable), or 'full' with the field itself."""

    def __init__(self, energy):
        e = np.asarray(energy, dtype=np.float64)
        self.shape = e.shape
        kind, vals = _axes_profile(e)
        if kind is not None:
            self.kind, self.vals = kind, vals
            return
        sep = split_separable(e)
        if sep is not None:
            self.kind, self.vals = 'sep', sep
        else:
            self.kind, self.vals = 'full', e


def _decomposed(energy):
    return energy if isinstance(energy, Decomposition) else Decomposition(energy)


def phase_op(energy, t):
    """exp(-i E t) for a real FP64 field E (an array or its
    ``Decomposition``) as a pair of specs (a, b) whose product is the
    operator."""
    d = _decomposed(energy)
    nx = d.shape[1]
    if d.kind == 'sep':
        a, b = d.vals
        return (_spec(np.exp(-1.0j * a * t), 'x', nx),
                _spec(np.exp(-1.0j * b * t), 'y', nx))
    return _spec(np.exp(-1.0j * d.vals * t), d.kind, nx), one()


def value_op(values, nx):
    """A complex field as one spec, compressed along constant axes."""
    v = np.asarray(values, dtype=np.complex128)
    kind, vals = _axes_profile(v)
    if kind is None:
        return _spec(v, 'full', nx)
    return _spec(vals, kind, nx)


class Compressed:
    """A field reduced along its constant axes (``_axes_profile``), so that
    element-wise functions are evaluated once per distinct value; ``apply``
    returns the spec of f(field), value for value what f of the full field
    gives."""

    def __init__(self, values):
        v = np.asarray(values)
        self.nx = v.shape[1]
        kind, vals = _axes_profile(v)
        self.kind, self.vals = (kind, vals) if kind is not None else ('full', v)

    def apply(self, fn):
        out = np.asarray(fn(self.vals), dtype=np.complex128)
        if self.kind == 'full':
            return value_op(out, self.nx)
        return _spec(out, self.kind, self.nx)


def zero():
    return FieldSpec(np.zeros(1, dtype=np.complex128), 0, 0)


def energy_pair(energy):
    """A real FP64 energy field (an array or its ``Decomposition``) as two
    specs whose sum is the field: one compressed spec and zero when it is
    constant along an axis, an x-table plus a y-table when it is separable
    (a(x) + b(y) to 8 ulp), else the full field and zero."""
    d = _decomposed(energy)
    nx = d.shape[1]
    if d.kind == 'sep':
        a, b = d.vals
        return _spec(a, 'x', nx), _spec(b, 'y', nx)
    return _spec(d.vals, d.kind, nx), zero()


def natural_order(k_field):
    """Centred (fftshift) k-space field -> natural FFT order."""
    return np.fft.ifftshift(np.asarray(k_field))


class Prepared:
    """The sub-step inputs decomposed once for both sub-steps: kinetic
    fields in natural order and potentials as ``Decomposition`` objects
    (equal fields share one), coupling and Raman phase as ``Compressed``."""

    def __init__(self, kin_eng_spin, pot_eng_spin, coupling, expon):
        self.kin = self.decompose([natural_order(k) for k in kin_eng_spin])
        self.pot = self.decompose(pot_eng_spin)
        self.coupling = Compressed(np.asarray(coupling, dtype=np.float64))
        self.expon = (None if expon is None else
                      Compressed(np.asarray(expon, dtype=np.float64)))

    @staticmethod
    def decompose(fields):
        """Decompositions of two component fields (one shared when equal)."""
        f = [np.asarray(x, dtype=np.float64) for x in fields]
        d0 = Decomposition(f[0])
        if f[1] is f[0] or np.array_equal(f[1], f[0]):
            return [d0, d0]
        return [d0, Decomposition(f[1])]


def build_substep(t_sub, kin_eng_spin, pot_eng_spin, coupling, expon, outer,
                  prepared=None):
    """Operators of one sub-step of duration ``t_sub`` (complex in imaginary
    time).  ``prepared`` (a ``Prepared`` of the same inputs) skips the
    decomposition of the fields.

    kinetic  exp(-i K_c t/2)                 (tensor_propagator.py:138, 144)
    potential exp(-i V_c t)                  (:140, 146)
    coupling  arg = (Omega/2) t / 2 (outer) or Omega (t/2) / 2 (inner);
              [[cos arg, -i sin arg e^{-i expon}], [.. e^{+i expon}, cos arg]]
                                             (:142, 148; tensor_tools.py:586-590)
    interaction exp(-i E_int t/2) = exp(z E_int), z = -i t/2  (:247-249)
    """
    if prepared is None:
        prepared = Prepared(kin_eng_spin, pot_eng_spin, coupling, expon)
    spec = SubstepSpec()
    for c in range(2):
        ka, kb = phase_op(prepared.kin[c], t_sub / 2)
        spec.kin_a.append(ka)
        spec.kin_b.append(kb)
        pa, pb = phase_op(prepared.pot[c], t_sub)
        spec.pot_a.append(pa)
        spec.pot_b.append(pb)
    if outer:
        def arg(omega):
            return (omega / 2) * t_sub / 2
    else:
        def arg(omega):
            return omega * (t_sub / 2) / 2
    spec.cpl_c = prepared.coupling.apply(lambda w: np.cos(arg(w)))
    spec.cpl_s = prepared.coupling.apply(lambda w: -1.0j * np.sin(arg(w)))
    if prepared.expon is None:
        spec.cpl_e = one()
    else:
        spec.cpl_e = prepared.expon.apply(lambda e: np.exp(1.0j * e))
    spec.int_z = -1.0j * t_sub / 2
    return spec
