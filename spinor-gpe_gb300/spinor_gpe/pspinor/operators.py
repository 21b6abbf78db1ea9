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


class SepField:
    """A real FP64 field on the (Ny, Nx) grid kept as two 1-D parts,
    value[y, x] = a[x] + b[y]: the separable energy grids and axis-aligned
    coupling/detuning fields of a device-built spinor, which never need the
    full 2-D array on the host.  ``np.asarray`` materialises it."""
    __array_priority__ = 100

    def __init__(self, a, b):
        self.a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        self.b = np.ascontiguousarray(b, dtype=np.float64).ravel()

    @property
    def shape(self):
        return (self.b.size, self.a.size)

    def __array__(self, dtype=None, copy=None):
        arr = self.b[:, None] + self.a[None, :]
        return arr if dtype is None else arr.astype(dtype)

    def min(self):
        return float(self.a.min() + self.b.min())

    def max(self):
        return float(self.a.max() + self.b.max())

    def __add__(self, o):
        if isinstance(o, SepField):
            return SepField(self.a + o.a, self.b + o.b)
        return SepField(self.a + float(o), self.b)

    __radd__ = __add__

    def __sub__(self, o):
        if isinstance(o, SepField):
            return SepField(self.a - o.a, self.b - o.b)
        return SepField(self.a - float(o), self.b)

    def __rsub__(self, o):
        return SepField(float(o) - self.a, -self.b)

    def __neg__(self):
        return SepField(-self.a, -self.b)

    def __mul__(self, o):
        return SepField(self.a * float(o), self.b * float(o))

    __rmul__ = __mul__

    def __truediv__(self, o):
        return SepField(self.a / float(o), self.b / float(o))

    def __pow__(self, k):
        if np.all(self.b == 0):
            return SepField(self.a ** k, self.b)
        if np.all(self.a == 0):
            return SepField(self.a, self.b ** k)
        raise ValueError('a power of a field varying along both axes is not separable')

    def kind(self):
        """'uniform', 'x', 'y' or 'sep'."""
        a_const = bool(np.all(self.a == self.a[0]))
        b_const = bool(np.all(self.b == self.b[0]))
        if a_const and b_const:
            return 'uniform'
        if b_const:
            return 'x'
        if a_const:
            return 'y'
        return 'sep'

    def profile(self):
        """(kind, values) as _axes_profile gives for the materialised field."""
        k = self.kind()
        if k == 'uniform':
            return k, np.array([self.a[0] + self.b[0]])
        if k == 'x':
            return k, self.a + self.b[0]
        if k == 'y':
            return k, self.b + self.a[0]
        return None, None


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
        if isinstance(energy, SepField):
            self.shape = energy.shape
            kind, vals = energy.profile()
            if kind is not None:
                self.kind, self.vals = kind, vals
            else:
                self.kind, self.vals = 'sep', (energy.a.copy(), energy.b.copy())
            return
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

    @classmethod
    def with_y_table(cls, energy, b, ulps=8):
        """The separable decomposition of ``energy`` with the given y-table
        ``b`` (a(x) = energy[0, :] - b[0]), or None when energy[y, x]
        differs from a[x] + b[y] by more than ``ulps`` FP64 ulps of
        max|energy| (the tolerance of ``split_separable``)."""
        e = np.asarray(energy, dtype=np.float64)
        b = np.asarray(b, dtype=np.float64)
        a = e[0, :] - b[0]
        resid = np.abs(e - (a[None, :] + b[:, None]))
        scale = max(float(np.max(np.abs(e))), np.finfo(np.float64).tiny)
        if np.max(resid) > ulps * np.finfo(np.float64).eps * scale:
            return None
        d = cls.__new__(cls)
        d.shape = e.shape
        d.kind, d.vals = 'sep', (a, b)
        return d


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
        if isinstance(values, SepField):
            self.nx = values.shape[1]
            kind, vals = values.profile()
            if kind is not None:
                self.kind, self.vals = kind, vals
                return
            values = np.asarray(values)
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
    if isinstance(k_field, SepField):
        return SepField(np.fft.ifftshift(k_field.a), np.fft.ifftshift(k_field.b))
    return np.fft.ifftshift(np.asarray(k_field))


def as_field(v):
    """A separable field as it is, anything else as an FP64 array."""
    return v if isinstance(v, SepField) else np.asarray(v, dtype=np.float64)


def coupling_energy_spec(coupling, theta, nx):
    """The coupling-energy field (Omega/2) exp(-i theta) as one spec
    (theta = None: no Raman phase), element for element what
    value_op(coupling / 2 * exp(-i theta)) gives, without forming 2-D arrays
    when both factors are constant along an axis."""
    cc = Compressed(coupling)
    if theta is None:
        return cc.apply(lambda w: w / 2 + 0j)
    th = Compressed(theta)
    kinds = {cc.kind, th.kind}
    if kinds <= {'uniform', 'x'} or kinds <= {'uniform', 'y'}:
        kind = 'uniform' if kinds == {'uniform'} else (kinds - {'uniform'}).pop()
        vals = np.asarray(cc.vals / 2 * np.exp(-1.0j * th.vals), dtype=np.complex128)
        return _spec(vals, kind, nx)
    return value_op(np.asarray(coupling) / 2 * np.exp(-1.0j * np.asarray(theta)), nx)


class Prepared:
    """The sub-step inputs decomposed once for both sub-steps: kinetic
    fields in natural order and potentials as ``Decomposition`` objects
    (equal fields share one), coupling and Raman phase as ``Compressed``."""

    def __init__(self, kin_eng_spin, pot_eng_spin, coupling, expon):
        self.kin = self.decompose([natural_order(k) for k in kin_eng_spin])
        self.pot = self.decompose(pot_eng_spin)
        self.coupling = Compressed(as_field(coupling))
        self.expon = (None if expon is None else Compressed(as_field(expon)))

    @staticmethod
    def decompose(fields):
        """Decompositions of two component fields (one shared when equal)."""
        f = [as_field(x) for x in fields]
        d0 = Decomposition(f[0])
        if f[1] is f[0]:
            return [d0, d0]
        if isinstance(f[0], SepField) and isinstance(f[1], SepField):
            same = np.array_equal(f[0].a, f[1].a) and np.array_equal(f[0].b, f[1].b)
        elif isinstance(f[0], SepField) or isinstance(f[1], SepField):
            same = False
        else:
            same = np.array_equal(f[1], f[0])
        if same:
            return [d0, d0]
        d1 = Decomposition(f[1])
        if d0.kind == 'sep' and d1.kind == 'sep' and not isinstance(f[1], SepField):
            # fields that differ by a constant (a uniform detuning) share
            # the first one's y-table, so that the two components' y
            # factors are proportional exactly and not only to rounding of
            # the independent splits (large trap energies at the grid edge
            # leave the independent tables ulps apart)
            d1 = Decomposition.with_y_table(f[1], d0.vals[1]) or d1
        return [d0, d1]


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
