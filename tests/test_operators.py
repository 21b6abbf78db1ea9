"""Host-side operator construction (``spinor_gpe.pspinor.operators``).

The propagator uploads each FP64 operator field in the most compact exact
form: uniform values, x- or y-tables, separable a(x) + b(y) pairs or the full
field.  These tests check each form against the dense field it stands for.
"""
import numpy as np
import pytest

from spinor_gpe.pspinor import operators as ops

NY, NX = 24, 40
Y, X = np.mgrid[0:NY, 0:NX]
XS = (X - NX / 2) * 0.25
YS = (Y - NY / 2) * 0.5


def _eps(field):
    return 8 * np.finfo(np.float64).eps * np.max(np.abs(field))


def test_split_separable_recovers_a_trap():
    v = 0.5 * (XS**2 + 1.44 * YS**2)
    a, b = ops.split_separable(v)
    assert np.max(np.abs(a[None, :] + b[:, None] - v)) <= _eps(v)


def test_split_separable_rejects_a_bump():
    v = np.exp(-(XS**2 + YS**2))
    assert ops.split_separable(v) is None


@pytest.mark.parametrize('field,kind', [
    (np.full((NY, NX), 3.5), 'uniform'),
    (XS**2 + 0 * YS, 'x'),
    (YS**3 + 0 * XS, 'y'),
    (XS**2 + np.sin(YS), 'sep'),
    (XS * YS, 'full'),
])
def test_decomposition_kinds_and_values(field, kind):
    d = ops.Decomposition(field)
    assert d.kind == kind
    a, b = ops.energy_pair(d)
    dense = a.dense(NY, NX).real + b.dense(NY, NX).real
    assert np.max(np.abs(dense - field)) <= _eps(field)


@pytest.mark.parametrize('t', [0.01, -0.02j])
def test_phase_op_product_is_the_operator(t):
    for field in (XS**2 + np.sin(YS), XS * YS, np.full((NY, NX), 2.0)):
        a, b = ops.phase_op(field, t)
        got = a.dense(NY, NX) * b.dense(NY, NX)
        ref = np.exp(-1.0j * field * t)
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_sepfield_matches_its_dense_array():
    f = ops.SepField(np.linspace(-1, 2, NX), np.cos(np.arange(NY)))
    dense = np.asarray(f)
    assert dense.shape == (NY, NX)
    g = (2.0 * f - 1.0) / 4.0 + f
    np.testing.assert_allclose(np.asarray(g), (2.0 * dense - 1.0) / 4.0 + dense, rtol=0, atol=1e-15)
    assert f.min() == pytest.approx(dense.min())
    assert f.max() == pytest.approx(dense.max())
    assert ops.Decomposition(f).kind == 'sep'
    assert ops.SepField(np.arange(NX) * 1.0, np.zeros(NY)).kind() == 'x'
    with pytest.raises(ValueError):
        _ = f ** 2


def test_compressed_apply_matches_the_full_field():
    for field in (XS**2 + 0 * YS, YS + 0 * XS, XS * YS):
        spec = ops.Compressed(field).apply(lambda w: np.exp(0.3j * w))
        np.testing.assert_array_equal(spec.dense(NY, NX), np.exp(0.3j * field))


def test_coupling_energy_spec_matches_dense():
    omega = np.full((NY, NX), 1.5)
    theta = 2 * 3.0 * XS
    spec = ops.coupling_energy_spec(omega, theta, NX)
    assert spec.kind == 'x'
    np.testing.assert_allclose(spec.dense(NY, NX), omega / 2 * np.exp(-1.0j * theta), rtol=0, atol=1e-15)
    spec = ops.coupling_energy_spec(omega, None, NX)
    assert spec.kind == 'uniform'


def test_detuned_components_share_the_y_table():
    """Potentials that differ by a uniform detuning (V + delta/2, V - delta/2)
    share one y-table even where a large trap energy at the grid edge leaves
    independent splits ulps apart, so their y factors are exactly
    proportional; each split still reproduces its field to 8 ulps."""
    x = np.arange(-64.0, 64.0, 0.125)
    X, Y = np.meshgrid(x, x)
    V = 0.5 * (X ** 2 + (1.909 * Y) ** 2)
    pot = [V + 0.43 / 2, V - 0.43 / 2]
    d0, d1 = ops.Prepared([np.zeros_like(V)] * 2, pot, np.zeros_like(V), None).pot
    assert d0.kind == d1.kind == 'sep'
    assert d1.vals[1] is d0.vals[1]
    for d, e in zip((d0, d1), pot):
        a, b = d.vals
        resid = np.abs(e - (a[None, :] + b[:, None]))
        assert resid.max() <= 8 * np.finfo(np.float64).eps * np.abs(e).max()
    p0 = ops.phase_op(d0, 0.008)[1].values
    p1 = ops.phase_op(d1, 0.008)[1].values
    np.testing.assert_array_equal(p0, p1)
    # a field that is not the first plus a constant keeps its own split
    other = 0.5 * (X ** 2 + (1.5 * Y) ** 2)
    e0, e1 = ops.Prepared([np.zeros_like(V)] * 2, [V, other], np.zeros_like(V), None).pot
    assert e1.vals[1] is not e0.vals[1]
