"""Synthetic problem set-ups for the split-step solver, built through the
public ``PSpinor`` API.

Every function here takes the ``PSpinor`` class and an ``fft_2d`` callable as
arguments, so the identical recipe can build a problem for this package or
for any object with the spinor-gpe ``PSpinor`` interface
(``spinor_gpe/pspinor/pspinor.py:113-196`` for the constructor,
``:469-501`` ``coupling_setup``, ``:571-575`` the detuning setter,
``:608-625`` ``coupling_uniform``, ``:680-745`` ``seed_vortices``).

The named workloads follow the dimensionless problem statements used for the
solver's measurements:

* ``ground_state_256``   -- 256^2 over [-16,16)^2, g=(1000,995,990), no coupling,
  Thomas-Fermi start with seeded +/-0.01 rad phase noise, imaginary dt=0.02.
* ``raman_quench_1024``  -- 1024^2 over [-32,32)^2, g=(1000,1000,990), Raman
  Omega=1, k_L=3, theta=2 k_L x (non-rotated frame), detuning quenched 0 -> 0.5,
  real dt=1e-3.
* ``vortex_2048``        -- 2048^2 over [-48,48)^2, V=(x^2+1.44 y^2)/2,
  g=(2000,1990,1980), Omega=0.5, k_L=2, 8 seeded +/-1 vortices, imaginary dt=0.01.

Only numpy is used: the set-up runs on the host once per problem, as in the
original package.
"""
import numpy as np


def thomas_fermi_state(ps, g_eff, lam, seed, phase_noise=0.01):
    """Equal-population Thomas-Fermi spinor with seeded per-point phase noise.

    psi_c = sqrt(max(mu - V, 0) / g_eff / 2) * exp(i phi_c),
    mu = sqrt(g_eff * N * lam / pi), phi_c ~ U(-phase_noise, phase_noise),
    for the trap V = (x^2 + lam^2 y^2) / 2 with aspect ``lam``.
    """
    pot = np.asarray(ps.pot_eng, dtype=np.float64)
    mu = np.sqrt(g_eff * ps.atom_num * lam / np.pi)
    profile = np.sqrt(np.maximum(mu - pot, 0.0) / g_eff * 0.5)
    rng = np.random.default_rng(seed)
    phases = [rng.uniform(-phase_noise, phase_noise, size=pot.shape)
              for _ in range(2)]
    return [profile * np.exp(1j * ph) for ph in phases]


def build(spinor_cls, fft_2d, path, *, nx, ny, half_x, half_y, g,
          atom_num=1.0, lam=1.0, omega=None, k_l=None, delta=0.0,
          rot_coupling=False, kin_shift=False, seed=0, phase_noise=0.01,
          vortices=None):
    """Build one problem through the ``PSpinor`` API.

    Parameters mirror the dimensionless problem statement: grid ``nx`` x ``ny``
    over [-half_x, half_x) x [-half_y, half_y), couplings ``g`` = (uu, dd, ud)
    written verbatim to ``g_sc`` (the propagator reads ``g_sc`` as given),
    trap aspect ``lam``, Raman coupling ``omega`` with recoil ``k_l`` (``None``
    leaves the coupling branch off), uniform detuning ``delta``.
    ``vortices`` is ``None`` or ``(positions, windings)`` passed to
    ``seed_vortices``.
    """
    ps = spinor_cls(path, overwrite=True, atom_num=atom_num,
                    mesh_points=(nx, ny), r_sizes=(half_x, half_y))
    ps.g_sc = {'uu': float(g[0]), 'dd': float(g[1]), 'ud': float(g[2])}
    if lam != 1.0:
        ps.pot_eng = 0.5 * (ps.space['x_mesh']**2
                            + (lam * ps.space['y_mesh'])**2)
    if omega is not None:
        ps.coupling_setup(kin_shift=kin_shift)
        if k_l is not None:
            ps.kL_recoil = float(k_l)
        ps.rot_coupling = bool(rot_coupling)
        ps.coupling_uniform(float(omega))
        ps.detuning_uniform(float(delta))
    elif delta:
        ps.detuning_uniform(float(delta))
    g_eff = 0.5 * (g[0] + g[2])
    ps.psi = thomas_fermi_state(ps, g_eff, lam, seed, phase_noise)
    ps.psik = fft_2d(ps.psi, ps.space['dr'])
    if vortices is not None:
        positions, windings = vortices
        ps.seed_vortices(positions, list(windings))
    return ps


def vortex_positions(g, atom_num, lam, n_vort, seed, frac=0.6):
    """Seeded uniform vortex positions within ``frac`` of the Thomas-Fermi
    radius along x, with alternating +/-1 windings."""
    rng = np.random.default_rng(seed)
    g_eff = 0.5 * (g[0] + g[2])
    mu = np.sqrt(g_eff * atom_num * lam / np.pi)
    r_tf = np.sqrt(2 * mu)
    pos = []
    while len(pos) < n_vort:
        x, y = rng.uniform(-frac * r_tf, frac * r_tf, size=2)
        if x * x + y * y < (frac * r_tf)**2:
            pos.append((float(x), float(y)))
    wind = [1 if i % 2 == 0 else -1 for i in range(n_vort)]
    return pos, wind


# Named workloads -------------------------------------------------------

def ground_state_256(spinor_cls, fft_2d, path, n=256, seed=1):
    """Plain imaginary-time ground state (complex128 in its statement)."""
    half = n * 0.125 / 2
    return build(spinor_cls, fft_2d, path, nx=n, ny=n, half_x=half,
                 half_y=half, g=(1000.0, 995.0, 990.0), seed=seed)


def raman_quench_1024(spinor_cls, fft_2d, path, n=1024, seed=2, delta=0.0):
    """Raman-dressed state over [-32,32)^2 (complex64 in its statement)."""
    half = n * 0.0625 / 2
    return build(spinor_cls, fft_2d, path, nx=n, ny=n, half_x=half,
                 half_y=half, g=(1000.0, 1000.0, 990.0), omega=1.0, k_l=3.0,
                 delta=delta, rot_coupling=False, seed=seed)


def vortex_2048(spinor_cls, fft_2d, path, n=2048, seed=3):
    """Anisotropic vortex lattice start over [-48,48)^2."""
    half = n * (96.0 / 2048) / 2
    g = (2000.0, 1990.0, 1980.0)
    vort = vortex_positions(g, 1.0, 1.2, 8, seed + 100)
    return build(spinor_cls, fft_2d, path, nx=n, ny=n, half_x=half,
                 half_y=half, g=g, lam=1.2, omega=0.5, k_l=2.0, seed=seed,
                 vortices=vort)


def batched_uneven(spinor_cls, fft_2d, path, n_solves=96, seed=4,
                   sizes=(128, 192, 256, 384, 512, 768, 1024)):
    """Independent ground-state problems with seeded uneven grids and
    parameters: side N from ``sizes`` with dx = 0.125, trap aspect
    lam ~ U[0.5, 2], g_uu ~ U[100, 2000], g_dd = 0.995 g_uu, g_ud = 0.99 g_uu,
    Omega ~ U[0, 2], delta ~ U[-0.5, 0.5], k_L = 3 (non-rotated frame).
    Returns a list of PSpinor objects."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_solves):
        n = int(rng.choice(sizes))
        lam = float(rng.uniform(0.5, 2.0))
        guu = float(rng.uniform(100.0, 2000.0))
        omega = float(rng.uniform(0.0, 2.0))
        delta = float(rng.uniform(-0.5, 0.5))
        half = n * 0.125 / 2
        out.append(build(spinor_cls, fft_2d, f'{path}solve{i:03d}/', nx=n, ny=n,
                         half_x=half, half_y=half,
                         g=(guu, 0.995 * guu, 0.99 * guu), lam=lam,
                         omega=omega, k_l=3.0, delta=delta,
                         rot_coupling=False, seed=seed * 1000 + i))
    return out


def served_stream(rate=200.0, window=60.0, seed=5, ground_frac=0.7,
                  ground_sizes=(256, 512), quench_size=1024):
    """Seeded request stream: Poisson arrivals at ``rate`` per second over
    ``window`` seconds.  A fraction ``ground_frac`` are imaginary-time ground
    states (side from ``ground_sizes``, dx = 0.125, parameters drawn as in
    ``batched_uneven``, dt = 0.02, stop at |dE| < 1e-8 per step or 3000
    steps); the rest are real-time quenches (side ``quench_size`` over
    [-32, 32)^2, g = (1000, 1000, 990), Omega = 1, k_L = 3, detuning
    0 -> U[0.1, 1], dt = 1e-3, 5000 steps) from the Thomas-Fermi start.
    Returns request descriptions (dicts); ``request_spin`` builds one."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= window:
            return out
        rid = len(out)
        if rng.uniform() < ground_frac:
            n = int(rng.choice(ground_sizes))
            guu = float(rng.uniform(100.0, 2000.0))
            out.append({'rid': rid, 'arrival': t, 'kind': 'ground', 'n': n,
                        'half': n * 0.125 / 2,
                        'g': (guu, 0.995 * guu, 0.99 * guu),
                        'lam': float(rng.uniform(0.5, 2.0)),
                        'omega': float(rng.uniform(0.0, 2.0)),
                        'delta': float(rng.uniform(-0.5, 0.5)),
                        'time': 'imag', 'dt': 0.02, 'max_steps': 3000,
                        'tol': 1e-8, 'seed': seed * 100000 + rid})
        else:
            n = int(quench_size)
            out.append({'rid': rid, 'arrival': t, 'kind': 'quench', 'n': n,
                        'half': n * 0.0625 / 2, 'g': (1000.0, 1000.0, 990.0),
                        'lam': 1.0, 'omega': 1.0,
                        'delta': float(rng.uniform(0.1, 1.0)),
                        'time': 'real', 'dt': 1e-3, 'max_steps': 5000,
                        'tol': None, 'seed': seed * 100000 + rid})


def request_spin(spinor_cls, fft_2d, path, req):
    """The PSpinor of one ``served_stream`` request."""
    return build(spinor_cls, fft_2d, f"{path}req{req['rid']:06d}/",
                 nx=req['n'], ny=req['n'], half_x=req['half'],
                 half_y=req['half'], g=req['g'], lam=req['lam'],
                 omega=req['omega'], k_l=3.0, delta=req['delta'],
                 rot_coupling=False, seed=req['seed'])


def build_device(path, *, nx, ny, half_x, half_y, g, atom_num=1.0, lam=1.0,
                 omega=None, k_l=None, delta=0.0, rot_coupling=False,
                 kin_shift=False, seed=0, phase_noise=0.01, vortices=None,
                 device='cuda', dtype=64):
    """``build`` with the set-up on the GPU (``DeviceSpinor``): separable
    operator fields (O(Nx + Ny) host work) and the Thomas-Fermi state,
    phase noise (a seeded counter hash instead of NumPy's generator) and
    vortices written by native kernels.  Same problem statement as
    ``build``; the state differs from it only through the noise draws."""
    from .pspinor.device_spinor import DeviceSpinor
    from .pspinor import operators as ops
    ps = DeviceSpinor(path, overwrite=True, atom_num=atom_num,
                      mesh_points=(nx, ny), r_sizes=(half_x, half_y),
                      device=device, dtype=dtype)
    ps.g_sc = {'uu': float(g[0]), 'dd': float(g[1]), 'ud': float(g[2])}
    if lam != 1.0:
        ps.pot_eng = ops.SepField(ps.space['x']**2 / 2, (lam * ps.space['y'])**2 / 2)
    if omega is not None:
        ps.coupling_setup(kin_shift=kin_shift)
        if k_l is not None:
            ps.kL_recoil = float(k_l)
        ps.rot_coupling = bool(rot_coupling)
        ps.coupling_uniform(float(omega))
        ps.detuning_uniform(float(delta))
    elif delta:
        ps.detuning_uniform(float(delta))
    g_eff = 0.5 * (g[0] + g[2])
    mu = np.sqrt(g_eff * ps.atom_num * lam / np.pi)
    amp = np.sqrt(0.5 / g_eff)
    ps.set_tf_state(mu, [amp, amp], noise=phase_noise, seed=seed, renorm=False)
    if vortices is not None:
        positions, windings = vortices
        ps.seed_vortices(positions, list(windings))
    return ps


def request_spin_device(path, req, device='cuda', dtype=64):
    """The ``DeviceSpinor`` of one ``served_stream`` request."""
    return build_device(f"{path}req{req['rid']:06d}/", nx=req['n'], ny=req['n'],
                        half_x=req['half'], half_y=req['half'], g=req['g'],
                        lam=req['lam'], omega=req['omega'], k_l=3.0,
                        delta=req['delta'], rot_coupling=False, seed=req['seed'],
                        device=device, dtype=dtype)
