"""Seeded synthetic ensembles for the five benchmark configurations.

All draws use ``numpy.random.default_rng(seed)`` in the order written below;
species constants are those of rapt/__init__.py:5-10. Each generator returns a
dict: ``field`` (class name, constructor args), ``params`` (solver options),
``kind`` ("particle" | "gc" | "adaptive"), ``delta`` (scalar or per-tracer)
and the initial state arrays (``pos`` and ``vel`` for particles; ``pos``,
``v``, ``pa`` for guiding centres), plus ``mass`` and ``charge`` per tracer.
"""
import numpy as np

e = 1.602176565e-19
m_pr = 1.672621777e-27
m_el = 9.10938291e-31
c = 299792458.0
Re = 6378137.0
B0 = 3.07e-5
MeV = 1e6


def speed_from_ke(ke_ev, mass):
    """utils.speedfromKE (rapt/utils.py:218-249), vectorised."""
    ke = np.asarray(ke_ev, float) * e
    mc2 = mass * c ** 2
    nr = ke / mc2 < 1e-6
    return np.where(nr, np.sqrt(2 * ke / mass), c * np.sqrt(1 - (mc2 / (mc2 + ke)) ** 2))


def _perp_basis(b):
    """Two unit vectors perpendicular to each row of b (deterministic)."""
    a = np.where(np.abs(b[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    e1 = a - np.sum(a * b, axis=1, keepdims=True) * b
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(b, e1)
    return e1, e2


def _velocity(b, v, alpha, phase):
    e1, e2 = _perp_basis(b)
    return v[:, None] * (np.cos(alpha)[:, None] * b + np.sin(alpha)[:, None] *
                         (np.cos(phase)[:, None] * e1 + np.sin(phase)[:, None] * e2))


def _dipole_bhat(pos, coeff=-3 * B0 * Re ** 3):
    x, y, z = pos.T
    r2 = x * x + y * y + z * z
    B = (coeff / r2 ** 2.5)[:, None] * np.column_stack([x * z, y * z, z * z - r2 / 3])
    return B / np.linalg.norm(B, axis=1, keepdims=True)


def config1(n=256, seed=0):
    """Plain Particle.advance: protons in EarthDipole from (6 Re, 0, 0), KE log-uniform
    0.1-10 MeV, pitch angle uniform 10-80 deg to the local field, gyrophase uniform,
    cyclotronresolution 20, 10 s, rtol = atol = 1e-8."""
    rng = np.random.default_rng(seed)
    ke = 10 ** rng.uniform(np.log10(0.1 * MeV), np.log10(10 * MeV), n)
    alpha = np.deg2rad(rng.uniform(10, 80, n))
    phase = rng.uniform(0, 2 * np.pi, n)
    pos = np.tile([6 * Re, 0.0, 0.0], (n, 1))
    v = speed_from_ke(ke, m_pr)
    vel = _velocity(_dipole_bhat(pos), v, alpha, phase)
    return dict(name="config1", field=("EarthDipole", {}), kind="particle", delta=10.0,
                params=dict(rtol=1e-8, atol=1e-8, cyclotronresolution=20),
                pos=pos, vel=vel, mass=np.full(n, m_pr), charge=np.full(n, e), ke=ke)


def _equatorial(rng, n, lmin, lmax):
    L = rng.uniform(lmin, lmax, n)
    mlt = rng.uniform(0, 24, n)
    phi = np.deg2rad((mlt - 12.0) * 15.0)   # noon (MLT 12) faces +x, the image dipole
    return np.column_stack([L * Re * np.cos(phi), L * Re * np.sin(phi), np.zeros(n)])


def config2(n=65536, seed=0):
    """Plain GuidingCenter.advance: electrons in DoubleDipole (image at x = 20 Re,
    strength 1), equatorial start at L uniform 4-7, MLT uniform 0-24 h, KE
    log-uniform 0.1-10 MeV, equatorial pitch angle uniform 15-85 deg, 100 s with
    GCtimestep 1 s (100 output times), rtol = atol = 1e-8."""
    rng = np.random.default_rng(seed)
    pos = _equatorial(rng, n, 4.0, 7.0)
    ke = 10 ** rng.uniform(np.log10(0.1 * MeV), np.log10(10 * MeV), n)
    pa = rng.uniform(15, 85, n)
    return dict(name="config2", field=("DoubleDipole", {}), kind="gc", delta=100.0,
                params=dict(rtol=1e-8, atol=1e-8, gctimestep=1.0),
                pos=pos, v=speed_from_ke(ke, m_el), pa=pa, mass=np.full(n, m_el), charge=np.full(n, -e), ke=ke)


def gc_bench(n=1048576, seed=0):
    """The 1M guiding-centre ensemble: config2's distributions at n = 2^20."""
    w = config2(n, seed)
    w["name"] = "gc_doubledipole_1M"
    return w


def _isotropic(rng, n):
    u = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - u * u)
    return np.column_stack([s * np.cos(ph), s * np.sin(ph), u])


def config3(n=262144, seed=0):
    """Adaptive protons in a Harris sheet (B0 20 nT, L 0.5 Re, Bn 2 nT, Ey 0.2 mV/m),
    x = y = 0, z uniform +-3 Re, KE log-uniform 1-50 keV, isotropic directions,
    durations log-uniform 1-300 s, GCtimestep 0.5 s, rtol = atol = 1e-8."""
    rng = np.random.default_rng(seed)
    z = rng.uniform(-3 * Re, 3 * Re, n)
    ke = 10 ** rng.uniform(np.log10(1e3), np.log10(50e3), n)
    d = _isotropic(rng, n)
    dur = 10 ** rng.uniform(0, np.log10(300), n)
    pos = np.column_stack([np.zeros(n), np.zeros(n), z])
    vel = speed_from_ke(ke, m_pr)[:, None] * d
    return dict(name="config3", field=("Harris", {}), kind="adaptive", delta=dur,
                params=dict(rtol=1e-8, atol=1e-8, gctimestep=0.5),
                pos=pos, vel=vel, mass=np.full(n, m_pr), charge=np.full(n, e), ke=ke)


def config4(n=1048576, seed=0):
    """Precision: protons and electrons 50/50 in EarthDipole, equatorial L uniform
    3-8 Re, MLT uniform, KE log-uniform 10 keV-10 MeV, isotropic pitch
    (cos alpha uniform), 50 gyro-periods each, rtol = atol = 1e-8."""
    rng = np.random.default_rng(seed)
    pos = _equatorial(rng, n, 3.0, 8.0)
    ke = 10 ** rng.uniform(np.log10(1e4), np.log10(1e7), n)
    alpha = np.arccos(rng.uniform(-1, 1, n))
    phase = rng.uniform(0, 2 * np.pi, n)
    electron = np.arange(n) % 2 == 1
    mass = np.where(electron, m_el, m_pr)
    charge = np.where(electron, -e, e)
    v = speed_from_ke(ke, mass)
    vel = _velocity(_dipole_bhat(pos), v, alpha, phase)
    gamma = 1 / np.sqrt(1 - v * v / c ** 2)
    x, y, z = pos.T
    Bmag = 3 * B0 * Re ** 3 / (x * x + y * y + z * z) ** 1.5 / 3  # equatorial |B| = B0 Re^3 / r^3
    Tc = 2 * np.pi * gamma * mass / Bmag / e
    return dict(name="config4", field=("EarthDipole", {}), kind="particle", delta=50 * Tc,
                params=dict(rtol=1e-8, atol=1e-8, cyclotronresolution=10),
                pos=pos, vel=vel, mass=mass, charge=charge, ke=ke)


def config5(n=1048576, seed=0):
    """Learned: mixed species (50/50) in the compressed dipole
    B0(t) = B0 (1 + 0.1 sin(2 pi t / 60 s)) with its induced E, Adaptive, 200 s,
    equatorial L uniform 3-8 Re, KE log-uniform 10 keV-10 MeV, isotropic pitch,
    GCtimestep 1 s, rtol = atol = 1e-8."""
    rng = np.random.default_rng(seed)
    pos = _equatorial(rng, n, 3.0, 8.0)
    ke = 10 ** rng.uniform(np.log10(1e4), np.log10(1e7), n)
    alpha = np.arccos(rng.uniform(-1, 1, n))
    phase = rng.uniform(0, 2 * np.pi, n)
    electron = np.arange(n) % 2 == 1
    mass = np.where(electron, m_el, m_pr)
    charge = np.where(electron, -e, e)
    vel = _velocity(_dipole_bhat(pos), speed_from_ke(ke, mass), alpha, phase)
    return dict(name="config5", field=("CompressedDipole", {}), kind="adaptive", delta=200.0,
                params=dict(rtol=1e-8, atol=1e-8, gctimestep=1.0),
                pos=pos, vel=vel, mass=mass, charge=charge, ke=ke)


CONFIGS = {"config1": config1, "config2": config2, "config3": config3, "config4": config4,
           "config5": config5, "gc_bench": gc_bench}


def subsample(w, idx):
    """The same workload restricted to tracers ``idx`` (for CPU-oracle checks)."""
    out = dict(w)
    n = len(w["mass"])
    for k, v in w.items():
        if isinstance(v, np.ndarray) and v.shape[:1] == (n,):
            out[k] = v[idx]
    return out


def dipole_grid(nx=241, ny=241, nz=121, half=12.0, halfz=6.0, times=(0.0, 10.0, 20.0)):
    """A gridded field as an MHD code would write it: the Earth's dipole
    B = -B0 Re^3 (3xz, 3yz, 2z^2 - x^2 - y^2) / r^5 scaled by (1 + 0.05 k) in
    snapshot k, with a dawn-dusk E_y = 2e-4 (1 + 0.1 (x/Re - 6)) (1 + 0.25 k) V/m
    and E_x = -1e-5 (y/Re) V/m, on a uniform grid |x|, |y| <= half Re,
    |z| <= halfz Re (default 241 x 241 x 121 nodes, 0.1 Re, three snapshots 10 s
    apart: 1.0 GB of B and E). Returned as a Grid subclass whose parsefile
    serves the snapshots (the reference's recipe for gridded data); static False."""
    from .fields import Grid

    x = np.linspace(-half, half, nx) * Re
    y = np.linspace(-half, half, ny) * Re
    z = np.linspace(-halfz, halfz, nz) * Re

    class _DipoleGrid(Grid):
        def parsefile(self, k):
            X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
            r2 = X * X + Y * Y + Z * Z
            r5 = r2 * r2 * np.sqrt(r2)
            r5[r5 == 0] = np.inf  # the node at the origin: B = 0 there
            cst = -B0 * Re ** 3 * (1.0 + 0.05 * k)
            s = 1.0 + 0.25 * k
            return {"time": float(times[k]), "x": x, "y": y, "z": z,
                    "Bx": cst * 3 * X * Z / r5, "By": cst * 3 * Y * Z / r5, "Bz": cst * (2 * Z * Z - X * X - Y * Y) / r5,
                    "Ex": -1e-5 * (Y / Re) * s, "Ey": 2e-4 * (1 + 0.1 * (X / Re - 6)) * s, "Ez": np.zeros_like(X)}

    g = _DipoleGrid(list(range(len(times))))
    g.static = False
    return g


def gc_grid(n=262144, seed=0):
    """Guiding centres in the gridded dipole (dipole_grid): config 2's
    distributions (electrons, L 4-7 in the equator, KE 0.1-10 MeV, pitch angle
    15-85 deg), GCtimestep 0.5 s, starting at t = 0.5 s (the time-derivative
    stencil reaches t - 1e-3). rtol = atol = 1e-6: at 1e-8 the error control
    rejects most steps at the cell faces, where linear interpolation makes the
    right-hand side's derivatives jump, and three quarters of the tracers exceed
    SciPy's 500 steps per output interval (as they would in the reference)."""
    w = config2(n, seed)
    w["name"] = "gc_grid_262k"
    w["field"] = ("dipole_grid", {})
    w["params"] = dict(rtol=1e-6, atol=1e-6, gctimestep=0.5)
    w["t0"] = 0.5
    return w


def bc_drift(n=65536, seed=0):
    """Bounce centres (BounceCenter): protons in the DoubleDipole field,
    equatorial start at L uniform 4-7, MLT uniform 0-24 h, KE log-uniform
    0.5-5 MeV, equatorial pitch angle uniform 70-88 deg (the range where the
    reference's second-invariant integral runs), BCtimestep 0.1 bounce periods,
    eyegradientstep 0.03 Re, SciPy's default tolerances. mu from the pitch angle
    (gamma^2 m v^2 sin^2(a) / (2 |B|))."""
    rng = np.random.default_rng(seed)
    pos = _equatorial(rng, n, 4.0, 7.0)
    ke = 10 ** rng.uniform(np.log10(0.5 * MeV), np.log10(5 * MeV), n)
    eqpa = rng.uniform(70.0, 88.0, n)
    return dict(name="bc_drift", field=("DoubleDipole", {}), kind="bc", pos=pos, ke=ke, eqpa=eqpa,
                v=speed_from_ke(ke, m_pr), mass=np.full(n, m_pr), charge=np.full(n, e),
                params=dict(rtol=1.49012e-8, atol=1.49012e-8, bctimestep=0.1, eyegradientstep=0.03 * Re))
