"""ctypes wrapper around the CPU oracle (oracle/librapt_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``, always as the checker or the timed CPU
baseline, never as part of the product path.

The oracle restates RAPT's hot path (rapt/fields.py, rapt/Particle.py,
rapt/GuidingCenter.py, rapt/Adaptive.py, rapt/utils.py, rapt/rkf.py and the
SciPy ``ode`` dopri5/dop853 drivers the reference calls). Its agreement with the
reference itself is pinned by tests/test_oracle.py against fixtures written by
tests/golden/make_golden.py.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librapt_oracle.so")

FIELD_IDS = {
    "EarthDipole": 0, "DoubleDipole": 1, "UniformBz": 2, "UniformCrossedEB": 3,
    "VarEarthDipole": 4, "Parabolic": 5, "Harris": 6, "CompressedDipole": 7, "Grid": 8,
}

ST = dict(OK=0, MAXSTEPS=2, HMIN=3, NONFINITE=4, GC_NOCONV=5, ROWS_FULL=6, BAD_INPUT=7,
          RKF_HMIN=8, ADAPTIVE_LIMIT=9, FIELDLINE=10, OUT_OF_GRID=11)


class Field(C.Structure):
    _fields_ = [("model", C.c_int), ("is_static", C.c_int), ("p", C.c_double * 8),
                ("gradstep", C.c_double), ("timestep", C.c_double),
                ("gt", C.POINTER(C.c_double)), ("gx", C.POINTER(C.c_double)), ("gy", C.POINTER(C.c_double)),
                ("gz", C.POINTER(C.c_double)), ("gB", C.POINTER(C.c_double)), ("gE", C.POINTER(C.c_double)),
                ("nt", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int)]


class Config(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("cycres", C.c_double),
                ("gctimestep", C.c_double), ("epss", C.c_double), ("epst", C.c_double),
                ("enforce_equatorial", C.c_int), ("tableau", C.c_int), ("gc_eom", C.c_int),
                ("nsteps", C.c_int), ("rkf_tol", C.c_double), ("rkf_hmin", C.c_double),
                ("bounceres", C.c_double), ("flres", C.c_double), ("bounce_quad", C.c_int), ("dense", C.c_int)]


TRACER_DTYPE = np.dtype([
    ("mode", "i4"), ("status", "i4"), ("t", "f8"), ("s", "f8", 6), ("mu", "f8"), ("v", "f8"),
    ("mass", "f8"), ("charge", "f8"), ("tcur", "f8"), ("naccept", "i8"), ("nreject", "i8"),
    ("nfcn", "i8"), ("nstep", "i8")], align=True)


class Tracer(C.Structure):
    _fields_ = [("mode", C.c_int), ("status", C.c_int), ("t", C.c_double), ("s", C.c_double * 6),
                ("mu", C.c_double), ("v", C.c_double), ("mass", C.c_double),
                ("charge", C.c_double), ("tcur", C.c_double), ("naccept", C.c_int64),
                ("nreject", C.c_int64), ("nfcn", C.c_int64), ("nstep", C.c_int64)]


assert C.sizeof(Tracer) == TRACER_DTYPE.itemsize

_lib = None
_P = C.POINTER
_d = C.c_double
_dp = _P(C.c_double)


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        F, Cf, T = _P(Field), _P(Config), _P(Tracer)
        sig = {
            "orc_field_init": (None, [F, C.c_int, _dp, C.c_int]),
            "orc_config_default": (None, [Cf]),
            "orc_B": (None, [F, _dp, _dp]), "orc_E": (None, [F, _dp, _dp]),
            "orc_magB": (_d, [F, _dp]), "orc_unitb": (None, [F, _dp, _dp]),
            "orc_gradB": (None, [F, _dp, _dp]), "orc_jacobianB": (None, [F, _dp, _dp]),
            "orc_curvature": (_d, [F, _dp]), "orc_curlb": (None, [F, _dp, _dp]),
            "orc_dBdt": (_d, [F, _dp]), "orc_dbdt": (None, [F, _dp, _dp]),
            "orc_lengthscale": (_d, [F, _dp]), "orc_timescale": (_d, [F, _dp]),
            "orc_particle_rhs": (None, [F, Cf, _d, _d, _d, _d, _dp, _dp]),
            "orc_gc_rhs": (None, [F, Cf, C.c_int, _d, _d, _d, _d, _d, _dp, _dp]),
            "orc_integrate_particle": (C.c_int, [F, Cf, C.c_int, _d, _d, _d, _dp, _dp, _d, _d,
                                                 _P(C.c_int64)]),
            "orc_integrate_gc": (C.c_int, [F, Cf, C.c_int, _d, _d, _d, _d, _dp, _dp, _d,
                                           _P(C.c_int64)]),
            "orc_particle_new": (None, [_dp, _dp, _d, _d, _d, T]),
            "orc_gc_new_pa": (None, [F, _dp, _d, _d, _d, _d, _d, T]),
            "orc_guidingcenter": (C.c_int, [F, _d, _dp, _dp, _d, _d, _dp, _dp, _dp]),
            "orc_gctofp": (None, [F, _d, _dp, _d, _d, _d, _d, _d, _dp, _dp]),
            "orc_gc_from_particle": (C.c_int, [F, T, T]),
            "orc_particle_from_gc": (None, [F, T, T]),
            "orc_particle_isadiabatic": (C.c_int, [F, Cf, T]),
            "orc_gc_isadiabatic": (C.c_int, [F, Cf, T]),
            "orc_particle_advance": (C.c_int, [F, Cf, T, _d, C.c_int, _dp, C.c_int, _P(C.c_int)]),
            "orc_gc_advance": (C.c_int, [F, Cf, T, _d, C.c_int, _dp, C.c_int, _P(C.c_int)]),
            "orc_adaptive_init": (C.c_int, [F, Cf, _dp, _dp, _d, _d, _d, T]),
            "orc_adaptive_advance": (C.c_int, [F, Cf, T, _d, _dp, _P(C.c_int8), C.c_int,
                                               _P(C.c_int), _dp, _P(C.c_int8), C.c_int,
                                               _P(C.c_int)]),
            "orc_batch_advance": (None, [F, Cf, C.c_int, C.c_int64, C.c_void_p, _dp, C.c_int]),
            "orc_gc_bounceperiod": (_d, [F, T, _d, C.c_int]),
            "orc_halfbouncepath": (_d, [F, _dp, _d, _d, C.c_int, _P(C.c_int)]),
            "orc_fieldline_sB": (C.c_int, [F, _dp, _d, _d, _dp, _dp, C.c_int]),
            "orc_qags_test": (_d, [C.c_int, _d, _d, _d, _d, C.c_int, _P(C.c_int)]),
            "orc_eye": (_d, [F, _dp, _d, _d, C.c_int]),
            "orc_gradI": (None, [F, _dp, _d, _d, _d, C.c_int, _dp]),
            "orc_bc_mu": (_d, [F, _dp, _d, _d, _d, _d]),
            "orc_bc_rhs": (None, [F, _dp, _d, _d, _d, _d, _d, _d, C.c_int, _dp]),
            "orc_bc_advance": (C.c_int, [F, Cf, _dp, _d, _d, _d, _d, _d, _d, _d, C.c_int, _dp, C.c_int,
                                         _P(C.c_int), _P(C.c_int64)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _vec(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None:
        assert a.size == n
    return a, a.ctypes.data_as(_dp)


def field(name_or_id, params=()):
    """Build an oracle field struct; ``params`` override the model defaults in order."""
    mid = FIELD_IDS[name_or_id] if isinstance(name_or_id, str) else int(name_or_id)
    f = Field()
    p = np.ascontiguousarray(params, dtype=np.float64)
    lib().orc_field_init(C.byref(f), mid, p.ctypes.data_as(_dp), len(p))
    return f


def grid_field(t, x, y, z, B, E=None, static=True):
    """Oracle Grid field (rapt/fields.py:513-814) over snapshots at times t on the
    axes x, y, z; B, E: [nt][nx][ny][nz][3]. The struct keeps the arrays alive."""
    f = field("Grid")
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (t, x, y, z, B)]
    arrs.append(None if E is None else np.ascontiguousarray(E, dtype=np.float64))
    nt, nx, ny, nz = (len(a) for a in arrs[:4])
    for a in arrs[4:]:
        assert a is None or a.shape == (nt, nx, ny, nz, 3), a.shape
    f._keep = arrs
    f.gt, f.gx, f.gy, f.gz, f.gB = (a.ctypes.data_as(_dp) for a in arrs[:5])
    f.gE = arrs[5].ctypes.data_as(_dp) if arrs[5] is not None else None
    f.nt, f.nx, f.ny, f.nz = nt, nx, ny, nz
    f.is_static = 1 if static else 0
    return f


def config(rtol=1.49012e-8, atol=1.49012e-8, cycres=10, gctimestep=0.0, epss=5e-2, epst=5e-2,
           enforce_equatorial=False, tableau=0, gc_eom=0, nsteps=500, rkf_tol=1e-3,
           rkf_hmin=1e-12, bounceres=10, flres=50, bounce_quad=0, dense=0):
    c = Config()
    lib().orc_config_default(C.byref(c))
    c.bounceres, c.flres, c.bounce_quad, c.dense = bounceres, flres, bounce_quad, int(dense)
    c.rtol, c.atol, c.cycres, c.gctimestep = rtol, atol, cycres, gctimestep
    c.epss, c.epst, c.enforce_equatorial = epss, epst, int(bool(enforce_equatorial))
    c.tableau, c.gc_eom, c.nsteps, c.rkf_tol, c.rkf_hmin = tableau, gc_eom, nsteps, rkf_tol, rkf_hmin
    return c


def field_eval(f, what, tpos):
    """Evaluate one _Field quantity at a (t,x,y,z) point."""
    L = lib()
    tp, ptp = _vec(tpos, 4)
    if what in ("magB", "curvature", "dBdt", "lengthscale", "timescale"):
        return getattr(L, "orc_" + what)(C.byref(f), ptp)
    n = 9 if what == "jacobianB" else 3
    out = np.zeros(n)
    getattr(L, "orc_" + what)(C.byref(f), ptp, out.ctypes.data_as(_dp))
    return out.reshape(3, 3) if n == 9 else out


def particle_rhs(f, cfg, mass, charge, gm, t, Y):
    Y, pY = _vec(Y, 6)
    out = np.zeros(6)
    lib().orc_particle_rhs(C.byref(f), C.byref(cfg), mass, charge, gm, t, pY, out.ctypes.data_as(_dp))
    return out


def gc_rhs(f, cfg, mass, charge, mu, v, t, Y, eom=0):
    Y, pY = _vec(Y, 4)
    out = np.zeros(4)
    lib().orc_gc_rhs(C.byref(f), C.byref(cfg), eom, mass, charge, mu, v, t, pY,
                     out.ctypes.data_as(_dp))
    return out


def particle_new(pos, vel, t0, mass, charge):
    tr = Tracer()
    p, pp = _vec(pos, 3)
    v, pv = _vec(vel, 3)
    lib().orc_particle_new(pp, pv, t0, mass, charge, C.byref(tr))
    return tr


def gc_new_pa(f, pos, v, pa, t0, mass, charge):
    tr = Tracer()
    p, pp = _vec(pos, 3)
    lib().orc_gc_new_pa(C.byref(f), pp, v, pa, t0, mass, charge, C.byref(tr))
    return tr


def tracer_to_dict(tr):
    return {k: (list(getattr(tr, k)) if k == "s" else getattr(tr, k)) for k, _ in Tracer._fields_}


def advance(f, cfg, tr, delta, check=False, max_rows=100000):
    """Advance one Particle/GC tracer; returns (raised, rows[n,7])."""
    rows = np.zeros((max_rows, 7))
    n = C.c_int(0)
    fn = lib().orc_particle_advance if tr.mode == 0 else lib().orc_gc_advance
    raised = fn(C.byref(f), C.byref(cfg), C.byref(tr), delta, int(check),
                rows.ctypes.data_as(_dp), max_rows, C.byref(n))
    return raised, rows[: min(n.value, max_rows)].copy()


def adaptive_init(f, cfg, pos, vel, t0, mass, charge):
    tr = Tracer()
    p, pp = _vec(pos, 3)
    v, pv = _vec(vel, 3)
    lib().orc_adaptive_init(C.byref(f), C.byref(cfg), pp, pv, t0, mass, charge, C.byref(tr))
    return tr


def adaptive_advance(f, cfg, tr, delta, max_rows=200000, max_sw=10000):
    rows = np.zeros((max_rows, 7))
    rmode = np.zeros(max_rows, dtype=np.int8)
    swt = np.zeros(max_sw)
    swm = np.zeros(max_sw, dtype=np.int8)
    n, ns = C.c_int(0), C.c_int(0)
    rc = lib().orc_adaptive_advance(
        C.byref(f), C.byref(cfg), C.byref(tr), delta, rows.ctypes.data_as(_dp),
        rmode.ctypes.data_as(_P(C.c_int8)), max_rows, C.byref(n), swt.ctypes.data_as(_dp),
        swm.ctypes.data_as(_P(C.c_int8)), max_sw, C.byref(ns))
    k, m = min(n.value, max_rows), min(ns.value, max_sw)
    return rc, rows[:k].copy(), rmode[:k].copy(), swt[:m].copy(), swm[:m].copy()


def batch_advance(f, cfg, kind, tracers, delta, nthreads=None):
    """Advance a structured array of TRACER_DTYPE in place (kind 0 P, 1 GC, 2 Adaptive)."""
    assert tracers.dtype == TRACER_DTYPE and tracers.flags.c_contiguous
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(delta, np.float64), tracers.shape))
    nthreads = nthreads or os.cpu_count()
    lib().orc_batch_advance(C.byref(f), C.byref(cfg), kind, tracers.size, tracers.ctypes.data,
                            d.ctypes.data_as(_dp), nthreads)
    return tracers


def tracers_from_structs(structs):
    arr = np.zeros(len(structs), dtype=TRACER_DTYPE)
    for i, s in enumerate(structs):
        C.memmove(arr[i:i + 1].ctypes.data, C.byref(s), C.sizeof(Tracer))
    return arr


def halfbouncepath(f, tpos, Bm, flres=50.0, quad=0):
    """flutils.halfbouncepath (rapt/flutils.py:254-316); returns (S_b, points kept).
    quad 0: QAGS as the reference; 1: the converged integral of the same spline."""
    t, tp = _vec(tpos, 4)
    n = C.c_int(0)
    return lib().orc_halfbouncepath(C.byref(f), tp, float(Bm), float(flres), int(quad), C.byref(n)), n.value


def gc_bounceperiod(f, tr, flres=50.0, quad=0):
    """GuidingCenter.bounceperiod (rapt/GuidingCenter.py:593-606) of a GC tracer struct."""
    return lib().orc_gc_bounceperiod(C.byref(f), C.byref(tr), float(flres), int(quad))


def fieldline_sB(f, tpos, Bm, flres=50.0, cap=100000):
    """(s, |B|) samples of Fieldline(tpos, field, Bmax=Bm).trace() (rapt/fieldline.py)."""
    t, tp = _vec(tpos, 4)
    s = np.zeros(cap)
    b = np.zeros(cap)
    n = lib().orc_fieldline_sB(C.byref(f), tp, float(Bm), float(flres), s.ctypes.data_as(_dp),
                               b.ctypes.data_as(_dp), cap)
    return s[:n], b[:n]


def qags_test(which, a, b, epsabs=1.49e-8, epsrel=1.49e-8, limit=50):
    """QUADPACK QAGS restatement on test integrand `which`; returns (result, ier)."""
    ier = C.c_int(0)
    r = lib().orc_qags_test(int(which), float(a), float(b), float(epsabs), float(epsrel), int(limit), C.byref(ier))
    return r, ier.value


def eye(f, tpos, Bm, flres=50.0, quad=0):
    """flutils.eye: NaN where the reference raises."""
    tp, ptp = _vec(tpos, 4)
    return lib().orc_eye(C.byref(f), ptp, float(Bm), float(flres), int(quad))


def gradI(f, tpos, Bm, d, flres=50.0, quad=0):
    tp, ptp = _vec(tpos, 4)
    out = np.zeros(3)
    lib().orc_gradI(C.byref(f), ptp, float(Bm), float(d), float(flres), int(quad), out.ctypes.data_as(_dp))
    return out


def bc_mu(f, pos, v, pa, t0, mass):
    p, pp = _vec(pos, 3)
    return lib().orc_bc_mu(C.byref(f), pp, float(v), float(pa), float(t0), float(mass))


def bc_rhs(f, tpos, mass, charge, v, Bm, d, flres=50.0, quad=0):
    tp, ptp = _vec(tpos, 4)
    out = np.zeros(3)
    lib().orc_bc_rhs(C.byref(f), ptp, float(mass), float(charge), float(v), float(Bm), float(d), float(flres),
                     int(quad), out.ctypes.data_as(_dp))
    return out


def bc_advance(f, cfg, state, v, mu, mass, charge, delta, bctimestep, d, quad=0, max_rows=10000):
    """BounceCenter.advance; state = (t, x, y, z, tcur) updated in place.
    Returns (status, rows[n, 4], counters[4])."""
    st = np.ascontiguousarray(state, dtype=np.float64)
    assert st.size == 5
    rows = np.zeros((max_rows, 7))
    n = C.c_int(0)
    cnt = np.zeros(4, np.int64)
    status = lib().orc_bc_advance(C.byref(f), C.byref(cfg), st.ctypes.data_as(_dp), float(v), float(mu),
                                  float(mass), float(charge), float(delta), float(bctimestep), float(d), int(quad),
                                  rows.ctypes.data_as(_dp), max_rows, C.byref(n), cnt.ctypes.data_as(_P(C.c_int64)))
    state[:] = st
    return status, rows[:n.value, :4].copy(), cnt
