#!/usr/bin/env python3
"""Generate tests/golden/golden.npz by running the unmodified RAPT reference.

Run where the reference is checked out, with RAPT_REFERENCE_ROOT naming that
directory; the hosts that run the tests do not need it -- only the .npz travels.

The reference is imported through oracle/shim.py. Per-call SciPy counters
(NFCN, NSTEP, NACCPT, NREJCT = iwork[16:20]) are recorded by replacing the
name ``ode`` inside the reference's Particle and GuidingCenter modules with a
thin subclass that logs them after each integrate() call; the reference source
is not modified. The Particle equation of motion (a closure inside
Particle.advance, rapt/Particle.py:284-298) is captured the same way.

Contents (all seeded):
  kat_*             known answers recorded in the reference's notebooks
  field_<model>_*   _Field quantities at random points (fields.py:42-280)
  eom_*             Particle closure and the three GuidingCenter EOMs
  conv_*            utils.guidingcenter / utils.GCtoFP / isadiabatic
  traj_<case>_*     trajectories, tcur, per-interval counters
"""
import os
import sys
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import shim  # noqa: E402

rapt = shim.load()
Re, m_pr, m_el, e, c = rapt.Re, rapt.m_pr, rapt.m_el, rapt.e, rapt.c
from scipy.integrate import ode as _ode  # noqa: E402

P_MOD = sys.modules["rapt.Particle"]
G_MOD = sys.modules["rapt.GuidingCenter"]
LOG = []          # per-integrate counters of the current run
CAPTURED = {}     # last eom passed to ode()


class LoggingODE(_ode):
    def __init__(self, f, jac=None):
        CAPTURED["f"] = f
        super().__init__(f, jac)

    def integrate(self, t, step=False, relax=False):
        y = super().integrate(t, step, relax)
        LOG.append(tuple(int(x) for x in self._integrator.iwork[16:20]))
        return y


P_MOD.ode = LoggingODE
G_MOD.ode = LoggingODE


class Harris(rapt.fields._Field):
    """CPU stand-in with the reference's _Field machinery: B = (B0 tanh(z/L), 0, Bn), E = (0, Ey, 0)."""

    def __init__(self, B0=20e-9, L=0.5 * Re, Bn=2e-9, Ey=0.2e-3):
        rapt.fields._Field.__init__(self)
        self.static = False
        self.B0_, self.L, self.Bn, self.Ey = B0, L, Bn, Ey
        self.gradientstepsize = L * 1e-4

    def B(self, tpos):
        return np.array([self.B0_ * np.tanh(tpos[3] / self.L), 0, self.Bn])

    def E(self, tpos):
        return np.array([0, self.Ey, 0])


class CompressedDipole(rapt.fields._Field):
    """CPU stand-in: VarEarthDipole form with B0(t) = B0 (1 + amp sin(2 pi t/P)) and
    the induced E = -dB0/dt Re^3 (y, -x, 0) / r^3."""

    def __init__(self, B0=3.07e-5, amp=0.1, period=60.0):
        rapt.fields._Field.__init__(self)
        self.gradientstepsize = Re / 1000
        self.static = False
        self.B0_, self._amp, self._period = B0, amp, period

    def B(self, tpos):
        t, x, y, z = tpos
        return -self.B0_ * Re ** 3 * (1 + self._amp * np.sin(2 * np.pi * t / self._period)) * \
            np.array([3 * x * z, 3 * y * z, (2 * z * z - x * x - y * y)]) / pow(x * x + y * y + z * z, 5.0 / 2.0)

    def E(self, tpos):
        t, x, y, z = tpos
        w = 2 * np.pi / self._period
        dB0dt = self.B0_ * self._amp * w * np.cos(w * t)
        s = -dB0dt * Re ** 3 / pow(x * x + y * y + z * z, 1.5)
        return np.array([s * y, -s * x, 0.0])


def reference_fields():
    F = rapt.fields
    return {
        "EarthDipole": (F.EarthDipole(), []),
        "DoubleDipole": (F.DoubleDipole(), []),
        "UniformBz": (F.UniformBz(2e-5), [2e-5]),
        "UniformCrossedEB": (F.UniformCrossedEB(1e-3, 3e-5), [1e-3, 3e-5]),
        "VarEarthDipole": (F.VarEarthDipole(), []),
        "Parabolic": (F.Parabolic(), []),
        "Harris": (Harris(), []),
        "CompressedDipole": (CompressedDipole(), []),
    }


def points(name, n, rng):
    if name == "Parabolic":
        p = rng.uniform(-2, 2, (n, 3))
    elif name == "Harris":
        p = rng.uniform(-3 * Re, 3 * Re, (n, 3))
    else:
        r = rng.uniform(3, 9, n) * Re
        d = rng.standard_normal((n, 3))
        p = r[:, None] * d / np.linalg.norm(d, axis=1, keepdims=True)
    return np.column_stack([rng.uniform(0, 50, n), p])


QUANT = ["B", "E", "unitb", "magB", "gradB", "jacobianB", "curvature", "curlb", "dBdt", "dbdt",
         "lengthscale", "timescale"]


def main():
    warnings.simplefilter("ignore")
    out = {}
    # ---- notebook known answers
    dd = rapt.fields.DoubleDipole()
    out["kat_doubledipole_tpos"] = np.array([[0, -7.8 * Re, 0, 0], [0, 10 * Re, 0, 0]])
    out["kat_doubledipole_magB_recorded"] = np.array([6.6121501357170836e-08, 6.1400000000000007e-08])
    out["kat_doubledipole_magB_here"] = np.array([dd.magB(t) for t in out["kat_doubledipole_tpos"]])
    out["kat_speiser_switch_recorded"] = np.array([168.0, 271.537802289])

    rng = np.random.default_rng(2024)
    # ---- fields
    for name, (fld, params) in reference_fields().items():
        tp = points(name, 24, rng)
        out["field_%s_params" % name] = np.array(params, float)
        out["field_%s_tpos" % name] = tp
        for q in QUANT:
            vals = []
            for t in tp:
                r = getattr(fld, q)(t)
                r = np.nan if r is None else r
                vals.append(np.ravel(np.asarray(r, float)))
            out["field_%s_%s" % (name, q)] = np.array(vals)
    # ---- equations of motion
    fld = rapt.fields.DoubleDipole()
    tp = points("DoubleDipole", 16, rng)
    v = rng.uniform(1e7, 2.5e8, 16)
    pa = rng.uniform(5, 175, 16)
    eom_gc = {0: [], 1: [], 2: []}
    gc_state = []
    for i in range(16):
        g = rapt.GuidingCenter(tp[i, 1:], v[i], pa=pa[i], t0=tp[i, 0], mass=m_el, charge=-e, field=fld)
        Y = g.trajectory[-1, 1:].copy()
        gc_state.append(np.r_[tp[i, 0], Y, g.mu, v[i]])
        eom_gc[0].append(g._TaoChanBrizardEOM(tp[i, 0], Y))
        eom_gc[1].append(g._BrizardChanEOM(tp[i, 0], Y))
        eom_gc[2].append(g._NorthropTellerEOM(tp[i, 0], Y))
    out["eom_gc_state"] = np.array(gc_state)  # t, x, y, z, ppar, mu, v
    for k in eom_gc:
        out["eom_gc_%d" % k] = np.array(eom_gc[k])
    # Particle closure in a non-static field (gm recomputed from the stage momentum)
    for fname, fobj in (("UniformCrossedEB", rapt.fields.UniformCrossedEB(1e-3, 3e-5)),
                        ("EarthDipole", rapt.fields.EarthDipole())):
        tp = points(fname if fname != "UniformCrossedEB" else "EarthDipole", 8, rng)
        rows = []
        for i in range(8):
            vel = rng.standard_normal(3)
            vel *= rng.uniform(1e6, 1e8) / np.linalg.norm(vel)
            p = rapt.Particle(tp[i, 1:], vel, tp[i, 0], m_pr, e, fobj)
            rapt.params["cyclotronresolution"] = 10
            p.advance(1e-12)  # builds the closure; one tiny interval
            f = CAPTURED["f"]
            Y = np.r_[tp[i, 1:], m_pr * vel / np.sqrt(1 - vel @ vel / c ** 2)]
            gm0 = np.sqrt(m_pr ** 2 + np.dot(p.trajectory[0, 4:], p.trajectory[0, 4:]) / c ** 2)
            rows.append(np.r_[tp[i, 0], Y, gm0, f(tp[i, 0], Y)])
        out["eom_particle_%s" % fname] = np.array(rows)  # t, Y(6), gm frozen, out(6)
    # ---- conversions and adiabaticity
    fld = rapt.fields.EarthDipole()
    conv = []
    for i in range(12):
        r = np.array([rng.uniform(3, 7) * Re, rng.uniform(-1, 1) * Re, rng.uniform(-1, 1) * Re])
        vel = rng.standard_normal(3)
        vel *= rng.uniform(1e6, 5e7) / np.linalg.norm(vel)
        res = rapt.utils.guidingcenter(0.0, r, vel, fld, m_pr, e)
        gc, vp, sp = res
        pos2, vel2 = rapt.utils.GCtoFP(0.0, gc, vp, sp, fld, m_pr, e, 0.0)
        p = rapt.Particle(r, vel, 0.0, m_pr, e, fld)
        rapt.params["epss"] = 0.05
        conv.append(np.r_[r, vel, gc, vp, sp, pos2, vel2, float(p.isadiabatic()), p.cycrad(), p.cycper()])
    out["conv_earthdipole"] = np.array(conv)
    # ---- trajectories with per-interval counters
    def run(case, tracer, delta, **params):
        saved = dict(rapt.params)
        rapt.params.update(params)
        LOG.clear()
        raised = 0
        try:
            tracer.advance(delta)
        except (rapt.Adiabatic, rapt.NonAdiabatic):
            raised = 1
        rapt.params.clear()
        rapt.params.update(saved)
        out["traj_%s_rows" % case] = tracer.trajectory
        out["traj_%s_counters" % case] = np.array(LOG, np.int64).reshape(-1, 4)
        out["traj_%s_tcur" % case] = np.array([tracer.tcur, raised], float)

    def proton(pos, ke, pa_deg, fld):
        v = rapt.utils.speedfromKE(ke, m_pr)
        b = fld.unitb(np.r_[0, pos])
        u = np.cross(b, [0, 0, 1.0]) if abs(b[2]) < 0.9 else np.cross(b, [1.0, 0, 0])
        u /= np.linalg.norm(u)
        a = np.deg2rad(pa_deg)
        return v * (np.cos(a) * b + np.sin(a) * u)

    ed = rapt.fields.EarthDipole()
    for k, (ke, pa_deg) in enumerate([(1e6, 45), (1e5, 20), (5e6, 80)]):
        pos = np.array([6 * Re, 0, 0])
        vel = proton(pos, ke, pa_deg, ed)
        out["traj_p%d_init" % k] = np.r_[pos, vel, m_pr, e]
        run("p%d" % k, rapt.Particle(pos, vel, 0, m_pr, e, ed), 2.0, solvertolerances=(1e-8, 1e-8),
            cyclotronresolution=20)
    # particle in a time-dependent field, and with enforce equatorial
    vd = rapt.fields.VarEarthDipole()
    pos = np.array([5 * Re, 0, 0])
    vel = proton(pos, 1e6, 50, ed)
    out["traj_pvar_init"] = np.r_[pos, vel, m_pr, e]
    run("pvar", rapt.Particle(pos, vel, 0, m_pr, e, vd), 1.0, solvertolerances=(1e-9, 1e-9))
    vel = np.array([0, 1e7, 0.0])
    out["traj_peq_init"] = np.r_[pos, vel, m_pr, e]
    run("peq", rapt.Particle(pos, vel, 0, m_pr, e, ed), 1.0, **{"enforce equatorial": True})
    # guiding centres, three EOMs
    ddf = rapt.fields.DoubleDipole()
    for k, (ke, pa_deg, L) in enumerate([(1e6, 45, 5.0), (2e5, 70, 6.5)]):
        pos = np.array([L * Re, 0, 0])
        v = rapt.utils.speedfromKE(ke, m_el)
        out["traj_g%d_init" % k] = np.r_[pos, v, pa_deg, m_el, -e]
        run("g%d" % k, rapt.GuidingCenter(pos, v, pa=pa_deg, t0=0, mass=m_el, charge=-e, field=ddf), 3.0,
            solvertolerances=(1e-8, 1e-8), GCtimestep=1.0)
    for eom in ("BrizardChanEOM", "NorthropTellerEOM"):
        pos = np.array([5 * Re, 0, 0])
        v = rapt.utils.speedfromKE(1e6, m_el)
        g = rapt.GuidingCenter(pos, v, pa=45, t0=0, mass=m_el, charge=-e, field=ddf)
        saved = dict(rapt.params)
        rapt.params.update(solvertolerances=(1e-8, 1e-8), GCtimestep=1.0)
        LOG.clear()
        g.advance(2.0, eom=eom)
        rapt.params.clear()
        rapt.params.update(saved)
        out["traj_g%s_rows" % eom] = g.trajectory
        out["traj_g%s_counters" % eom] = np.array(LOG, np.int64).reshape(-1, 4)
    # failure path: nsteps exceeded -> the loop ends silently (Particle.py:304)
    # (recorded with a coarse cadence so that one interval needs > 500 steps)
    pos = np.array([6 * Re, 0, 0])
    vel = proton(pos, 1e6, 45, ed)
    out["traj_pfail_init"] = np.r_[pos, vel, m_pr, e]
    run("pfail", rapt.Particle(pos, vel, 0, m_pr, e, ed), 50.0, solvertolerances=(1e-8, 1e-8),
        cyclotronresolution=0.02)
    # ---- Adaptive: Speiser orbit (notebook case) and a Harris-sheet proton
    saved = dict(rapt.params)
    rapt.params.update(solvertolerances=(1e-12, 1e-12), epss=0.02, GCtimestep=1, cyclotronresolution=10)
    import io
    import contextlib
    a = rapt.Adaptive([5, -5, 0.9], [-0.1, 0.1, 0], 0, 1, 1, rapt.fields.Parabolic())
    with contextlib.redirect_stdout(io.StringIO()):
        a.advance(300)
    rapt.params.clear()
    rapt.params.update(saved)
    out["adaptive_speiser_modes"] = np.array([0 if isinstance(s, rapt.Particle) else 1 for s in a.trajlist])
    out["adaptive_speiser_t0s"] = np.array([s.trajectory[0, 0] for s in a.trajlist])
    out["adaptive_speiser_final"] = a.trajlist[-1].trajectory[-1]
    out["adaptive_speiser_nrows"] = np.array([len(s.trajectory) for s in a.trajlist])
    # Harris sheet: proton crossing the sheet
    saved = dict(rapt.params)
    rapt.params.update(solvertolerances=(1e-8, 1e-8), GCtimestep=0.5, cyclotronresolution=10)
    hs = Harris()
    v = rapt.utils.speedfromKE(10e3, m_pr)
    pos = np.array([0, 0, 1.5 * Re])
    vel = v * np.array([0.3, 0.2, -np.sqrt(1 - 0.13)])
    a = rapt.Adaptive(pos, vel, 0, m_pr, e, hs)
    with contextlib.redirect_stdout(io.StringIO()):
        a.advance(60)
    rapt.params.clear()
    rapt.params.update(saved)
    out["adaptive_harris_init"] = np.r_[pos, vel, m_pr, e]
    out["adaptive_harris_modes"] = np.array([0 if isinstance(s, rapt.Particle) else 1 for s in a.trajlist])
    out["adaptive_harris_t0s"] = np.array([s.trajectory[0, 0] for s in a.trajlist])
    out["adaptive_harris_final"] = np.r_[a.trajlist[-1].trajectory[-1], np.zeros(7 - a.trajlist[-1].trajectory.shape[1])]
    out["adaptive_harris_nrows"] = np.array([len(s.trajectory) for s in a.trajlist])
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    # bounce period (flutils.halfbouncepath, GuidingCenter.bounceperiod) and the
    # bounce-period cadence of GuidingCenter.advance (GCtimestep = 0)
    bp = []
    for mid, fobj in ((0, ed), (1, ddf)):
        for L, pa_deg, phi in ((5.0, 45, 180), (6.0, 15, 180), (4.5, 80, 90), (7.0, 30, 0), (5.5, 89.5, 45)):
            tpos = np.array([0, L * Re * np.cos(np.radians(phi)), L * Re * np.sin(np.radians(phi)), 0.0])
            Bm = fobj.magB(tpos) / np.sin(np.radians(pa_deg)) ** 2
            bp.append((mid, L, pa_deg, phi, Bm, rapt.flutils.halfbouncepath(tpos, fobj, Bm)))
    out["bounce_halfpath"] = np.array(bp)  # model id, L, pa, phi, Bm, S_b
    gbp = []
    for ke, pa_deg, L, mass, q in ((1e6, 45, 5.0, m_el, -e), (1e5, 30, 6.0, m_pr, e), (5e6, 70, 4.0, m_el, -e)):
        pos = np.array([L * Re, 0, 0])
        v = rapt.utils.speedfromKE(ke, mass)
        g = rapt.GuidingCenter(pos, v, pa=pa_deg, t0=0, mass=mass, charge=q, field=ddf)
        gbp.append(np.r_[pos, v, pa_deg, mass, q, g.bounceperiod()])
    out["bounce_gc_period"] = np.array(gbp)  # pos(3), v, pa, mass, charge, T_b
    pos = np.array([5 * Re, 0, 0])
    v = rapt.utils.speedfromKE(1e6, m_el)
    out["traj_gbounce_init"] = np.r_[pos, v, 45, m_el, -e]
    run("gbounce", rapt.GuidingCenter(pos, v, pa=45, t0=0, mass=m_el, charge=-e, field=ddf), 0.5,
        solvertolerances=(1e-8, 1e-8), GCtimestep=0)

    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
