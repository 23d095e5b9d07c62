#!/usr/bin/env python3
"""Generate tests/golden/rkf_golden.npz: the reference's tracers driven by its
own RKF45 stepper (rapt/rkf.py:13-143).

The reference integrates tracers with SciPy's dop853 / dopri5 and uses rkf()
only for field lines. The RKF45 tracer tableau of this package
(rapt_config.tableau = 1) runs Particle.advance and GuidingCenter.advance with
rkf() in place of SciPy's integrate(): each output interval [t, t + dt] is one
rkf(f, t, t + dt, y, tol, hmax = dt, hmin) call. The fixtures are made the same
way from the unmodified reference: the name ``ode`` inside its Particle and
GuidingCenter modules is replaced by a stand-in whose integrate() calls
rapt.rkf.rkf on the equations of motion the reference passes to it (the
Particle closure, GuidingCenter._TaoChanBrizardEOM and the other EOMs). rkf()
takes f(x, t); the EOMs take (t, y), so the stand-in swaps the arguments.

Per output interval the stand-in records (NFCN, NSTEP, NACCPT, NREJCT) from a
call counter on f (6 calls per attempt) and the accepted points rkf returns.
Where rkf raises RuntimeError at hmin the exception leaves advance() as in the
reference; the fixture records the rows written before it.

Run where the reference is checked out, with RAPT_REFERENCE_ROOT naming that
directory; only the .npz travels.
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
RKF = sys.modules["rapt.rkf"].rkf
P_MOD = sys.modules["rapt.Particle"]
G_MOD = sys.modules["rapt.GuidingCenter"]
OPT = {"tol": 1e-3, "hmin": 1e-12}
LOG = []


class RkfODE:
    """The subset of scipy.integrate.ode that Particle.advance and
    GuidingCenter.advance use, integrating each interval with rapt.rkf.rkf."""

    def __init__(self, f, jac=None):
        self.f = f
        self.t = 0.0
        self.y = None

    def set_integrator(self, name, **kw):
        return self

    def set_initial_value(self, y, t=0.0):
        self.y = np.array(y, float)
        self.t = float(t)
        return self

    def successful(self):
        return True

    def integrate(self, t):
        calls = [0]

        def g(x, tt):
            calls[0] += 1
            return self.f(tt, x)

        try:
            T, X = RKF(g, self.t, t, self.y, OPT["tol"], t - self.t, OPT["hmin"])
        finally:
            nst = calls[0] // 6
            LOG.append((calls[0], nst, -1, -1))
        acc = len(T) - 1
        LOG[-1] = (calls[0], nst, acc, nst - acc)
        self.t = float(T[-1])
        self.y = np.array(X[-1], float)
        return self.y


P_MOD.ode = RkfODE
G_MOD.ode = RkfODE


def proton(fld, pos, ke, pa_deg):
    v = rapt.utils.speedfromKE(ke, m_pr)
    b = fld.unitb(np.r_[0, pos])
    u = np.cross(b, [0, 0, 1.0]) if abs(b[2]) < 0.9 else np.cross(b, [1.0, 0, 0])
    u /= np.linalg.norm(u)
    a = np.deg2rad(pa_deg)
    return v * (np.cos(a) * b + np.sin(a) * u)


def main():
    warnings.simplefilter("ignore")
    out = {}

    def run(case, tracer, delta, tol, hmin=1e-12, eom=None, **params):
        saved = dict(rapt.params)
        rapt.params.update(params)
        OPT["tol"], OPT["hmin"] = tol, hmin
        LOG.clear()
        raised = 0
        try:
            if eom is None:
                tracer.advance(delta)
            else:
                tracer.advance(delta, eom=eom)
        except RuntimeError:
            raised = 1
        rapt.params.clear()
        rapt.params.update(saved)
        out["%s_rows" % case] = tracer.trajectory
        out["%s_counters" % case] = np.array(LOG, np.int64).reshape(-1, 4)
        out["%s_meta" % case] = np.array([tracer.tcur, raised, tol, hmin], float)

    ed = rapt.fields.EarthDipole()
    vd = rapt.fields.VarEarthDipole()
    dd = rapt.fields.DoubleDipole()
    # particles: static field (gamma m frozen) and a time-dependent one (recomputed per stage)
    for case, fld, pos, ke, pa, tol, delta in (("p_earth", ed, [6 * Re, 0, 0], 1e6, 45, 1e-3, 0.5),
                                                ("p_earth_lo", ed, [5 * Re, 0, 0], 1e5, 20, 1e-2, 0.3),
                                                ("p_var", vd, [5 * Re, 0, 0], 1e6, 50, 1e-2, 0.3)):
        pos = np.array(pos, float)
        vel = proton(ed, pos, ke, pa)
        out["%s_init" % case] = np.r_[pos, vel, m_pr, e]
        run(case, rapt.Particle(pos, vel, 0, m_pr, e, fld), delta, tol, cyclotronresolution=20)
    # guiding centres: the three equations of motion
    for case, ke, pa, L, tol, eom in (("g_tcb", 1e6, 45, 5.0, 1e-3, None),
                                      ("g_tcb_lo", 2e5, 70, 6.5, 1e-2, None),
                                      ("g_bc", 1e6, 45, 5.0, 1e-2, "BrizardChanEOM"),
                                      ("g_nt", 1e6, 30, 5.5, 1e-2, "NorthropTellerEOM")):
        pos = np.array([L * Re, 0, 0])
        v = rapt.utils.speedfromKE(ke, m_el)
        out["%s_init" % case] = np.r_[pos, v, pa, m_el, -e]
        run(case, rapt.GuidingCenter(pos, v, pa=pa, t0=0, mass=m_el, charge=-e, field=dd), 2.0, tol, eom=eom,
            GCtimestep=1.0)
    # rkf raises at hmin in the first interval: advance() adds no row
    pos = np.array([5 * Re, 0, 0])
    v = rapt.utils.speedfromKE(1e6, m_el)
    out["g_hmin_init"] = np.r_[pos, v, 45, m_el, -e]
    run("g_hmin", rapt.GuidingCenter(pos, v, pa=45, t0=0, mass=m_el, charge=-e, field=dd), 3.0, 1e-5,
        hmin=1.5e-3, GCtimestep=1.0)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rkf_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes,", len(out), "arrays")
    for k in sorted(out):
        if k.endswith("_meta"):
            print(k, out[k], "rows", len(out[k[:-5] + "_rows"]), "counters", out[k[:-5] + "_counters"].sum(0))


if __name__ == "__main__":
    main()
