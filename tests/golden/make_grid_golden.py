#!/usr/bin/env python3
"""Generate tests/golden/grid_golden.npz from the unmodified RAPT reference's Grid.

Run where the reference is checked out, with RAPT_REFERENCE_ROOT naming that
directory; only the .npz travels. The snapshots come from grid_data.py
(computed, not stored). The reference's Grid is subclassed with a parsefile()
that returns those snapshots by name -- the subclassing the reference asks for
(fields.py:536-545) -- and is otherwise used as is.

Reference quirk: with a single file, Grid.__init__ sets ``time_indep``
(fields.py:596) while Bgrid/Egrid test ``_time_indep`` (fields.py:728, :761),
so evaluation fails with AttributeError. The single-snapshot cases set
``_time_indep = True`` after construction, the behaviour the docstring
describes (fields.py:553).

Contents:
  g4_*   five snapshots (0, 2, 4, 6, 8 s), static False: B, E at points sorted
         by time (the reference's window only moves forward), derived _Field
         quantities, a proton and an electron guiding centre over the window moves
         (the proton's last interval passes t = 8 s: the reference raises there)
  g3_*   one snapshot (time-independent), static True as the reference leaves it
  gout_* a proton that leaves the grid: the reference raises ValueError
  ga*_   Adaptive protons switching between particle and guiding-centre modes
"""
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
from oracle import shim  # noqa: E402
import grid_data as GD  # noqa: E402

rapt = shim.load()
Re, m_pr, m_el, e = rapt.Re, rapt.m_pr, rapt.m_el, rapt.e


class SynthGrid(rapt.fields.Grid):
    def __init__(self, times):
        self._snaps = {"snap%d" % k: g for k, g in enumerate(GD.snapshots(times))}
        rapt.fields.Grid.__init__(self, list(self._snaps))

    def parsefile(self, filename):
        return self._snaps[filename]


def single():
    g = SynthGrid((0.0,))
    g._time_indep = True
    return g


def inside_points(rng, n, tmax):
    x, y, z = GD.axes()
    p = np.column_stack([rng.uniform(0, tmax, n), rng.uniform(x[0], x[-1], n), rng.uniform(y[0], y[-1], n),
                         rng.uniform(z[0], z[-1], n)])
    # grid nodes, snapshot times and the far corner
    k = n // 8
    p[:k, 1] = rng.choice(x, k)
    p[k:2 * k, 3] = rng.choice(z, k)
    p[2 * k:3 * k, 0] = rng.choice(np.array([t for t in GD.TIMES if t <= tmax]), k)
    p[3 * k] = [tmax, x[-1], y[-1], z[-1]]
    p[3 * k + 1] = [0.0, x[0], y[0], z[0]]
    return p[np.argsort(p[:, 0], kind="stable")]


DERIVED = ["magB", "unitb", "gradB", "jacobianB", "curvature", "curlb", "dBdt", "dbdt", "lengthscale",
           "timescale"]


def derived(f, pts):
    rows = []
    for p in pts:
        r = []
        for q in DERIVED:
            v = np.atleast_1d(np.asarray(getattr(f, q)(p), float)).ravel()
            r.extend(v)
        rows.append(r)
    return np.array(rows)


def proton_vel(f, pos, ke, pa_deg, t0=0.0):
    v = rapt.utils.speedfromKE(ke, m_pr)
    b = f.unitb(np.r_[t0, pos])
    u = np.cross(b, [0, 0, 1.0]) if abs(b[2]) < 0.9 else np.cross(b, [1.0, 0, 0])
    u /= np.linalg.norm(u)
    a = np.deg2rad(pa_deg)
    return v * (np.cos(a) * b + np.sin(a) * u)


def run(out, case, tracer, delta, **params):
    saved = dict(rapt.params)
    rapt.params.update(params)
    raised = 0
    try:
        tracer.advance(delta)
    except ValueError:
        raised = 1
    finally:
        rapt.params.clear()
        rapt.params.update(saved)
    out[case + "_rows"] = tracer.trajectory
    out[case + "_raised"] = np.array([raised])


def main():
    rng = np.random.default_rng(20240611)
    out = {}
    # ---- five snapshots
    f4 = SynthGrid(GD.TIMES)
    f4.static = False
    p = inside_points(rng, 400, 8.0)
    out["g4_points"] = p
    out["g4_B"] = np.array([f4.B(q) for q in p])
    f4 = SynthGrid(GD.TIMES)  # a fresh window for each pass
    f4.static = False
    out["g4_E"] = np.array([f4.E(q) for q in p])
    # derived quantities, away from the edges so that the stencils stay inside
    x, y, z = GD.axes()
    q = np.column_stack([np.sort(rng.uniform(0.1, 7.9, 40)), rng.uniform(4 * Re, 8 * Re, 40),
                         rng.uniform(-3 * Re, 3 * Re, 40), rng.uniform(-2.5 * Re, 2.5 * Re, 40)])
    f4 = SynthGrid(GD.TIMES)
    f4.static = False
    out["g4_dpoints"] = q
    out["g4_derived"] = derived(f4, q)
    # proton over 8 s (two window moves), static False
    f4 = SynthGrid(GD.TIMES)
    f4.static = False
    pos = np.array([5.5 * Re, 0.0, 0.2 * Re])
    vel = proton_vel(f4, pos, 1e6, 45)
    out["g4_p_init"] = np.r_[pos, vel, m_pr, e]
    run(out, "g4_p", rapt.Particle(pos, vel, 0, m_pr, e, f4), 8.0, solvertolerances=(1e-8, 1e-8))
    # electron guiding centre from 0.5 s (dB/dt differences reach t - 1e-3) to 7.5 s
    f4 = SynthGrid(GD.TIMES)
    f4.static = False
    pos = np.array([5.0 * Re, 0.5 * Re, 0.0])
    v = rapt.utils.speedfromKE(1e5, m_el)
    out["g4_g_init"] = np.r_[pos, v, 50, m_el, -e, 0.5]
    run(out, "g4_g", rapt.GuidingCenter(pos, v, pa=50, t0=0.5, mass=m_el, charge=-e, field=f4), 7.0,
        solvertolerances=(1e-8, 1e-8), GCtimestep=0.5)
    # ---- one snapshot, static True
    f3 = single()
    p3 = inside_points(rng, 200, 0.0)
    p3[:, 0] = rng.uniform(-100, 100, len(p3))  # time is ignored
    out["g3_points"] = p3
    out["g3_B"] = np.array([f3.B(q) for q in p3])
    out["g3_E"] = np.array([f3.E(q) for q in p3])
    q3 = q.copy()
    out["g3_dpoints"] = q3
    out["g3_derived"] = _derived_static(f3, q3)
    pos = np.array([6.0 * Re, 0.0, 0.0])
    vel = proton_vel(f3, pos, 5e5, 60)
    out["g3_p_init"] = np.r_[pos, vel, m_pr, e]
    run(out, "g3_p", rapt.Particle(pos, vel, 0, m_pr, e, f3), 3.0, solvertolerances=(1e-8, 1e-8))
    # ---- leaving the grid: a 1 MeV proton gyrating through the x = 9.5 Re face
    f3 = single()
    pos = np.array([9.0 * Re, 0.0, 0.0])
    vel = proton_vel(f3, pos, 1e6, 90)
    out["gout_p_init"] = np.r_[pos, vel, m_pr, e]
    run(out, "gout_p", rapt.Particle(pos, vel, 0, m_pr, e, f3), 5.0, solvertolerances=(1e-8, 1e-8))
    # ---- Adaptive in the five snapshots (static False) from t0 = 0.5 s: protons
    # that start as particles and switch between the modes as they bounce
    for case, (L, ke, pa) in (("ga0", (6.5, 1e6, 40.0)), ("ga1", (7.0, 2e6, 20.0))):
        f4 = SynthGrid(GD.TIMES)
        f4.static = False
        pos = np.array([L * Re, 0.0, 0.0])
        b = f4.unitb(np.r_[0.5, pos])
        u = np.cross(b, [1.0, 0, 0])
        u /= np.linalg.norm(u)
        a = np.deg2rad(pa)
        vel = rapt.utils.speedfromKE(ke, m_pr) * (np.cos(a) * b + np.sin(a) * u)
        saved = dict(rapt.params)
        rapt.params.update(solvertolerances=(1e-8, 1e-8), GCtimestep=0.5, cyclotronresolution=10)
        ad = rapt.Adaptive(pos, vel, 0.5, m_pr, e, f4)
        with contextlib.redirect_stdout(io.StringIO()):
            ad.advance(3.0)  # Adaptive compares the absolute time with delta: ends at t = 3
        rapt.params.clear()
        rapt.params.update(saved)
        out[case + "_init"] = np.r_[pos, vel, m_pr, e]
        out[case + "_modes"] = np.array([0 if isinstance(s, rapt.Particle) else 1 for s in ad.trajlist])
        out[case + "_t0s"] = np.array([s.trajectory[0, 0] for s in ad.trajlist])
        last = ad.trajlist[-1].trajectory[-1]
        out[case + "_final"] = np.r_[last, np.zeros(7 - len(last))]
    dst = os.path.join(HERE, "grid_golden.npz")
    np.savez_compressed(dst, **out)
    for k in sorted(out):
        print(k, np.shape(out[k]), out[k] if k.endswith("raised") else "")


def _derived_static(f, pts):
    # the static quantities only: dBdt, dbdt and timescale are 0 / None there
    rows = []
    for p in pts:
        r = []
        for q in ("magB", "unitb", "gradB", "jacobianB", "curvature", "curlb", "lengthscale"):
            r.extend(np.atleast_1d(np.asarray(getattr(f, q)(p), float)).ravel())
        rows.append(r)
    return np.array(rows)


if __name__ == "__main__":
    main()
