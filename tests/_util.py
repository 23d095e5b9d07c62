"""Shared helpers of the test suite: build the same tracers for the GPU ensemble
and for the CPU oracle, and compare them."""
import numpy as np

from rapt_gb300 import fields as F


def field_of(w):
    name, kw = w["field"]
    if name == "SynthGrid":
        return synth_grid(**kw)
    return getattr(F, name)(**kw)


def oracle_field(O, w):
    name, kw = w["field"]
    fld = field_of(w)
    if isinstance(fld, F.Grid):
        return oracle_grid(O, fld)
    return O.field(name, fld.device_params())


def oracle_config(O, w, **over):
    p = dict(w["params"])
    p.update(over)
    return O.config(rtol=p.get("rtol", 1.49012e-8), atol=p.get("atol", 1.49012e-8),
                    cycres=p.get("cyclotronresolution", 10), gctimestep=p.get("gctimestep", 0.0),
                    epss=p.get("epss", 5e-2), epst=p.get("epst", 5e-2), tableau=p.get("tableau", 0),
                    gc_eom=p.get("gc_eom", 0), nsteps=p.get("nsteps", 500),
                    rkf_tol=p.get("rkf_tol", 1e-3), rkf_hmin=p.get("rkf_hmin", 1e-12),
                    enforce_equatorial=p.get("enforce_equatorial", 0), bounce_quad=p.get("bounce_quad", 0))


def oracle_tracers(O, w, kind):
    n = len(w["mass"])
    f = oracle_field(O, w)
    cfg = oracle_config(O, w)
    out = []
    for i in range(n):
        if kind == "gc":
            out.append(O.gc_new_pa(f, w["pos"][i], w["v"][i], w["pa"][i], 0.0, w["mass"][i], w["charge"][i]))
        elif kind == "particle":
            out.append(O.particle_new(w["pos"][i], w["vel"][i], 0.0, w["mass"][i], w["charge"][i]))
        else:
            out.append(O.adaptive_init(f, cfg, w["pos"][i], w["vel"][i], 0.0, w["mass"][i], w["charge"][i]))
    return f, cfg, O.tracers_from_structs(out)


def gpu_ensemble(w, kind, max_rows=4, max_switch=0, form=0, **over):
    from rapt_gb300 import Ensemble
    n = len(w["mass"])
    ens = Ensemble(field_of(w), n, max_rows=max_rows, max_switch=max_switch)
    p = dict(w["params"])
    p.update(over)
    ens.configure(form=form, **p)
    if kind == "gc":
        ens.set_guiding_centers(w["pos"], w["v"], pa=w["pa"], t0=0.0, mass=w["mass"], charge=w["charge"])
    else:
        ens.set_particles(w["pos"], w["vel"], 0.0, w["mass"], w["charge"])
    ens.upload()
    if kind == "adaptive":
        ens.adaptive_init()
    return ens


def rel_state_error(gpu_s, orc_s, ncomp):
    """Per-tracer relative error of position and of momentum (or ppar)."""
    g = np.asarray(gpu_s)[:ncomp].T
    o = np.asarray(orc_s)[:, :ncomp]
    pos = np.linalg.norm(g[:, :3] - o[:, :3], axis=1) / np.linalg.norm(o[:, :3], axis=1)
    if ncomp == 6:
        mom = np.linalg.norm(g[:, 3:6] - o[:, 3:6], axis=1) / np.linalg.norm(o[:, 3:6], axis=1)
    else:
        mom = np.abs(g[:, 3] - o[:, 3]) / np.maximum(np.abs(o[:, 3]), 1e-300)
    return pos, mom


def sensitivity_envelope(O, w, kind, delta, rel=1e-15, **over):
    """Per-tracer divergence of the oracle from itself when the start position and
    momentum are scaled by (1 + rel): how far rounding-level differences can grow
    along each trajectory (large for chaotic, nonadiabatic orbits)."""
    w2 = dict(w)
    if kind == "gc":
        w2["pos"] = w["pos"] * (1 + rel)
    else:
        w2["pos"] = w["pos"] * (1 + rel)
        w2["vel"] = w["vel"] * (1 + rel)
    f, cfg, a = oracle_tracers(O, w, kind)
    _, _, b = oracle_tracers(O, w2, kind)
    if over:
        cfg = oracle_config(O, w, **over)
    k = {"particle": 0, "gc": 1, "adaptive": 2}[kind]
    O.batch_advance(f, cfg, k, a, delta)
    O.batch_advance(f, cfg, k, b, delta)
    n = 6 if kind == "particle" else 4
    pos, mom = rel_state_error(a["s"].T, b["s"], n)
    return a, pos, mom


def synth_grid(times, static=True):
    """Facade Grid over the synthetic snapshots of tests/golden/grid_data.py, by
    the reference's recipe: a subclass whose parsefile returns a snapshot."""
    from tests.golden import grid_data as GD

    class SynthGrid(F.Grid):
        def __init__(self, times):
            self._snaps = {"snap%d" % k: g for k, g in enumerate(GD.snapshots(times))}
            F.Grid.__init__(self, list(self._snaps))

        def parsefile(self, filename):
            return self._snaps[filename]

    g = SynthGrid(times)
    g.static = static
    return g


def oracle_grid(O, g):
    """The oracle's copy of a facade Grid."""
    return O.grid_field(g._t, g._x, g._y, g._z, g._B, g._E, static=g.static)


def within_envelope(err, env):
    """Device-oracle differences against the oracle's own divergence under a
    1e-15 perturbation of the start: the same distribution up to small factors
    (one perturbed run is a noisy per-tracer estimate, so the tail is bounded as
    a distribution, not tracer by tracer)."""
    assert np.median(err) <= max(1e-12, 10 * np.median(env)), (np.median(err), np.median(env))
    assert np.quantile(err, 0.9) <= max(1e-11, 10 * np.quantile(env, 0.9)), (np.quantile(err, 0.9),
                                                                              np.quantile(env, 0.9))
    assert err.max() <= max(1e-9, 10 * env.max()), (err.max(), env.max())
    assert np.mean(err > np.maximum(1e-9, 100 * env)) <= 0.03
