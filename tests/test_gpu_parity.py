"""GPU kernels against the CPU oracle on the same seeded inputs (through the C ABI)."""
import numpy as np
import pytest

from rapt_gb300 import workloads as W
from tests._util import (field_of, gpu_ensemble, oracle_config, oracle_field, oracle_tracers,
                         rel_state_error, sensitivity_envelope)

pytestmark = pytest.mark.gpu

MODELS = [("EarthDipole", {}), ("DoubleDipole", {}), ("UniformBz", {"Bz": 2e-5}),
          ("UniformCrossedEB", {"Ey": 1e-3, "Bz": 3e-5}), ("VarEarthDipole", {}), ("Parabolic", {}),
          ("Harris", {}), ("CompressedDipole", {})]


def _points(name, n, rng):
    if name == "Parabolic":
        p = rng.uniform(-2, 2, (n, 3))
    elif name == "Harris":
        p = rng.uniform(-3 * W.Re, 3 * W.Re, (n, 3))
    else:
        r = rng.uniform(3, 9, n) * W.Re
        d = rng.standard_normal((n, 3))
        p = r[:, None] * d / np.linalg.norm(d, axis=1, keepdims=True)
    return np.column_stack([rng.uniform(0, 50, n), p])


@pytest.mark.parametrize("name,kw", MODELS)
def test_field_quantities_match_oracle(oracle, name, kw):
    from rapt_gb300 import fields as F
    fld = getattr(F, name)(**kw)
    of = oracle.field(name, fld.device_params())
    rng = np.random.default_rng(3)
    tp = _points(name, 64, rng)
    # (quantity, relative tolerance): direct values to a few ulp; finite
    # differences amplify ulp differences by r/d (up to ~1e7 for EarthDipole).
    for q, tol in [("B", 1e-14), ("E", 1e-14), ("magB", 1e-14), ("unitb", 1e-14), ("gradB", 1e-7),
                   ("curlb", 1e-6), ("jacobianB", 1e-7), ("lengthscale", 1e-7)]:
        g = np.asarray(getattr(fld, q)(tp), float).reshape(len(tp), -1)
        o = np.array([np.ravel(oracle.field_eval(of, q, t)) for t in tp]).reshape(len(tp), -1)
        same = (g == o) | (np.isnan(g) & np.isnan(o))  # includes inf == inf (uniform fields)
        fin = np.where(np.isfinite(o), o, 0.0)
        scale = np.maximum(np.max(np.abs(fin), axis=1, keepdims=True), 1e-300)
        err = np.max(np.where(same, 0.0, np.abs(g - o) / scale))
        if name == "Harris" and q in ("gradB", "curlb", "jacobianB", "lengthscale"):
            # CUDA's and glibc's tanh differ by an ulp; far from the sheet the
            # differences over d = L * 1e-4 amplify that to ~1e-6
            tol = 1e-5
        assert err <= tol, (name, q, err)
    if not fld.static:
        # None of the time-dependent models turns its field direction, so db/dt is
        # central-difference rounding noise (~eps / timederivstepsize) in both codes.
        g = np.asarray(fld.dbdt(tp)).reshape(len(tp), -1)
        o = np.array([oracle.field_eval(of, "dbdt", t) for t in tp])
        assert np.all(np.abs(g) < 1e-11) and np.all(np.abs(o) < 1e-11)


@pytest.mark.parametrize("name,kw", MODELS)
def test_rhs_match_oracle(oracle, ctx, name, kw):
    from rapt_gb300 import fields as F
    fld = getattr(F, name)(**kw)
    fld.bind(ctx)
    of = oracle.field(name, fld.device_params())
    rng = np.random.default_rng(5)
    n = 32
    tp = _points(name, n, rng)
    m, q = W.m_pr, W.e
    v = rng.uniform(1e6, 1e7, n)
    vel = rng.standard_normal((n, 3))
    vel *= (v / np.linalg.norm(vel, axis=1))[:, None]
    gam = 1 / np.sqrt(1 - v ** 2 / W.c ** 2)
    mom = (m * gam)[:, None] * vel
    gm = np.sqrt(m * m + np.sum(mom * mom, 1) / W.c ** 2)
    cfg = oracle.config()
    st = np.column_stack([tp[:, 0], tp[:, 1:], mom, gm])
    out = ctx.rhs_eval(0, st, m, q)
    for i in range(n):
        o = oracle.particle_rhs(of, cfg, m, q, gm[i], tp[i, 0], np.r_[tp[i, 1:], mom[i]])
        assert np.allclose(out[i], o, rtol=1e-12, atol=1e-300), (name, i, out[i], o)
    # guiding centre, the three equations of motion
    ppar = m * gam * v * rng.uniform(-1, 1, n)
    mu = rng.uniform(1e-16, 1e-13, n)
    st = np.column_stack([tp[:, 0], tp[:, 1:], ppar, np.zeros(n), np.zeros(n), mu])
    for eom in (0, 1, 2):
        ctx.set_config(gc_eom=eom)
        out = ctx.rhs_eval(1, st, m, q, v)
        for i in range(n):
            o = oracle.gc_rhs(of, cfg, m, q, mu[i], v[i], tp[i, 0], np.r_[tp[i, 1:], ppar[i]], eom=eom)
            # drift terms come from central differences, whose relative rounding
            # error is amplified by r/d; bound them against the largest velocity
            vmax = np.max(np.abs(o[:3]))
            assert np.all(np.abs(out[i, :3] - o[:3]) <= 1e-7 * np.abs(o[:3]) + 1e-9 * vmax), (name, eom, i, out[i], o)
            # in non-static fields E* contains ppar * db/dt, and db/dt is central-
            # difference rounding noise (~eps / timederivstepsize) in both codes
            noise = 0.0 if fld.static else 1e-12 * abs(ppar[i])
            assert abs(out[i, 3] - o[3]) <= 1e-6 * abs(o[3]) + noise + 1e-300, (name, eom, i, out[i], o)
    ctx.set_config()


def test_config1_particle_dop853(oracle):
    """Config 1 in full: 256 protons, EarthDipole, 10 s, DOP853 (Particle.advance).

    GPU and oracle round differently (FMA contraction, rsqrt), so they take
    identical step sequences only until a rounding difference changes one
    controller decision; sensitive (nonadiabatic) orbits then amplify it. Each
    tracer's GPU-oracle difference is therefore bounded by 100x the oracle's own
    divergence under a 1e-15 relative perturbation of its start, or 1e-9."""
    w = W.config1()
    tr, env_pos, env_mom = sensitivity_envelope(oracle, w, "particle", w["delta"])
    ens = gpu_ensemble(w, "particle", max_rows=1024)
    stats = ens.advance("particle", w["delta"])
    h = ens.download()
    assert np.all(h["status"] == 0)
    pos, mom = rel_state_error(h["s"], tr["s"], 6)
    assert np.all(pos <= np.maximum(1e-9, 100 * env_pos)), (pos.max(), np.argmax(pos / np.maximum(1e-9, env_pos)))
    assert np.all(mom <= np.maximum(1e-9, 100 * env_mom)), (mom.max(), np.argmax(mom / np.maximum(1e-9, env_mom)))
    assert np.median(pos) < 1e-12 and np.median(mom) < 1e-11, (np.median(pos), np.median(mom))
    assert np.allclose(h["t_row"], tr["t"], rtol=1e-13, atol=0)
    steps_rel = np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]
    assert steps_rel.max() < 0.01, steps_rel.max()
    assert stats["accepted"] == h["naccept"].sum()
    # energy: |p| is conserved by the equations in the static dipole; the GPU's
    # drift matches the oracle's
    p0 = np.linalg.norm(w["mass"][:, None] * w["vel"] / np.sqrt(1 - np.sum(w["vel"] ** 2, 1) / W.c ** 2)[:, None], axis=1)
    dg = np.abs(np.linalg.norm(h["s"][3:6].T, axis=1) / p0 - 1)
    do = np.abs(np.linalg.norm(tr["s"][:, 3:6], axis=1) / p0 - 1)
    assert np.all(np.abs(dg - do) <= np.maximum(1e-12, 100 * env_mom)), np.max(np.abs(dg - do))
    # every output row of a few well-conditioned tracers against the oracle's rows
    rows, rm, nr, _, _ = ens.rows()
    f, cfg = oracle_field(oracle, w), oracle_config(oracle, w)
    for i in np.argsort(env_pos)[:3]:
        o = oracle.particle_new(w["pos"][i], w["vel"][i], 0.0, w["mass"][i], w["charge"][i])
        _, orows = oracle.advance(f, cfg, o, w["delta"])
        assert nr[i] == len(orows)
        assert np.allclose(rows[i, :nr[i], 1:4], orows[:, 1:4], rtol=1e-9, atol=0)


def test_config2_gc_dopri5(oracle):
    """Config 2 subsample: 64 electrons, DoubleDipole, GuidingCenter.advance (TCB,
    DOPRI5) for 10 s at 10 output times; same bound as config 1."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 1024))
    tr, env_pos, env_mom = sensitivity_envelope(oracle, w, "gc", 10.0)
    ens = gpu_ensemble(w, "gc", max_rows=16)
    ens.advance("gc", 10.0)
    h = ens.download()
    assert np.all(h["status"] == 0)
    assert np.allclose(h["mu"], tr["mu"], rtol=1e-13)
    pos, ppar = rel_state_error(h["s"], tr["s"], 4)
    assert np.all(pos <= np.maximum(1e-9, 100 * env_pos)), pos.max()
    pscale = w["mass"] * W.c
    dpp = np.abs(h["s"][3] - tr["s"][:, 3]) / pscale
    env_pp = env_mom * np.abs(tr["s"][:, 3]) / pscale
    assert np.all(dpp <= np.maximum(1e-9, 100 * env_pp)), dpp.max()
    assert np.median(pos) < 1e-11, np.median(pos)
    steps_rel = np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]
    assert steps_rel.max() < 0.01, steps_rel.max()


def test_config2_rows_1024_electrons_100s(oracle):
    """Config 2 at its stated horizon on 1,024 of its 65,536 electrons (evenly
    spaced): GuidingCenter.advance(100) with GCtimestep 1 s, all 100 output
    rows of every tracer against the oracle's rows. Each tracer's worst
    relative position difference over its rows is compared with the oracle's
    own divergence at t = 100 s under a 1e-15 relative perturbation of the
    start: over 1.5e7 steps the GPU's different rounding (FMA contraction,
    rsqrt) flips an accept/reject decision of a few tracers that the perturbed
    oracle run does not flip, and those then differ by the integration error
    (~1e-6 at 100 s, far below the tolerance-driven global error), so the bound
    holds as a distribution (median and 90th percentile within 10x the
    envelope's, at most 3 % of tracers beyond 100x their own envelope) and every
    tracer stays within 1e-5. mu is constant along a guiding-centre trajectory (GuidingCenter.py:63-133)."""
    from concurrent.futures import ThreadPoolExecutor
    import os
    w = W.subsample(W.config2(), np.arange(0, 65536, 64))
    n = len(w["mass"])
    tr, env_pos, env_mom = sensitivity_envelope(oracle, w, "gc", 100.0)
    f, cfg = oracle_field(oracle, w), oracle_config(oracle, w)

    def orows(i):
        o = oracle.gc_new_pa(f, w["pos"][i], w["v"][i], w["pa"][i], 0.0, w["mass"][i], w["charge"][i])
        _, r = oracle.advance(f, cfg, o, 100.0)
        return r

    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:  # ctypes releases the GIL during each call
        ref = list(ex.map(orows, range(n)))
    ens = gpu_ensemble(w, "gc", max_rows=104)
    ens.advance("gc", 100.0)
    h = ens.download()
    rows, rm, nr, _, _ = ens.rows()
    assert np.all(h["status"] == 0)
    assert np.all(nr == 100) and all(len(r) == 100 for r in ref)
    bound = np.maximum(1e-9, 100 * env_pos)
    worst = np.zeros(n)
    for i in range(n):
        assert np.array_equal(rows[i, :100, 0], ref[i][:, 0]), i  # row times t = 1..100
        d = np.linalg.norm(rows[i, :100, 1:4] - ref[i][:, 1:4], axis=1) / np.linalg.norm(ref[i][:, 1:4], axis=1)
        worst[i] = d.max()
    print("config 2, 100 rows: worst-row difference median %.2e p90 %.2e max %.2e; beyond 100x envelope: %d"
          % (np.median(worst), np.quantile(worst, 0.9), worst.max(), int(np.sum(worst > bound))))
    assert np.median(worst) <= max(1e-12, 10 * np.median(env_pos)), (np.median(worst), np.median(env_pos))
    assert np.quantile(worst, 0.9) <= max(1e-11, 10 * np.quantile(env_pos, 0.9))
    assert np.mean(worst > bound) <= 0.03 and worst.max() < 1e-5, (np.mean(worst > bound), worst.max())
    steps_rel = np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]
    assert np.median(steps_rel) < 1e-3 and steps_rel.max() < 0.01, steps_rel.max()
    assert np.allclose(h["mu"], tr["mu"], rtol=1e-13)


def test_adaptive_speiser_switch_times():
    """Known answer (reference notebook 'Adaptive Example - Speiser orbits', cell 8):
    Parabolic field, m = q = 1, rtol = atol = 1e-12, epss 0.02, GCtimestep 1,
    start (5, -5, 0.9), v = (-0.1, 0.1, 0), advance(300) switches to particle mode
    at 168.0 and back to guiding centre at 271.537802289."""
    from rapt_gb300 import Ensemble, fields as F
    ens = Ensemble(F.Parabolic(), 1, max_rows=4096, max_switch=8)
    ens.configure(rtol=1e-12, atol=1e-12, epss=0.02, gctimestep=1.0, cyclotronresolution=10)
    ens.set_particles([[5, -5, 0.9]], [[-0.1, 0.1, 0]], 0.0, 1.0, 1.0)
    ens.upload()
    ens.adaptive_init()
    assert ens.download()["mode"][0] == 1
    ens.advance("adaptive", 300.0)
    h = ens.download()
    rows, rm, nr, swt, swm = ens.rows()
    assert h["nswitch"][0] == 2 and h["mode"][0] == 1 and h["status"][0] == 0
    assert list(swm[0, :2]) == [0, 1]
    assert swt[0, 0] == 168.0
    assert abs(swt[0, 1] - 271.537802289) < 1e-8
