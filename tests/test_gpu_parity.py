"""GPU kernels against the CPU oracle on the same seeded inputs (through the C ABI)."""
import numpy as np
import pytest

from rapt_gb300 import workloads as W
from tests._util import field_of, gpu_ensemble, oracle_tracers, rel_state_error

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
        assert err <= tol, (name, q, err)
    if not fld.static:
        g = np.asarray(fld.dbdt(tp)).reshape(len(tp), -1)
        o = np.array([oracle.field_eval(of, "dbdt", t) for t in tp])
        assert np.allclose(g, o, rtol=1e-5, atol=1e-9 * np.max(np.abs(o)) + 1e-300)


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
            scale = np.abs(o) + 1e-12 * np.max(np.abs(o[:3]))
            assert np.all(np.abs(out[i, :4] - o) <= 1e-7 * scale + 1e-300), (name, eom, i, out[i, :4], o)
    ctx.set_config()


def test_config1_particle_dop853(oracle):
    """Config 1 in full: 256 protons, EarthDipole, 10 s, DOP853 (Particle.advance)."""
    w = W.config1()
    f, cfg, tr = oracle_tracers(oracle, w, "particle")
    oracle.batch_advance(f, cfg, 0, tr, w["delta"])
    ens = gpu_ensemble(w, "particle", max_rows=1024)
    stats = ens.advance("particle", w["delta"])
    h = ens.download()
    assert np.all(h["status"] == 0)
    pos, mom = rel_state_error(h["s"], tr["s"], 6)
    assert pos.max() < 1e-8 and mom.max() < 1e-8, (pos.max(), mom.max())
    assert np.allclose(h["t_row"], tr["t"], rtol=1e-13, atol=0)
    same = (h["naccept"] == tr["naccept"]) & (h["nreject"] == tr["nreject"]) & (h["nfcn"] == tr["nfcn"])
    assert same.mean() >= 0.99, same.mean()
    assert stats["accepted"] == h["naccept"].sum()
    # every output row against the oracle's rows for a few tracers
    rows, rm, nr, _, _ = ens.rows()
    for i in (0, 77, 255):
        o = oracle.particle_new(w["pos"][i], w["vel"][i], 0.0, w["mass"][i], w["charge"][i])
        _, orows = oracle.advance(f, cfg, o, w["delta"])
        assert nr[i] == len(orows)
        assert np.allclose(rows[i, :nr[i]], orows, rtol=1e-8, atol=0)


def test_config2_gc_dopri5(oracle):
    """Config 2 subsample: 64 electrons, DoubleDipole, GuidingCenter.advance (TCB, DOPRI5)
    for 10 s at 10 output times."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 1024))
    f, cfg, tr = oracle_tracers(oracle, w, "gc")
    oracle.batch_advance(f, cfg, 1, tr, 10.0)
    ens = gpu_ensemble(w, "gc", max_rows=16)
    ens.advance("gc", 10.0)
    h = ens.download()
    assert np.all(h["status"] == 0)
    assert np.allclose(h["mu"], tr["mu"], rtol=1e-13)
    pos, ppar = rel_state_error(h["s"], tr["s"], 4)
    assert pos.max() < 1e-8, pos.max()
    assert np.all(np.abs(h["s"][3] - tr["s"][:, 3]) <= 1e-7 * np.abs(w["mass"] * W.c) + 0)
    same = (h["naccept"] == tr["naccept"]) & (h["nreject"] == tr["nreject"])
    assert same.mean() >= 0.95, same.mean()


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
    rows, rm, nr, swt, swm = ens.rows()
    h = ens.download()
    assert h["nswitch"][0] == 2
    assert list(swm[0, :2]) == [0, 1]
    assert swt[0, 0] == 168.0
    assert abs(swt[0, 1] - 271.537802289) < 1e-8
