"""The FP32 form (float-float stages, FP32 stencil differences without
cancellation, FP64 time / error norm / step size) against the CPU oracle and
against the plain form."""
import numpy as np
import pytest

from rapt_gb300 import workloads as W
from tests._util import gpu_ensemble, oracle_config, oracle_tracers, rel_state_error, sensitivity_envelope

pytestmark = pytest.mark.gpu
FP32 = 1


def test_fp32_gc_matches_oracle():
    """Config 2 subsample (64 electrons), 10 s. The FP32 form takes the plain
    controller's steps (step counts within 1 %) and differs from the FP64
    oracle by rounding: the float-float stages and the FP32 stencil
    differences (~1e-7 relative noise on grad|B| and curl b). Yardstick: the
    oracle's own integration error against an rtol = atol = 1e-12 oracle run.
    The FP32 form must stay far inside it (median and maximum below a tenth)
    and be as accurate against the exact solution as the oracle itself."""
    O = oracle_mod()
    w = W.subsample(W.config2(), np.arange(0, 65536, 1024))
    f, cfg, tr = oracle_tracers(O, w, "gc")
    O.batch_advance(f, cfg, 1, tr, 10.0)
    _, _, ex = oracle_tracers(O, w, "gc")
    O.batch_advance(f, oracle_config(O, w, rtol=1e-12, atol=1e-12), 1, ex, 10.0)
    ens = gpu_ensemble(w, "gc", max_rows=16, form=FP32)
    ens.advance("gc", 10.0)
    h = ens.download()
    assert np.all(h["status"] == 0)
    pos, _ = rel_state_error(h["s"], tr["s"], 4)
    own, _ = rel_state_error(tr["s"].T, ex["s"], 4)
    vs_exact, _ = rel_state_error(h["s"], ex["s"], 4)
    assert np.median(pos) < 0.1 * np.median(own) and pos.max() < 0.1 * own.max(), (pos, own)
    assert np.median(pos) < 5e-7 and pos.max() < 5e-6, (np.median(pos), pos.max())
    assert np.median(vs_exact) <= 1.05 * np.median(own) and vs_exact.max() <= 1.05 * own.max(), (vs_exact, own)
    dpp = np.abs(h["s"][3] - tr["s"][:, 3]) / (w["mass"] * W.c)
    assert dpp.max() < 1e-4, dpp.max()
    assert np.max(np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]) < 0.01


def test_fp32_particle_config4_sample():
    """Config 4 subsample (256 protons and electrons, 50 gyro-periods): relative
    final-state error and energy drift against the FP64 oracle."""
    O = oracle_mod()
    w = W.subsample(W.config4(), np.arange(0, 1048576, 4096))
    tr, env_pos, env_mom = sensitivity_envelope(O, w, "particle", w["delta"], rel=3e-14)
    ens = gpu_ensemble(w, "particle", max_rows=1024, form=FP32)
    ens.advance("particle", w["delta"])
    h = ens.download()
    assert np.all(h["status"] == 0)
    pos, mom = rel_state_error(h["s"], tr["s"], 6)
    # float-float keeps ~48 bits: bounded by the oracle's own divergence under a
    # 3e-14 relative start perturbation, floor 1e-9; a start perturbation does
    # not bound per-operation differences along the few chaotic orbits, hence 97 %
    within = pos <= np.maximum(1e-9, 100 * env_pos)
    assert within.mean() >= 0.97, (within.mean(), pos.max())
    assert np.median(pos) < 1e-11 and np.median(mom) < 1e-9, (np.median(pos), np.median(mom))
    p0 = np.linalg.norm(w["mass"][:, None] * w["vel"] / np.sqrt(1 - np.sum(w["vel"] ** 2, 1) / W.c ** 2)[:, None],
                        axis=1)
    drift_gpu = np.abs(np.linalg.norm(h["s"][3:6].T, axis=1) / p0 - 1)
    drift_orc = np.abs(np.linalg.norm(tr["s"][:, 3:6], axis=1) / p0 - 1)
    assert np.median(drift_gpu) <= 2 * np.median(drift_orc) + 1e-12


def test_fp32_adaptive_matches_plain():
    """Adaptive in the Harris sheet (512 protons of config 3, a tenth of their
    durations): the FP32 form (float-float particle and guiding-centre
    segments) against the plain form -- switch counts, final modes and final
    positions follow the plain form's."""
    w = W.subsample(W.config3(), np.arange(0, 262144, 512))
    d = w["delta"] / 10
    res = {}
    for form in (0, FP32):
        e = gpu_ensemble(w, "adaptive", max_rows=4096, max_switch=64, form=form)
        st = e.advance("adaptive", d)
        res[form] = (st, e.download())
    (sa, ha), (sb, hb) = res[0], res[FP32]
    assert np.all(ha["status"] == 0) and np.all(hb["status"] == 0)
    assert abs(sb["switches"] - sa["switches"]) <= 0.02 * sa["switches"] + 2, (sa["switches"], sb["switches"])
    same = ha["mode"] == hb["mode"]
    assert same.mean() >= 0.95, same.mean()
    pos = np.linalg.norm(ha["s"][:3] - hb["s"][:3], axis=0) / np.linalg.norm(ha["s"][:3], axis=0)
    assert np.median(pos[same]) < 1e-6, np.median(pos[same])


@pytest.mark.parametrize("name", ["DoubleDipole", "EarthDipole"])
def test_fp32_rhs_matches_plain(ctx, name):
    """The FP32 form's right-hand sides against the plain FP64 ones at random
    states (L 3-8, |latitude| <= 45 deg). Guiding centres (Tao-Chan-Brizard):
    the velocity to 1e-8 of the speed (the drifts, up to ~1e-2 of it for
    10 MeV electrons, carry the FP32 stencil's ~1e-7 relative noise); the
    mirror force dp_par/dt, whose grad|B| comes from the FP32 stencil
    differences formed without cancellation, to 5e-6 of mu |grad B| / gamma and
    without bias (mean relative difference below 1e-7). A stencil that took
    the difference of two FP32 samples would be off by ~1e-3 of the gradient.
    Particles: float-float throughout, 1e-12."""
    from rapt_gb300 import fields as F
    fld = getattr(F, name)()
    fld.bind(ctx)
    rng = np.random.default_rng(11)
    n = 4096
    L = rng.uniform(3, 8, n)
    lat = rng.uniform(-np.pi / 4, np.pi / 4, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    pos = (L * W.Re)[:, None] * np.column_stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi),
                                                 np.sin(lat)])
    tp = np.column_stack([np.zeros(n), pos])
    m, q = W.m_el, -W.e
    ek = 10 ** rng.uniform(-1, 1, n) * W.MeV * W.e
    gam = 1 + ek / (m * W.c ** 2)
    v = W.c * np.sqrt(1 - 1 / gam ** 2)
    p = gam * m * v
    pa = np.radians(rng.uniform(15, 85, n))
    magB = ctx.field_eval("magB", tp)[:, 0]
    gB = np.linalg.norm(ctx.field_eval("gradB", tp)[:, :3], axis=1)
    mu = (p * np.sin(pa)) ** 2 / (2 * m * magB)
    ppar = p * np.cos(pa) * rng.choice([-1.0, 1.0], n)
    st = np.column_stack([tp, ppar, np.zeros(n), np.zeros(n), mu])
    try:
        ctx.set_config(form=0)
        ref = ctx.rhs_eval(1, st, m, q, v)
        ctx.set_config(form=FP32)
        got = ctx.rhs_eval(1, st, m, q, v)
        dv = np.linalg.norm(got[:, :3] - ref[:, :3], axis=1) / v
        assert dv.max() < 1e-8, (name, dv.max())
        scale = mu * gB / gam
        dp = (got[:, 3] - ref[:, 3]) / scale
        assert np.abs(dp).max() < 5e-6 and abs(dp.mean()) < 1e-7, (name, np.abs(dp).max(), dp.mean())
        # particles: the float-float Lorentz force
        vel = rng.standard_normal((n, 3))
        vel *= (v / np.linalg.norm(vel, axis=1))[:, None]
        mom = (gam * m)[:, None] * vel
        stp = np.column_stack([tp, mom, gam * m])
        ctx.set_config(form=0)
        refp = ctx.rhs_eval(0, stp, m, q)
        ctx.set_config(form=FP32)
        gotp = ctx.rhs_eval(0, stp, m, q)
        assert np.allclose(gotp, refp, rtol=1e-12, atol=1e-12 * np.abs(refp).max(axis=0)), name
    finally:
        ctx.set_config()


def oracle_mod():
    from oracle import oracle as O
    O.lib()
    return O
