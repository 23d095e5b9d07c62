"""Grid fields on the GPU (rapt/fields.py:513-814): SciPy's linear
RegularGridInterpolator restated in the device kernels, checked bit for bit
against the reference's values in tests/golden/grid_golden.npz, and tracers in
a gridded field against those fixtures and the CPU oracle."""
import os

import numpy as np
import pytest

from tests._util import oracle_grid, rel_state_error, synth_grid, within_envelope
from tests.golden import grid_data as GD

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "grid_golden.npz"))
Re = GD.Re
m_pr, m_el, e = 1.672621777e-27, 9.10938291e-31, 1.602176565e-19
DERIVED4 = ["magB", "unitb", "gradB", "jacobianB", "curvature", "curlb", "dBdt", "dbdt", "lengthscale",
            "timescale"]
DERIVED3 = ["magB", "unitb", "gradB", "jacobianB", "curvature", "curlb", "lengthscale"]


def test_grid_values_bit_exact(ctx):
    from rapt_gb300 import _native as N
    for times, case in ((GD.TIMES, "g4"), ((0.0,), "g3")):
        t, x, y, z, B, E = GD.stacked(times)
        ctx.grid_set(t, x, y, z, B, E)
        p = GOLD[case + "_points"]
        assert np.array_equal(ctx.field_eval("B", p)[:, :3], GOLD[case + "_B"]), case
        assert np.array_equal(ctx.field_eval("E", p)[:, :3], GOLD[case + "_E"]), case
    # outside the grid (and past the last snapshot): NaN, where the reference raises
    t, x, y, z, B, E = GD.stacked(GD.TIMES)
    ctx.grid_set(t, x, y, z, B, None)
    out = ctx.field_eval("B", np.array([[8.0 + 1e-9, 5 * Re, 0, 0], [1.0, 9.6 * Re, 0, 0], [1.0, 5 * Re, 0, 4.1 * Re],
                                        [-1e-9, 5 * Re, 0, 0], [np.nan, 5 * Re, 0, 0]]))
    assert np.all(np.isnan(out[:, :3]))
    assert np.all(ctx.field_eval("E", GOLD["g4_points"][:5])[:, :3] == 0.0)  # no E array: zero
    # re-selecting the resident grid after another model
    ctx.set_field(N.MODEL_IDS["DoubleDipole"])
    ctx.set_field(N.MODEL_IDS["Grid"])
    assert np.array_equal(ctx.field_eval("B", GOLD["g4_points"])[:, :3], GOLD["g4_B"])


@pytest.mark.parametrize("case", ["g4", "g3"])
def test_grid_derived_quantities_match_reference(case):
    """Through the facade's _Field methods. Differences of B over 1e-3 Re inside a
    cell are differences of exactly interpolated values, so the device agrees
    with the reference to rounding of the last operations."""
    g = synth_grid(GD.TIMES if case == "g4" else (0.0,), static=(case == "g3"))
    names = DERIVED4 if case == "g4" else DERIVED3
    p = GOLD[case + "_dpoints"]
    got = np.column_stack([np.asarray(getattr(g, q)(p), float).reshape(len(p), -1) for q in names])
    ref = GOLD[case + "_derived"]
    if case == "g4":
        # the snapshots differ by a scale factor, so the field direction does not
        # turn: db/dt is central-difference rounding noise in both codes
        k = 1 + 3 + 3 + 9 + 1 + 3 + 1
        assert np.all(np.abs(got[:, k:k + 3]) < 1e-11) and np.all(np.abs(ref[:, k:k + 3]) < 1e-11)
        got, ref = np.delete(got, np.s_[k:k + 3], 1), np.delete(ref, np.s_[k:k + 3], 1)
    scale = np.maximum(np.abs(ref), 1e-300)
    err = np.where(got == ref, 0.0, np.abs(got - ref) / scale)
    assert err.max() <= 1e-9, (err.max(), np.unravel_index(np.argmax(err), err.shape))


def test_grid_rhs_match_oracle(ctx, oracle):
    """Particle and guiding-centre right-hand sides (the three equations of
    motion) at states inside the five-snapshot field, static False."""
    g = synth_grid(GD.TIMES, static=False)
    g.bind(ctx)
    of = oracle_grid(oracle, g)
    rng = np.random.default_rng(21)
    n = 64
    tp = np.column_stack([rng.uniform(0.5, 7.5, n), rng.uniform(4, 8, n) * Re, rng.uniform(-3, 3, n) * Re,
                          rng.uniform(-2.5, 2.5, n) * Re])
    v = rng.uniform(1e6, 1e7, n)
    d = rng.standard_normal((n, 3))
    vel = d / np.linalg.norm(d, axis=1, keepdims=True) * v[:, None]
    c = 299792458.0
    gam = 1 / np.sqrt(1 - v ** 2 / c ** 2)
    mom = (m_pr * gam)[:, None] * vel
    gm = np.sqrt(m_pr ** 2 + np.sum(mom * mom, 1) / c ** 2)
    cfg = oracle.config()
    ctx.set_config()
    out = ctx.rhs_eval(0, np.column_stack([tp, mom, gm]), m_pr, e)
    for i in range(n):
        o = oracle.particle_rhs(of, cfg, m_pr, e, gm[i], tp[i, 0], np.r_[tp[i, 1:], mom[i]])
        assert np.allclose(out[i], o, rtol=1e-12, atol=1e-300), (i, out[i], o)
    ppar = m_el * gam * v * rng.uniform(-1, 1, n)
    mu = rng.uniform(1e-16, 1e-13, n)
    st = np.column_stack([tp, ppar, np.zeros(n), np.zeros(n), mu])
    for eom in (0, 1, 2):
        ctx.set_config(gc_eom=eom)
        out = ctx.rhs_eval(1, st, m_el, -e, v)
        for i in range(n):
            o = oracle.gc_rhs(of, cfg, m_el, -e, mu[i], v[i], tp[i, 0], np.r_[tp[i, 1:], ppar[i]], eom=eom)
            vmax = np.max(np.abs(o[:3]))
            assert np.all(np.abs(out[i, :3] - o[:3]) <= 1e-9 * vmax), (eom, i, out[i], o)
            assert abs(out[i, 3] - o[3]) <= 1e-9 * abs(o[3]) + 1e-12 * abs(ppar[i]), (eom, i, out[i], o)
    ctx.set_config()


def _single(case, kind, g, delta, **cfg):
    from rapt_gb300 import Ensemble
    init = GOLD[case + "_init"]
    ens = Ensemble(g, 1, max_rows=512)
    ens.configure(rtol=1e-8, atol=1e-8, **cfg)
    if kind == "particle":
        ens.set_particles(init[None, 0:3], init[None, 3:6], 0.0, init[6], init[7])
    else:
        ens.set_guiding_centers(init[None, 0:3], init[3], pa=init[4], t0=init[7], mass=init[5], charge=init[6])
    ens.upload()
    ens.advance(kind, delta)
    h = ens.download()
    rows, _, nr, _, _ = ens.rows()
    return h, rows[0, :nr[0]]


def _envelope(oracle, f, case, kind, delta, **cfg):
    """Row-wise divergence of the oracle (which reproduces the reference's rows
    bit for bit) from itself when the start is scaled by 1 + 1e-15. Linear
    interpolation makes the right-hand sides' derivatives jump at every cell face
    and snapshot, where the error control of an rtol = 1e-8 run breaks down:
    rounding-level differences grow to ~1e-6 (protons over 8 s) and ~1e-3
    (guiding centres bouncing through the z cells over 7 s), in the reference
    as in any restatement of it."""
    init = GOLD[case + "_init"]
    c = oracle.config(rtol=1e-8, atol=1e-8, **cfg)
    out = []
    for eps in (0.0, 1e-15):
        if kind == "particle":
            tr = oracle.particle_new(init[0:3] * (1 + eps), init[3:6] * (1 + eps), 0.0, init[6], init[7])
        else:
            tr = oracle.gc_new_pa(f, init[0:3] * (1 + eps), init[3], init[4], init[7], init[5], init[6])
        out.append(oracle.advance(f, c, tr, delta)[1])
    a, b = out
    w = 7 if kind == "particle" else 5
    return np.abs(a[:, :w] - b[:, :w]) / np.abs(a[:, :w]).max(0)


def test_grid_trajectories_match_reference(oracle):
    """Rows of the device against the reference's rows: the largest difference
    within 30x the largest of the oracle's own sensitivity envelope (or 1e-9)."""
    from rapt_gb300 import _native as N
    cases = [("g4_p", "particle", GD.TIMES, False, 8.0, {}, N.ST["OUT_OF_GRID"]),
             ("g4_g", "gc", GD.TIMES, False, 7.0, {"gctimestep": 0.5}, 0),
             ("g3_p", "particle", (0.0,), True, 3.0, {}, 0),
             ("gout_p", "particle", (0.0,), True, 5.0, {}, N.ST["OUT_OF_GRID"])]
    for case, kind, times, static, delta, cfg, status in cases:
        g = synth_grid(times, static=static)
        h, rows = _single(case, kind, g, delta, **cfg)
        ref = GOLD[case + "_rows"][1:]
        # the last interval of g4_p passes the last snapshot, gout_p leaves through
        # x = 9.5 Re: the reference raises there and neither adds a row
        assert h["status"][0] == status and len(rows) == len(ref), (case, h["status"][0], len(rows), len(ref))
        env = _envelope(oracle, oracle_grid(oracle, g), case, kind, delta, **cfg)
        d = np.abs(rows[:, :ref.shape[1]] - ref) / np.abs(ref).max(0)
        assert d.max() <= max(1e-9, 30 * env.max()), (case, d.max(), env.max())


def test_grid_object_api_raises_like_the_reference():
    import rapt_gb300 as R
    g3 = synth_grid((0.0,))
    init = GOLD["gout_p_init"]
    saved = dict(R.params)
    try:
        R.params.update(solvertolerances=(1e-8, 1e-8))
        p = R.Particle(init[0:3], init[3:6], 0, init[6], init[7], g3)
        with pytest.raises(ValueError):
            p.advance(5.0)
    finally:
        R.params.clear()
        R.params.update(saved)
    ref = GOLD["gout_p_rows"]
    assert p.trajectory.shape == ref.shape
    assert np.allclose(p.trajectory, ref, rtol=1e-5, atol=0)  # envelope ~2e-7
    with pytest.raises(ValueError):
        g3.B([0.0, 9.6 * Re, 0, 0])


def _ensemble(n, rng):
    r = rng.uniform(4.5, 7.0, n) * Re
    phi = rng.uniform(-0.3, 0.3, n)
    pos = np.column_stack([r * np.cos(phi), r * np.sin(phi), rng.uniform(-0.5, 0.5, n) * Re])
    return pos


def _oracle_gc(oracle, of, pos, vg, pa, t0, delta, rtol, eps=0.0):
    cfg = oracle.config(rtol=rtol, atol=rtol, gctimestep=0.5)
    tr = oracle.tracers_from_structs([oracle.gc_new_pa(of, pos[i] * (1 + eps), vg[i], pa[i], t0, m_el, -e)
                                      for i in range(len(vg))])
    oracle.batch_advance(of, cfg, 1, tr, delta)
    return tr


def test_grid_ensembles_match_oracle(oracle):
    """2048 protons and 2048 electron guiding centres in the five-snapshot field
    (static False) against the oracle, tracer by tracer. Linear interpolation
    makes the right-hand sides' derivatives jump at every cell face, and there
    the rtol = 1e-8 error control turns rounding differences into ~1e-5 state
    differences (the oracle against itself perturbed by 1e-15): the device's
    differences are checked against that envelope as a distribution."""
    from rapt_gb300 import Ensemble
    rng = np.random.default_rng(11)
    g = synth_grid(GD.TIMES, static=False)
    of = oracle_grid(oracle, g)
    n = 2048
    # protons for 1.5 s
    pos = _ensemble(n, rng)
    v = rng.uniform(3e6, 1.5e7, n)
    d = rng.standard_normal((n, 3))
    vel = d / np.linalg.norm(d, axis=1, keepdims=True) * v[:, None]
    ens = Ensemble(g, n, max_rows=256)
    ens.configure(rtol=1e-8, atol=1e-8)
    ens.set_particles(pos, vel, 0.0, m_pr, e)
    ens.upload()
    ens.advance("particle", 1.5)
    h = ens.download()
    cfg = oracle.config(rtol=1e-8, atol=1e-8)
    trs = []
    for eps in (0.0, 1e-15):
        tr = oracle.tracers_from_structs([oracle.particle_new(pos[i] * (1 + eps), vel[i] * (1 + eps), 0.0, m_pr, e)
                                          for i in range(n)])
        oracle.batch_advance(of, cfg, 0, tr, 1.5)
        trs.append(tr)
    tr, tp = trs
    # tracers that graze a face may leave the grid in one code and not the other
    assert np.sum(h["status"] != tr["status"]) <= 2
    ok = (h["status"] == 0) & (tr["status"] == 0) & (tp["status"] == 0)
    assert ok.mean() > 0.9
    pos_err, mom_err = rel_state_error(h["s"][:, ok], tr["s"][ok], 6)
    env_pos, env_mom = rel_state_error(tp["s"][ok].T, tr["s"][ok], 6)
    within_envelope(pos_err, env_pos)
    within_envelope(mom_err, env_mom)
    # guiding centres from t0 = 0.5 s (the time-derivative stencil needs t - 1e-3 >= 0)
    pos = _ensemble(n, rng)
    vg = rng.uniform(1e7, 1e8, n)
    pa = rng.uniform(30, 90, n)
    ens = Ensemble(g, n, max_rows=64)
    ens.configure(rtol=1e-8, atol=1e-8, gctimestep=0.5)
    ens.set_guiding_centers(pos, vg, pa=pa, t0=0.5, mass=m_el, charge=-e)
    ens.upload()
    ens.advance("gc", 3.0)
    h = ens.download()
    tr = _oracle_gc(oracle, of, pos, vg, pa, 0.5, 3.0, 1e-8)
    tp = _oracle_gc(oracle, of, pos, vg, pa, 0.5, 3.0, 1e-8, eps=1e-15)
    assert np.sum(h["status"] != tr["status"]) <= 2
    ok = (h["status"] == 0) & (tr["status"] == 0) & (tp["status"] == 0)
    assert ok.mean() > 0.9
    pos_err, ppar_err = rel_state_error(h["s"][:, ok], tr["s"][ok], 4)
    env_pos, env_ppar = rel_state_error(tp["s"][ok].T, tr["s"][ok], 4)
    within_envelope(pos_err, env_pos)
    within_envelope(ppar_err, env_ppar)
    assert np.allclose(h["t_row"][ok], tr["t"][ok], rtol=1e-12, atol=0)


def test_grid_fp32_form_and_static_flag(oracle):
    """The FP32 form runs gridded fields through the FP64 field path: its error
    against a tight (rtol 1e-11) oracle run is of the order of the FP64 form's.
    The static flag (Grid leaves it True) drops the time-derivative terms."""
    from rapt_gb300 import Ensemble
    rng = np.random.default_rng(12)
    n = 1024
    pos = _ensemble(n, rng)
    vg = rng.uniform(1e7, 1e8, n)
    pa = rng.uniform(30, 90, n)
    res = {}
    for form, static in ((0, False), (1, False), (0, True)):
        g = synth_grid(GD.TIMES, static=static)
        ens = Ensemble(g, n, max_rows=64)
        ens.configure(rtol=1e-8, atol=1e-8, gctimestep=0.5, form=form)
        ens.set_guiding_centers(pos, vg, pa=pa, t0=0.5, mass=m_el, charge=-e)
        ens.upload()
        ens.advance("gc", 2.0)
        h = ens.download()
        res[(form, static)] = {"status": h["status"].copy(), "s": np.array(h["s"], copy=True)}
    truth = _oracle_gc(oracle, oracle_grid(oracle, synth_grid(GD.TIMES, static=False)), pos, vg, pa, 0.5, 2.0,
                       1e-11)
    a, b, c = res[(0, False)], res[(1, False)], res[(0, True)]
    ok = (a["status"] == 0) & (b["status"] == 0) & (truth["status"] == 0)
    assert ok.mean() > 0.9
    ea, _ = rel_state_error(a["s"][:, ok], truth["s"][ok], 4)
    eb, _ = rel_state_error(b["s"][:, ok], truth["s"][ok], 4)
    assert np.median(eb) <= 10 * np.median(ea), (np.median(eb), np.median(ea))
    okc = ok & (c["status"] == 0)
    assert np.any(np.abs(c["s"][3, okc] - a["s"][3, okc]) > 0)
