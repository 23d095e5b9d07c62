"""The bounce period on the GPU (field-line trace, quadratic spline, brentq,
QAGS) and the bounce-period cadence of GuidingCenter.advance (GCtimestep = 0),
against the reference's golden values and the CPU oracle."""
import os

import numpy as np
import pytest

from rapt_gb300 import workloads as W
from tests._util import gpu_ensemble, oracle_tracers, rel_state_error

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
Re = 6378137.0


def test_bounce_period_matches_reference(ctx, oracle):
    from rapt_gb300 import fields as F
    F.DoubleDipole().bind(ctx)
    ctx.set_config()
    rows = GOLD["bounce_gc_period"]  # pos(3), v, pa, mass, charge, T_b
    f = oracle.field("DoubleDipole")
    st = []
    for r in rows:  # GuidingCenter.__init__ state (ppar, mu) as the reference builds it
        g = oracle.gc_new_pa(f, r[0:3], r[3], r[4], 0.0, r[5], r[6])
        st.append([0.0, *r[0:3], g.s[3], g.mu, r[5]])
    got = ctx.gc_bounce_period(np.array(st))
    # the device integrates the half-bounce path to convergence; the reference's
    # QAGS at epsrel 1e-4 is within ~5e-6 of that
    assert np.allclose(got, rows[:, 7], rtol=1e-5, atol=0), (got, rows[:, 7])


def test_bounce_period_matches_oracle_on_ensemble(ctx, oracle):
    """512 guiding centres of config 2 (double dipole): device against the
    oracle's converged-integral mode (the same algorithm)."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 128))
    f, cfg, tr = oracle_tracers(oracle, w, "gc")
    ref = np.array([oracle.gc_bounceperiod(f, _tracer(oracle, tr, i), quad=1) for i in range(len(tr))])
    from rapt_gb300 import fields as F
    F.DoubleDipole().bind(ctx)
    ctx.set_config()
    st = np.column_stack([tr["t"], tr["s"][:, 0:4], tr["mu"], tr["mass"]])
    got = ctx.gc_bounce_period(st)
    rel = np.abs(got - ref) / ref
    assert np.all(np.isfinite(got)) and np.median(rel) < 1e-12 and rel.max() < 1e-8, (np.median(rel), rel.max())


def _tracer(oracle, arr, i):
    import ctypes as C
    t = oracle.Tracer()
    C.memmove(C.byref(t), arr[i:i + 1].ctypes.data, C.sizeof(t))
    return t


def test_bounce_cadence_advance_matches_oracle(oracle):
    """GuidingCenter.advance with GCtimestep = 0 (rows every T_b / 10), 64
    electrons of config 2 for 2 s: final state and step counts against the oracle."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 1024))
    w["params"] = dict(w["params"], gctimestep=0.0)
    f, _, tr = oracle_tracers(oracle, w, "gc")
    from tests._util import oracle_config
    cfg = oracle_config(oracle, w, bounce_quad=1)
    oracle.batch_advance(f, cfg, 1, tr, 2.0)
    e = gpu_ensemble(w, "gc", max_rows=512)
    e.advance("gc", 2.0)
    h = e.download()
    assert np.all(h["status"] == 0) and np.all(tr["status"] == 0)
    assert np.allclose(h["t_row"], tr["t"], rtol=1e-9, atol=0)
    pos, _ = rel_state_error(h["s"], tr["s"], 4)
    assert np.median(pos) < 1e-10 and pos.max() < 1e-6, (np.median(pos), pos.max())
    assert np.max(np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]) < 0.01


def test_bounce_cadence_golden_trajectory():
    """The reference's GuidingCenter.advance(0.5) with GCtimestep = 0 through the
    object API."""
    import rapt_gb300 as R
    init = GOLD["traj_gbounce_init"]
    ref = GOLD["traj_gbounce_rows"]
    saved = dict(R.params)
    try:
        R.params.update(solvertolerances=(1e-8, 1e-8), GCtimestep=0)
        g = R.GuidingCenter(init[0:3], init[3], pa=init[4], t0=0, mass=init[5], charge=init[6],
                            field=R.fields.DoubleDipole())
        assert abs(g.bounceperiod() - 10 * ref[1, 0]) < 1e-5 * ref[1, 0] * 10
        g.advance(0.5)
    finally:
        R.params.clear()
        R.params.update(saved)
    got = g.trajectory
    # row times follow the bounce period (within the reference's quad error)
    assert got.shape == ref.shape
    assert np.allclose(got[:, 0], ref[:, 0], rtol=1e-5, atol=0)
    d = np.linalg.norm(got[:, 1:4] - ref[:, 1:4], axis=1) / np.linalg.norm(ref[:, 1:4], axis=1)
    assert d.max() < 1e-4, d.max()


def test_bounce_cadence_fp32_and_adaptive(oracle):
    """The FP32 form and Adaptive runs take the bounce-period cadence too."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 2048))
    w["params"] = dict(w["params"], gctimestep=0.0)
    a = gpu_ensemble(w, "gc", max_rows=512)
    a.advance("gc", 1.0)
    b = gpu_ensemble(w, "gc", max_rows=512, form=1)
    b.advance("gc", 1.0)
    ha, hb = a.download(), b.download()
    assert np.all(hb["status"] == 0)
    assert np.allclose(ha["t_row"], hb["t_row"], rtol=1e-9, atol=0)
    w5 = W.subsample(W.config5(), np.arange(0, 1 << 20, 32768))
    w5["params"] = dict(w5["params"], gctimestep=0.0)
    e = gpu_ensemble(w5, "adaptive", max_rows=4096, max_switch=64)
    e.advance("adaptive", 5.0)
    h = e.download()
    assert np.all((h["status"] == 0) | (h["status"] == 6)), np.unique(h["status"])
