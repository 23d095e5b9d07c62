"""Dense output of the guiding-centre advance on the GPU (rapt_config.dense_output)
against the oracle's restatement, its independence of launch boundaries, and
its use from Adaptive and the object API."""
import numpy as np
import pytest

from rapt_gb300 import workloads as W
from tests._util import gpu_ensemble, oracle_config, oracle_tracers, rel_state_error, within_envelope

pytestmark = pytest.mark.gpu


def _oracle(oracle, w, kind, delta, **over):
    f, _, tr = oracle_tracers(oracle, w, kind)
    cfg = oracle_config(oracle, w)
    for k, v in over.items():
        setattr(cfg, k, v)
    k = {"particle": 0, "gc": 1, "adaptive": 2}[kind]
    oracle.batch_advance(f, cfg, k, tr, delta)
    return tr


def test_dense_matches_oracle(oracle):
    """1,024 config-2 electrons, 0.05 s cadence, 5 s: same row times, states to
    rounding growth (bounded by the oracle's own 1e-15-perturbation envelope)."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 64))
    w["params"] = dict(w["params"], gctimestep=0.05)
    e = gpu_ensemble(w, "gc", max_rows=128, dense_output=1)
    e.advance("gc", 5.0)
    h = e.download()
    tr = _oracle(oracle, w, "gc", 5.0, dense=1)
    w2 = dict(w)
    w2["pos"] = w["pos"] * (1 + 1e-15)
    tp = _oracle(oracle, w2, "gc", 5.0, dense=1)
    assert np.all(h["status"] == 0) and np.all(tr["status"] == 0)
    assert np.array_equal(h["t_row"], tr["t"])
    pos, ppar = rel_state_error(h["s"], tr["s"], 4)
    env, _ = rel_state_error(tp["s"].T, tr["s"], 4)
    assert np.median(pos) < 1e-11, np.median(pos)
    within_envelope(pos, env)
    assert np.max(np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]) < 0.01
    rows, _, nr, _, _ = e.rows()
    t, times = 0.0, []  # the reference's row times: t += dt while t < t0 + delta
    while t < 5.0:
        t += 0.05
        times.append(t)
    assert np.all(nr == len(times))
    assert np.array_equal(rows[:, :len(times), 0], np.tile(times, (len(nr), 1)))


def test_dense_result_does_not_depend_on_launches():
    """A one-step budget per launch and a 20-row buffer (drained between
    resumes) give the default run's rows and states bit for bit."""
    from rapt_gb300 import _native as N
    w = W.subsample(W.config2(), np.arange(0, 65536, 256))
    w["params"] = dict(w["params"], gctimestep=0.02)
    a = gpu_ensemble(w, "gc", max_rows=512, dense_output=1)
    a.advance("gc", 2.0)
    ha = {k: np.copy(v) for k, v in a.download().items() if v is not None}
    ra, _, na, _, _ = a.rows()
    b = gpu_ensemble(w, "gc", max_rows=20, dense_output=1, max_steps_per_launch=1)
    b.advance("gc", 2.0)
    chunks = [[] for _ in range(len(w["mass"]))]
    for _ in range(10000):
        hb = b.download()
        rows, _, nr, _, _ = b.rows(reset=True)
        for i in range(len(nr)):
            chunks[i].append(rows[i, :nr[i]].copy())
        if not np.any(hb["status"] == N.ST["ROWS_FULL"]):
            break
        b.advance_resume("gc")
    for k in ("t_row", "naccept", "nreject", "nfcn", "status"):
        assert np.array_equal(hb[k], ha[k]), k
    assert np.array_equal(hb["s"], ha["s"])
    for i in range(len(chunks)):
        rb = np.concatenate(chunks[i])
        assert np.array_equal(rb, ra[i, :na[i]])


def test_dense_adaptive_matches_oracle(oracle):
    """Adaptive (config 5, compressed dipole with its induced E) with dense
    guiding-centre segments against the oracle: statuses, final modes and the
    times of the final rows."""
    w = W.subsample(W.config5(), np.arange(0, 1 << 20, 4096))
    e = gpu_ensemble(w, "adaptive", max_rows=2048, max_switch=64, dense_output=1)
    e.advance("adaptive", 20.0)
    h = e.download()
    tr = _oracle(oracle, w, "adaptive", 20.0, dense=1)
    ok = (h["status"] == 0) & (tr["status"] == 0)
    assert ok.mean() > 0.9
    assert np.mean(h["mode"][ok] == tr["mode"][ok]) > 0.95
    assert np.mean(np.isclose(h["t_row"][ok], tr["t"][ok], rtol=1e-9, atol=0)) > 0.9


def test_dense_object_api():
    import rapt_gb300 as R
    saved = dict(R.params)
    try:
        R.params.update(GCtimestep=0.01, solvertolerances=(1e-8, 1e-8))
        g = R.GuidingCenter([5 * R.Re, 0, 0], 1e7, pa=45, mass=R.m_el, charge=-R.e, field=R.fields.DoubleDipole())
        g.advance(0.5)
        R.params["dense output"] = True
        d = R.GuidingCenter([5 * R.Re, 0, 0], 1e7, pa=45, mass=R.m_el, charge=-R.e, field=R.fields.DoubleDipole())
        d.advance(0.5)
    finally:
        R.params.clear()
        R.params.update(saved)
    assert d.trajectory.shape == g.trajectory.shape
    assert np.allclose(d.trajectory[:, 0], g.trajectory[:, 0], rtol=1e-12)
    rel = np.abs(d.trajectory[:, 1:4] - g.trajectory[:, 1:4]).max() / np.abs(g.trajectory[:, 1:4]).max()
    assert rel < 1e-6, rel
