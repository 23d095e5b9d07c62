"""The RKF45 tracer tableau (rapt_config.tableau = 1, rapt/rkf.py:13-143) on the
GPU: the reference's own rkf() driven tracers (tests/golden/rkf_golden.npz),
ensembles against the oracle, and rkf's RuntimeError at hmin."""
import numpy as np
import pytest

from rapt_gb300 import Ensemble, fields as F, workloads as W
from tests._util import gpu_ensemble, rel_state_error, sensitivity_envelope
from tests.test_rkf_oracle import GC_CASES, GOLD, PARTICLE_CASES, RKF_HMIN

pytestmark = pytest.mark.gpu


def _rows_close(rows, ref, width, rtol):
    assert rows.shape[0] == ref.shape[0] - 1, (rows.shape, ref.shape)
    scale = np.abs(ref[1:]).max(0)
    err = np.max(np.abs(rows[:, :width] - ref[1:]) / np.where(scale > 0, scale, 1.0))
    assert err <= rtol, err


@pytest.mark.parametrize("case,field,delta", PARTICLE_CASES)
def test_rkf45_particle_matches_reference(case, field, delta):
    init = GOLD["%s_init" % case]
    tcur, _, tol, hmin = GOLD["%s_meta" % case]
    ens = Ensemble(getattr(F, field)(), 1, max_rows=64)
    ens.configure(tableau=1, rkf_tol=tol, rkf_hmin=hmin, cyclotronresolution=20)
    ens.set_particles(init[None, 0:3], init[None, 3:6], 0.0, init[6], init[7])
    ens.upload()
    ens.advance("particle", delta)
    h = ens.download()
    rows, _, nr, _, _ = ens.rows()
    assert h["status"][0] == 0
    _rows_close(rows[0, :nr[0]], GOLD["%s_rows" % case], 7, 1e-9)
    nacc = GOLD["%s_counters" % case][:, 2].sum()
    assert abs(h["naccept"][0] - nacc) <= max(1, 0.01 * nacc), (h["naccept"][0], nacc)
    assert h["tcur"][0] == pytest.approx(tcur, rel=1e-12)


@pytest.mark.parametrize("case,eom,delta", GC_CASES)
def test_rkf45_guiding_centre_matches_reference(case, eom, delta):
    init = GOLD["%s_init" % case]
    tcur, _, tol, hmin = GOLD["%s_meta" % case]
    ens = Ensemble(F.DoubleDipole(), 1, max_rows=8)
    ens.configure(tableau=1, rkf_tol=tol, rkf_hmin=hmin, gctimestep=1.0, gc_eom=eom)
    ens.set_guiding_centers(init[None, 0:3], init[3], pa=init[4], t0=0.0, mass=init[5], charge=init[6])
    ens.upload()
    ens.advance("gc", delta)
    h = ens.download()
    rows, _, nr, _, _ = ens.rows()
    assert h["status"][0] == 0
    _rows_close(rows[0, :nr[0]], GOLD["%s_rows" % case], 5, 1e-9)
    nacc = GOLD["%s_counters" % case][:, 2].sum()
    assert abs(h["naccept"][0] - nacc) <= max(1, 0.01 * nacc), (h["naccept"][0], nacc)
    assert h["tcur"][0] == tcur


def test_rkf45_hmin_stops_without_a_row():
    """rkf raises RuntimeError where the step falls below hmin (rkf.py:136-139):
    the tracer stops with RKF_HMIN and the failing interval adds no row."""
    init = GOLD["g_hmin_init"]
    _, raised, tol, hmin = GOLD["g_hmin_meta"]
    ens = Ensemble(F.DoubleDipole(), 1, max_rows=8)
    ens.configure(tableau=1, rkf_tol=tol, rkf_hmin=hmin, gctimestep=1.0)
    ens.set_guiding_centers(init[None, 0:3], init[3], pa=init[4], t0=0.0, mass=init[5], charge=init[6])
    ens.upload()
    ens.advance("gc", 3.0)
    h = ens.download()
    _, _, nr, _, _ = ens.rows()
    assert raised == 1 and h["status"][0] == RKF_HMIN and nr[0] == 0
    nfcn, nst = GOLD["g_hmin_counters"].sum(axis=0)[:2]
    assert h["nfcn"][0] == nfcn


def _ensemble_vs_oracle(oracle, w, kind, delta, **over):
    tr, env_pos, env_mom = sensitivity_envelope(oracle, w, kind, delta, **over)
    ens = gpu_ensemble(w, kind, max_rows=4096, **over)
    ens.advance(kind, delta)
    h = ens.download()
    assert np.all(h["status"] == 0), np.unique(h["status"], return_counts=True)
    n = 6 if kind == "particle" else 4
    pos, mom = rel_state_error(h["s"], tr["s"], n)
    assert np.all(pos <= np.maximum(1e-9, 100 * env_pos)), pos.max()
    assert np.median(pos) < 1e-11, np.median(pos)
    steps_rel = np.abs(h["naccept"] - tr["naccept"]) / tr["naccept"]
    assert steps_rel.max() < 0.01, steps_rel.max()
    return h, tr


def test_rkf45_config1_particles(oracle):
    """Config 1 (256 protons, EarthDipole) for 2 s on the RKF45 tableau."""
    w = W.config1()
    _ensemble_vs_oracle(oracle, w, "particle", 2.0, tableau=1, rkf_tol=1e-3)


def test_rkf45_config2_guiding_centres(oracle):
    """256 electrons of config 2 (DoubleDipole, TCB) for 3 s on the RKF45 tableau."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 256))
    _ensemble_vs_oracle(oracle, w, "gc", 3.0, tableau=1, rkf_tol=1e-2)
