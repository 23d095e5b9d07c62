"""Pin the oracle's RKF45 tracer tableau (rapt_config.tableau = 1) to the
reference: tests/golden/rkf_golden.npz holds the reference's Particle.advance
and GuidingCenter.advance run with its own rkf() (rapt/rkf.py:13-143) per
output interval (tests/golden/make_rkf_golden.py).

On the x86 host where the fixtures were generated the oracle reproduces every
row bit for bit; the bound below leaves room for another host's libm. The
reference's step counts (accepted points returned by rkf, right-hand sides
counted on the closure) are matched exactly, and rkf's RuntimeError at hmin is
the RKF_HMIN status with no row added for the failing interval.
"""
import os

import numpy as np
import pytest

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "rkf_golden.npz"))
RKF_HMIN = 8

PARTICLE_CASES = [("p_earth", "EarthDipole", 0.5), ("p_earth_lo", "EarthDipole", 0.3),
                  ("p_var", "VarEarthDipole", 0.3)]
GC_CASES = [("g_tcb", 0, 2.0), ("g_tcb_lo", 0, 2.0), ("g_bc", 1, 2.0), ("g_nt", 2, 2.0)]


def _check_rows(rows, ref, width):
    assert rows.shape[0] == ref.shape[0] - 1, (rows.shape, ref.shape)
    got = rows[:, :width]
    scale = np.abs(ref[1:]).max(0)
    err = np.max(np.abs(got - ref[1:]) / np.where(scale > 0, scale, 1.0))
    assert err <= 1e-12, err
    return err


@pytest.mark.parametrize("case,field,delta", PARTICLE_CASES)
def test_rkf45_particle_matches_reference(oracle, case, field, delta):
    init = GOLD["%s_init" % case]
    tcur, raised, tol, hmin = GOLD["%s_meta" % case]
    f = oracle.field(field)
    cfg = oracle.config(tableau=1, rkf_tol=tol, rkf_hmin=hmin, cycres=20)
    tr = oracle.particle_new(init[0:3], init[3:6], 0.0, init[6], init[7])
    _, rows = oracle.advance(f, cfg, tr, delta)
    _check_rows(rows, GOLD["%s_rows" % case], 7)
    tot = GOLD["%s_counters" % case].sum(axis=0)
    assert (tr.nfcn, tr.nstep, tr.naccept, tr.nreject) == tuple(tot)
    assert tr.status == 0 and not raised
    assert tr.tcur == pytest.approx(tcur, rel=1e-15)


@pytest.mark.parametrize("case,eom,delta", GC_CASES)
def test_rkf45_guiding_centre_matches_reference(oracle, case, eom, delta):
    init = GOLD["%s_init" % case]
    tcur, raised, tol, hmin = GOLD["%s_meta" % case]
    f = oracle.field("DoubleDipole")
    cfg = oracle.config(tableau=1, rkf_tol=tol, rkf_hmin=hmin, gctimestep=1.0, gc_eom=eom)
    tr = oracle.gc_new_pa(f, init[0:3], init[3], init[4], 0.0, init[5], init[6])
    _, rows = oracle.advance(f, cfg, tr, delta)
    _check_rows(rows, GOLD["%s_rows" % case], 5)
    tot = GOLD["%s_counters" % case].sum(axis=0)
    assert (tr.nfcn, tr.nstep, tr.naccept, tr.nreject) == tuple(tot)
    assert tr.status == 0 and not raised and tr.tcur == tcur


def test_rkf45_hmin_raises_without_a_row(oracle):
    init = GOLD["g_hmin_init"]
    tcur, raised, tol, hmin = GOLD["g_hmin_meta"]
    assert raised == 1
    f = oracle.field("DoubleDipole")
    cfg = oracle.config(tableau=1, rkf_tol=tol, rkf_hmin=hmin, gctimestep=1.0)
    tr = oracle.gc_new_pa(f, init[0:3], init[3], init[4], 0.0, init[5], init[6])
    _, rows = oracle.advance(f, cfg, tr, 3.0)
    ref = GOLD["g_hmin_rows"]
    assert len(rows) == len(ref) - 1 == 0
    assert tr.status == RKF_HMIN
    # right-hand sides and attempts of the failing rkf call
    nfcn, nst = GOLD["g_hmin_counters"].sum(axis=0)[:2]
    assert (tr.nfcn, tr.nstep) == (nfcn, nst)
