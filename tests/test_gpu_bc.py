"""BounceCenter and the second invariant on the GPU (rapt/BounceCenter.py,
rapt/flutils.py:65-229) against the CPU oracle's converged-integral mode (the
same algorithm) and the reference's values in tests/golden/bc_golden.npz."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "bc_golden.npz"))
Re = 6378137.0
NAMES = {0: "EarthDipole", 1: "DoubleDipole"}


def _bind(ctx, name):
    from rapt_gb300 import fields as F
    getattr(F, name)().bind(ctx)
    ctx.set_config()


def test_eye_matches_oracle_reference_and_dipole_formula(ctx, oracle):
    for mid in (0, 1):
        rows = GOLD["eye"][GOLD["eye"][:, 0] == mid]
        _bind(ctx, NAMES[mid])
        tpos = np.column_stack([np.zeros(len(rows)), rows[:, 1] * Re, np.zeros(len(rows)), np.zeros(len(rows))])
        got = ctx.bc_eval("eye", tpos, rows[:, 3], 0.03 * Re)[:, 0]
        f = oracle.field(NAMES[mid])
        conv = np.array([oracle.eye(f, tpos[i], rows[i, 3], quad=1) for i in range(len(rows))])
        assert np.all(np.abs(got - conv) <= 1e-10 * conv), np.max(np.abs(got - conv) / conv)
        ref = rows[:, 4]
        ok = np.isfinite(ref)  # the reference raises below 70 degrees
        assert np.all(rows[~ok, 2] < 70)
        assert np.all(np.abs(got[ok] - ref[ok]) <= 2e-5 * ref[ok])
        if mid == 0:
            assert np.all(np.abs(got - rows[:, 5]) <= 3e-6 * rows[:, 5])


def test_gradI_and_drift_match_oracle(ctx, oracle):
    for mid in (0, 1):
        rows = GOLD["gradI"][GOLD["gradI"][:, 0] == mid]
        _bind(ctx, NAMES[mid])
        tpos = np.column_stack([np.zeros(len(rows)), rows[:, 1:4]])
        got = ctx.bc_eval("gradI", tpos, rows[:, 4], 0.03 * Re)
        f = oracle.field(NAMES[mid])
        for i in range(len(rows)):
            conv = oracle.gradI(f, tpos[i], rows[i, 4], 0.03 * Re, quad=1)
            assert np.allclose(got[i], conv, rtol=1e-8, atol=1e-8 * np.abs(conv).max()), (got[i], conv)
            ref = rows[i, 5:8]
            assert np.allclose(got[i], ref, rtol=1e-3, atol=1e-3 * np.abs(ref).max()), (got[i], ref)
        cst = np.array([1.383e7, 1.0e-6, 1.672621777e-27, 1.602176565e-19])
        drift = ctx.bc_eval("drift", tpos, rows[:, 4], 0.03 * Re, cst)
        for i in range(len(rows)):
            o = oracle.bc_rhs(f, tpos[i], cst[2], cst[3], cst[0], rows[i, 4], 0.03 * Re, quad=1)
            assert np.allclose(drift[i], o, rtol=1e-8, atol=1e-8 * np.abs(o).max()), (drift[i], o)


def test_bounce_center_advance_matches_oracle_and_reference(ctx, oracle):
    for mid, v, pa, mass, charge, mu, bp, delta, tcur in GOLD["bc_cases"]:
        name = NAMES[int(mid)]
        _bind(ctx, name)
        ctx.set_config(rtol=1.49012e-8, atol=1.49012e-8)
        st = np.array([[0.0, 6 * Re, 0.0, 0.0, 0.0]])
        st, rows, nr, status, cnt = ctx.bc_advance(st, [[v, mu, mass, charge]], delta, 0.1, 0.03 * Re, 16)
        assert status[0] == 0 and nr[0] == 4
        got = rows[0, :4]
        f = oracle.field(name)
        ost = np.array([0.0, 6 * Re, 0.0, 0.0, 0.0])
        cfg = oracle.config(rtol=1.49012e-8, atol=1.49012e-8)
        s, orows, ocnt = oracle.bc_advance(f, cfg, ost, v, mu, mass, charge, delta, 0.1, 0.03 * Re, quad=1)
        assert s == 0
        assert np.allclose(got, orows, rtol=1e-9, atol=1e-9 * Re), np.abs(got - orows).max()
        assert np.array_equal(cnt[0], ocnt)
        ref = GOLD["bc_%s_rows" % name][1:]
        assert np.allclose(got[:, 0], ref[:, 0], rtol=1e-5, atol=0)  # dt from the bounce period (QAGS there)
        assert np.allclose(got[:, 1:], ref[:, 1:], rtol=1e-5, atol=1e-5 * Re), np.abs(got - ref).max()
        assert abs(st[0, 4] - tcur) <= 1e-5 * tcur


def test_bounce_center_object_api():
    import rapt_gb300 as R
    mid, v, pa, mass, charge, mu, bp, delta, tcur = GOLD["bc_cases"][1]
    b = R.BounceCenter([6 * Re, 0, 0], v, 0, pa, mass, charge, R.fields.DoubleDipole())
    assert abs(b.mu - mu) <= 1e-12 * mu
    b.advance(delta)
    ref = GOLD["bc_DoubleDipole_rows"]
    assert b.trajectory.shape == ref.shape
    assert np.allclose(b.trajectory[:, 1:], ref[:, 1:], rtol=1e-5, atol=1e-5 * Re)
    assert abs(b.tcur - tcur) <= 1e-5 * tcur
    b.advance(delta)  # continues from trajectory[-1]
    assert b.trajectory.shape == (9, 4) and np.all(np.diff(b.gety()) < 0)


def test_flutils_facade(oracle):
    """rapt_gb300.flutils: the half-bounce path against the reference's golden
    values and the oracle; eye and gradI through the object API."""
    import rapt_gb300 as R
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
    for mid, L, pa, phi, Bm, Sb in gold["bounce_halfpath"]:
        name = NAMES.get(int(mid))
        if name is None:
            continue
        fld = getattr(R.fields, name)()
        tpos = np.array([0.0, L * Re * np.cos(np.radians(phi)), L * Re * np.sin(np.radians(phi)), 0.0])
        got = R.flutils.halfbouncepath(tpos, fld, Bm)
        conv = oracle.halfbouncepath(oracle.field(name), tpos, Bm, quad=1)[0]
        assert abs(got - conv) <= 1e-10 * conv and abs(got - Sb) <= 1e-5 * Sb, (got, conv, Sb)
    rows = GOLD["eye"][(GOLD["eye"][:, 0] == 0) & np.isfinite(GOLD["eye"][:, 4])]
    fld = R.fields.EarthDipole()
    for mid, L, eqpa, Bm, ref, dip in rows:
        tpos = np.array([0.0, L * Re, 0.0, 0.0])
        assert abs(R.flutils.eye(tpos, fld, Bm) - ref) <= 2e-5 * ref
        assert abs(R.flutils.eye(tpos, fld, Bm, usedipole=True) - dip) <= 1e-11 * dip
    mid, x, y, z, Bm, gx, gy, gz = GOLD["gradI"][0]
    g = R.flutils.gradI(np.array([0.0, x, y, z]), fld, Bm)
    assert np.allclose(g, [gx, gy, gz], rtol=1e-3, atol=1e-3 * abs(gx))


def test_mirror_field_and_eye_error():
    """rapt_gb300.utils.Bm (|B| from the device) against the closed dipole form
    dipoleBm at the Earth dipole's equator, and flutils.eye_error as the
    difference of the field-line and dipole-form invariants."""
    import rapt_gb300 as R
    fld = R.fields.EarthDipole()
    for L, pa in ((3.0, 30.0), (5.5, 60.0), (7.0, 85.0)):
        tpos = np.array([0.0, L * Re, 0.0, 0.0])
        assert abs(R.utils.Bm(tpos, pa, fld) / R.utils.dipoleBm(L, pa) - 1) < 1e-12, (L, pa)
    rows = GOLD["eye"][(GOLD["eye"][:, 0] == 0) & np.isfinite(GOLD["eye"][:, 4])]
    for mid, L, eqpa, Bm, ref, dip in rows:
        tpos = np.array([0.0, L * Re, 0.0, 0.0])
        err = R.flutils.eye_error(tpos, fld, Bm)
        want = R.flutils.eye(tpos, fld, Bm) - R.flutils.eye(tpos, fld, Bm, usedipole=True)
        assert err == want and abs(err) <= 2e-5 * ref + 1e-11 * dip, (err, want, ref, dip)
