"""Grid fields (rapt/fields.py:513-814) in the CPU oracle, pinned against SciPy's
RegularGridInterpolator and against tests/golden/grid_golden.npz, written by
tests/golden/make_grid_golden.py from the unmodified reference's Grid. Also the
facade's host-side Grid logic (parsing, bounds errors, device binding rules)."""
import os

import numpy as np
import pytest

from tests.golden import grid_data as GD

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "grid_golden.npz"))
Re = GD.Re
DERIVED4 = ["magB", "unitb", "gradB", "jacobianB", "curvature", "curlb", "dBdt", "dbdt", "lengthscale",
            "timescale"]
DERIVED3 = ["magB", "unitb", "gradB", "jacobianB", "curvature", "curlb", "lengthscale"]


def grid4(oracle):
    t, x, y, z, B, E = GD.stacked(GD.TIMES)
    return oracle.grid_field(t, x, y, z, B, E, static=False)


def grid3(oracle):
    t, x, y, z, B, E = GD.stacked((0.0,))
    return oracle.grid_field(t, x, y, z, B, E, static=True)


def test_interpolation_matches_scipy_bit_for_bit(oracle):
    from scipy.interpolate import RegularGridInterpolator as RGI
    rng = np.random.default_rng(5)
    t = np.array([0.0, 0.7, 2.0, 2.1, 5.0])
    x = np.sort(rng.uniform(-3, 3, 9))
    y = np.linspace(-1, 1, 4)
    z = np.cumsum(rng.uniform(0.1, 1, 6))
    B = rng.normal(size=(5, 9, 4, 6, 3))
    n = 2000
    p = np.column_stack([rng.uniform(t[0], t[-1], n), rng.uniform(x[0], x[-1], n), rng.uniform(y[0], y[-1], n),
                         rng.uniform(z[0], z[-1], n)])
    p[:100, 0] = rng.choice(t, 100)
    p[100:200, 1] = rng.choice(x, 100)
    p[200:300, 3] = rng.choice(z, 100)
    p[300] = [t[-1], x[-1], y[-1], z[-1]]
    p[301] = [t[0], x[0], y[0], z[0]]
    f = oracle.grid_field(t, x, y, z, B, None, static=False)
    got = np.array([oracle.field_eval(f, "B", q) for q in p])
    for c in range(3):
        assert np.array_equal(got[:, c], RGI((t, x, y, z), B[..., c])(p))
    f1 = oracle.grid_field(t[:1], x, y, z, B[:1], None)
    got = np.array([oracle.field_eval(f1, "B", q) for q in p])
    for c in range(3):
        assert np.array_equal(got[:, c], RGI((x, y, z), B[0, ..., c])(p[:, 1:]))
    # outside any axis (or the time span) the reference raises; the oracle gives NaN
    for q in ([t[-1] + 1e-9, 0, 0, z[0]], [1.0, x[-1] * (1 + 1e-12) + 1e-12, 0, z[0]], [1.0, 0, 1.5, z[0]],
              [1.0, 0, 0, np.nan]):
        assert np.all(np.isnan(oracle.field_eval(f, "B", q)))


def test_grid_values_match_reference(oracle):
    f = grid4(oracle)
    p = GOLD["g4_points"]
    assert np.array_equal(np.array([oracle.field_eval(f, "B", q) for q in p]), GOLD["g4_B"])
    assert np.array_equal(np.array([oracle.field_eval(f, "E", q) for q in p]), GOLD["g4_E"])
    f = grid3(oracle)
    p = GOLD["g3_points"]
    assert np.array_equal(np.array([oracle.field_eval(f, "B", q) for q in p]), GOLD["g3_B"])
    assert np.array_equal(np.array([oracle.field_eval(f, "E", q) for q in p]), GOLD["g3_E"])


@pytest.mark.parametrize("case", ["g4", "g3"])
def test_grid_derived_quantities_match_reference(oracle, case):
    f = grid4(oracle) if case == "g4" else grid3(oracle)
    names = DERIVED4 if case == "g4" else DERIVED3
    got = np.array([np.concatenate([np.ravel(oracle.field_eval(f, q, p)) for q in names])
                    for p in GOLD[case + "_dpoints"]])
    ref = GOLD[case + "_derived"]
    assert got.shape == ref.shape
    scale = np.maximum(np.abs(ref), 1e-300)
    err = np.where(got == ref, 0.0, np.abs(got - ref) / scale)
    assert err.max() <= 1e-12, err.max()


def _run(oracle, f, case, kind, delta, **cfgkw):
    init = GOLD[case + "_init"]
    cfg = oracle.config(rtol=1e-8, atol=1e-8, **cfgkw)
    if kind == "particle":
        tr = oracle.particle_new(init[0:3], init[3:6], 0.0, init[6], init[7])
    else:
        tr = oracle.gc_new_pa(f, init[0:3], init[3], init[4], init[7], init[5], init[6])
    raised, rows = oracle.advance(f, cfg, tr, delta)
    return tr, rows


def test_grid_trajectories_match_reference(oracle):
    ST = oracle.ST
    # proton through two window moves; its last interval passes the last snapshot
    f = grid4(oracle)
    tr, rows = _run(oracle, f, "g4_p", "particle", 8.0)
    ref = GOLD["g4_p_rows"]
    assert GOLD["g4_p_raised"][0] == 1 and tr.status == ST["OUT_OF_GRID"]
    assert len(rows) + 1 == len(ref)  # the reference's trajectory includes the initial row
    assert np.allclose(rows, ref[1:], rtol=1e-10, atol=0)
    # electron guiding centre, static False
    tr, rows = _run(oracle, f, "g4_g", "gc", 7.0, gctimestep=0.5)
    ref = GOLD["g4_g_rows"]
    assert GOLD["g4_g_raised"][0] == 0 and tr.status == ST["OK"]
    assert np.allclose(rows[:, :5], ref[1:], rtol=1e-10, atol=0)
    # one snapshot, static True
    f = grid3(oracle)
    tr, rows = _run(oracle, f, "g3_p", "particle", 3.0)
    ref = GOLD["g3_p_rows"]
    assert tr.status == ST["OK"]
    assert np.allclose(rows, ref[1:], rtol=1e-10, atol=0)
    # a proton gyrating out through the x = 9.5 Re face
    tr, rows = _run(oracle, f, "gout_p", "particle", 5.0)
    ref = GOLD["gout_p_rows"]
    assert GOLD["gout_p_raised"][0] == 1 and tr.status == ST["OUT_OF_GRID"]
    assert len(rows) + 1 == len(ref) and np.allclose(rows, ref[1:], rtol=1e-10, atol=0)
    # no row for the failing interval: the state is the last row's
    assert np.array_equal(np.r_[tr.t, list(tr.s)], ref[-1])


# ---- facade host logic (no device calls)

def test_facade_grid_parses_and_checks_bounds():
    from tests._util import synth_grid
    g = synth_grid(GD.TIMES)
    assert g.has_device_impl() and g.static and g.gradientstepsize == 1e-3 * Re
    assert g._B.shape == (5, 29, 33, 25, 3) and g._E is not None and g.files == []
    assert (g.t0, g.t1, g.t2) == (0.0, 2.0, 4.0)
    with pytest.raises(ValueError):
        g._check_bounds([8.5, 5 * Re, 0, 0])
    with pytest.raises(ValueError):
        g._check_bounds([1.0, 10 * Re, 0, 0])
    g._check_bounds([1.0, 5 * Re, 0, 0])
    g1 = synth_grid((0.0,))
    g1._check_bounds([1e9, 5 * Re, 0, 0])  # one snapshot: time is not an axis
    with pytest.raises(ValueError):
        g1._check_bounds([0.0, 5 * Re, 5 * Re, 0])

    from rapt_gb300 import fields as F

    class Tweaked(type(g)):
        def B(self, tpos):
            return self.Bgrid(tpos) + 1e-9

    assert not Tweaked(GD.TIMES).has_device_impl()
    with pytest.raises(AssertionError):  # fields.py:576
        F.Grid.__init__(type(g).__new__(type(g)), [])


def test_grid_adaptive_matches_reference(oracle):
    """Adaptive protons in the five-snapshot field (static False) that switch
    between particle and guiding-centre modes: the switch sequence, the switch
    times and the final state against the reference."""
    f = grid4(oracle)
    cfg = oracle.config(rtol=1e-8, atol=1e-8, gctimestep=0.5, cycres=10)
    for case in ("ga0", "ga1"):
        init = GOLD[case + "_init"]
        tr = oracle.adaptive_init(f, cfg, init[0:3], init[3:6], 0.5, init[6], init[7])
        modes = GOLD[case + "_modes"]
        assert tr.mode == modes[0]
        rc, rows, rmode, swt, swm = oracle.adaptive_advance(f, cfg, tr, 3.0)
        assert tr.status == 0 and list(swm) == list(modes[1:]) and tr.mode == modes[-1], (case, list(swm))
        assert np.allclose(swt, GOLD[case + "_t0s"][1:], rtol=1e-12, atol=0)
        fin = GOLD[case + "_final"]
        n = 7 if tr.mode == 0 else 5
        assert np.allclose([tr.t, *tr.s[:n - 1]], fin[:n], rtol=1e-9), (case, [tr.t, *tr.s[:n - 1]], fin[:n])
