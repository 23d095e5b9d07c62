"""The object API (Particle / GuidingCenter / Adaptive) against trajectories the
unmodified reference produced (tests/golden/golden.npz)."""
import os

import numpy as np
import pytest

import rapt_gb300 as R

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


@pytest.fixture
def params():
    saved = dict(R.params)
    yield R.params
    R.params.clear()
    R.params.update(saved)


@pytest.mark.parametrize("case", ["p0", "p1", "p2"])
def test_particle_advance_matches_reference(params, case):
    params.update(solvertolerances=(1e-8, 1e-8), cyclotronresolution=20)
    init = GOLD["traj_%s_init" % case]
    p = R.Particle(init[0:3], init[3:6], 0, init[6], init[7], R.fields.EarthDipole())
    p.advance(2.0)
    ref = GOLD["traj_%s_rows" % case]
    assert p.trajectory.shape == ref.shape
    np.testing.assert_allclose(p.trajectory, ref, rtol=1e-8, atol=0)
    assert np.isclose(p.tcur, GOLD["traj_%s_tcur" % case][0], rtol=1e-13)


@pytest.mark.parametrize("case", ["g0", "g1"])
def test_guidingcenter_advance_matches_reference(params, case):
    params.update(solvertolerances=(1e-8, 1e-8), GCtimestep=1.0)
    init = GOLD["traj_%s_init" % case]
    g = R.GuidingCenter(init[0:3], init[3], pa=init[4], t0=0, mass=init[5], charge=init[6],
                        field=R.fields.DoubleDipole())
    g.advance(3.0)
    ref = GOLD["traj_%s_rows" % case]
    assert g.trajectory.shape == ref.shape
    np.testing.assert_allclose(g.trajectory[:, :4], ref[:, :4], rtol=1e-8, atol=0)
    # ppar oscillates through zero along a bounce: compare against its amplitude
    np.testing.assert_allclose(g.trajectory[:, 4], ref[:, 4], rtol=0, atol=1e-8 * np.max(np.abs(ref[:, 4])))


def test_adaptive_speiser_matches_reference(params, capsys):
    params.update(solvertolerances=(1e-12, 1e-12), epss=0.02, GCtimestep=1, cyclotronresolution=10)
    a = R.Adaptive([5, -5, 0.9], [-0.1, 0.1, 0], 0, 1, 1, R.fields.Parabolic())
    a.advance(300)
    modes = [0 if isinstance(s, R.Particle) else 1 for s in a.trajlist]
    assert modes == list(GOLD["adaptive_speiser_modes"])
    t0s = [s.trajectory[0, 0] for s in a.trajlist]
    np.testing.assert_allclose(t0s, GOLD["adaptive_speiser_t0s"], rtol=1e-10)
    assert [len(s.trajectory) for s in a.trajlist] == list(GOLD["adaptive_speiser_nrows"])
    fin = GOLD["adaptive_speiser_final"]
    np.testing.assert_allclose(a.trajlist[-1].trajectory[-1], fin, rtol=1e-7)
    out = capsys.readouterr().out
    assert "Switched to particle mode at time 168.0" in out


def test_adaptive_harris_matches_reference(params):
    params.update(solvertolerances=(1e-8, 1e-8), GCtimestep=0.5, cyclotronresolution=10)
    init = GOLD["adaptive_harris_init"]
    a = R.Adaptive(init[0:3], init[3:6], 0, init[6], init[7], R.fields.Harris())
    a.advance(60)
    modes = [0 if isinstance(s, R.Particle) else 1 for s in a.trajlist]
    assert modes == list(GOLD["adaptive_harris_modes"])
    t0s = [s.trajectory[0, 0] for s in a.trajlist]
    np.testing.assert_allclose(t0s, GOLD["adaptive_harris_t0s"], rtol=1e-9)


def test_batch_equals_individual(params):
    params.update(solvertolerances=(1e-8, 1e-8), cyclotronresolution=20)
    f = R.fields.EarthDipole()
    rng = np.random.default_rng(7)
    mk = lambda: [R.Particle([6 * R.Re, 0, 0], v, 0, R.m_pr, R.e, f) for v in vs]  # noqa: E731
    vs = [rng.standard_normal(3) * 3e7 for _ in range(5)]
    a, b = mk(), mk()
    R.advance_batch(a, 1.0)
    for p in b:
        p.advance(1.0)
    for p, q in zip(a, b):
        np.testing.assert_array_equal(p.trajectory, q.trajectory)


def test_particle_raises_adiabatic(params):
    params.update(solvertolerances=(1e-8, 1e-8), epss=0.05)
    p = R.Particle([5 * R.Re, 0, 0], [0, 1e6, 1e6], 0, R.m_pr, R.e, R.fields.EarthDipole())
    p.check_adiabaticity = True
    with pytest.raises(R.Adiabatic):
        p.advance(1.0)
    assert len(p.trajectory) == 2


def test_fields_without_device_implementation_raise(params):
    class MyField(R.fields.EarthDipole):
        def B(self, tpos):
            return np.array([0.0, 0.0, 1e-5])

    p = R.Particle([6 * R.Re, 0, 0], [0, 1e6, 0], 0, R.m_pr, R.e, MyField())
    with pytest.raises(NotImplementedError):
        p.advance(1.0)
    # GCtimestep = 0 selects the bounce-period cadence, which runs on the device
    params.update(GCtimestep=0)
    g = R.GuidingCenter([5 * R.Re, 0, 0], 1e7, pa=45, mass=R.m_el, charge=-R.e, field=R.fields.DoubleDipole())
    tb = g.bounceperiod()
    g.advance(0.3 * tb)
    assert np.allclose(np.diff(g.trajectory[:, 0]), tb / 10, rtol=1e-9)
