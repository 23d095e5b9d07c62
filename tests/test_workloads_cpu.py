"""The seeded synthetic workloads that stand in for the benchmark
configurations: shapes, value ranges and distributions as the configurations
state them, and reproducibility from the seed (rapt_gb300.workloads)."""
import numpy as np

from rapt_gb300 import workloads as W

N = 4096


def _L(pos):
    return np.linalg.norm(pos, axis=1) / W.Re


def _ke_from_speed(v, m):
    """Kinetic energy in eV (the workloads' unit)."""
    return (1 / np.sqrt(1 - (v / W.c) ** 2) - 1) * m * W.c ** 2 / W.e


def _pitch_deg(pos, vel):
    b = W._dipole_bhat(pos)
    return np.degrees(np.arccos(np.clip(np.sum(b * vel, 1) / np.linalg.norm(vel, axis=1), -1, 1)))


def test_particle_config_earth_dipole_protons():
    w = W.config1()
    assert w["pos"].shape == (256, 3) and np.allclose(w["pos"], [6 * W.Re, 0, 0])
    assert np.all(w["mass"] == W.m_pr) and np.all(w["charge"] == W.e) and w["delta"] == 10.0
    ke = _ke_from_speed(np.linalg.norm(w["vel"], axis=1), W.m_pr)
    np.testing.assert_allclose(ke, w["ke"], rtol=1e-9)
    assert ke.min() >= 0.1 * W.MeV * (1 - 1e-9) and ke.max() <= 10 * W.MeV * (1 + 1e-9)
    pa = _pitch_deg(w["pos"], w["vel"])
    assert pa.min() >= 10 - 1e-6 and pa.max() <= 80 + 1e-6


def test_guiding_centre_config_double_dipole_electrons():
    w = W.config2(N)
    L = _L(w["pos"])
    assert np.all(w["pos"][:, 2] == 0) and L.min() >= 4 and L.max() <= 7
    assert w["pa"].min() >= 15 and w["pa"].max() <= 85 and w["delta"] == 100.0
    assert w["params"]["gctimestep"] == 1.0 and w["field"][0] == "DoubleDipole"
    lk = np.log10(_ke_from_speed(w["v"], W.m_el) / W.MeV)
    assert lk.min() >= -1 - 1e-9 and lk.max() <= 1 + 1e-9
    assert abs(np.mean(lk)) < 0.05  # log-uniform over two decades, centred on 1 MeV
    # the 1M benchmark ensemble is the same distributions at 2^20
    b = W.gc_bench(N)
    assert np.array_equal(b["pos"], w["pos"]) and np.array_equal(b["v"], w["v"])


def test_adaptive_harris_config_durations_and_directions():
    w = W.config3(N)
    assert np.all(w["pos"][:, :2] == 0) and np.abs(w["pos"][:, 2]).max() <= 3 * W.Re
    assert w["delta"].min() >= 1 and w["delta"].max() <= 300
    d = w["vel"] / np.linalg.norm(w["vel"], axis=1, keepdims=True)
    assert np.all(np.abs(d.mean(axis=0)) < 0.05)  # isotropic
    ke = _ke_from_speed(np.linalg.norm(w["vel"], axis=1), W.m_pr)
    assert ke.min() >= 1e3 * (1 - 1e-9) and ke.max() <= 50e3 * (1 + 1e-9)


def test_precision_and_learned_configs_mixed_species():
    for fn, field in ((W.config4, "EarthDipole"), (W.config5, "CompressedDipole")):
        w = fn(N)
        assert w["field"][0] == field
        assert np.sum(w["mass"] == W.m_el) == N // 2 and np.sum(w["charge"] < 0) == N // 2
        L = _L(w["pos"])
        assert L.min() >= 3 and L.max() <= 8
        ke = _ke_from_speed(np.linalg.norm(w["vel"], axis=1), w["mass"])
        np.testing.assert_allclose(ke, w["ke"], rtol=1e-9)
        cosa = np.cos(np.radians(_pitch_deg(w["pos"], w["vel"])))
        assert abs(cosa.mean()) < 0.05 and 0.28 < np.mean(cosa ** 2) < 0.39  # isotropic: E[cos^2] = 1/3
    w = W.config4(N)
    assert np.all(w["delta"] > 0)  # 50 gyro-periods at the start
    assert W.config5(N)["delta"] == 200.0


def test_workloads_are_reproducible_from_the_seed():
    for name, fn in W.CONFIGS.items():
        a, b = fn(512, seed=3), fn(512, seed=3)
        for k in ("pos", "mass", "charge"):
            assert np.array_equal(a[k], b[k]), (name, k)
        c = fn(512, seed=4)
        assert not np.array_equal(a["pos"], c["pos"]) or name == "config1", name
