"""Faraday's law for the time-dependent compressed dipole (no reference
counterpart): its induced electric field E = -(dB0/dt) Re^3 (y, -x, 0) / r^3 is
minus the time derivative of the vector potential A = B0(t) Re^3 (y, -x, 0) / r^3,
whose curl is the VarEarthDipole-form field (rapt/fields.py:455-470 with the
period of the compression). So curl E = -dB/dt everywhere: checked here with
central differences at random points and times, for the oracle's field and
(marked gpu) for the device's."""
import numpy as np
import pytest

Re = 6378137.0


def _points(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.uniform(2.5, 9.0, n) * Re
    d = rng.standard_normal((n, 3))
    p = r[:, None] * d / np.linalg.norm(d, axis=1, keepdims=True)
    return np.column_stack([rng.uniform(0, 120, n), p])


def _check(Efun, Bfun, tp):
    """max over points of |curl E + dB/dt| / |dB/dt| (central differences)."""
    worst = 0.0
    for t, x, y, z in tp:
        r = np.sqrt(x * x + y * y + z * z)
        d = 1e-4 * r
        J = np.zeros((3, 3))  # J[i, j] = dE_i / dx_j
        for j in range(3):
            e = np.zeros(4)
            e[1 + j] = d
            J[:, j] = (Efun(np.array([t, x, y, z]) + e) - Efun(np.array([t, x, y, z]) - e)) / (2 * d)
        curl = np.array([J[2, 1] - J[1, 2], J[0, 2] - J[2, 0], J[1, 0] - J[0, 1]])
        dt = 1e-3
        dBdt = (Bfun(np.array([t + dt, x, y, z])) - Bfun(np.array([t - dt, x, y, z]))) / (2 * dt)
        worst = max(worst, np.linalg.norm(curl + dBdt) / np.linalg.norm(dBdt))
    return worst


def test_compressed_dipole_faraday_oracle(oracle):
    f = oracle.field("CompressedDipole")
    err = _check(lambda p: oracle.field_eval(f, "E", p), lambda p: oracle.field_eval(f, "B", p), _points(64, 11))
    # central-difference truncation ~ (1e-4)^2 in space, (w dt)^2 ~ 1e-8 in time
    assert err < 1e-6, err


def test_compressed_dipole_e_is_azimuthal_and_zero_at_extremes(oracle):
    """E is azimuthal (E . r = 0, E_z = 0) and vanishes where dB0/dt does
    (t = period / 4)."""
    f = oracle.field("CompressedDipole")
    for t, x, y, z in _points(16, 12):
        E = oracle.field_eval(f, "E", np.array([t, x, y, z]))
        assert abs(E[2]) == 0 and abs(E @ [x, y, z]) <= 1e-12 * np.linalg.norm(E) * Re * 10
        E0 = oracle.field_eval(f, "E", np.array([15.0, x, y, z]))
        assert np.all(np.abs(E0) <= 1e-15 * np.linalg.norm(E) + 1e-30)


@pytest.mark.gpu
def test_compressed_dipole_faraday_device():
    from rapt_gb300 import fields as F
    fld = F.CompressedDipole()
    tp = _points(64, 13)
    err = _check(lambda p: np.asarray(fld.E(p[None, :]), float).reshape(3),
                 lambda p: np.asarray(fld.B(p[None, :]), float).reshape(3), tp)
    assert err < 1e-6, err
