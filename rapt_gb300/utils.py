"""Physics utilities of rapt/utils.py used by the tracer classes (host side).

Field quantities are evaluated by the GPU library through the field objects.
Formulas and evaluation order follow rapt/utils.py (line numbers cited).
"""
import numpy as np

c = 299792458
e = 1.602176565e-19
Re = 6378137  # rapt/__init__.py:11-12
B0 = 3.07e-5


def gamma(mass=0, **kwargs):
    """rapt/utils.py:15-27."""
    if "velocity" in kwargs:
        return 1 / np.sqrt(1 - np.dot(kwargs["velocity"], kwargs["velocity"]) / c ** 2)
    elif "momentum" in kwargs:
        if mass == 0:
            raise ValueError("Particle mass not given.")
        return np.sqrt(1 + np.dot(kwargs["momentum"], kwargs["momentum"]) / (mass * c) ** 2)
    raise ValueError("Either velocity of momentum vectors should be given.")


def cyclotron_period(t, pos, vel, field, mass, charge):
    """rapt/utils.py:29-66: 2 pi gamma m / (q B) from the velocity vector."""
    vel = np.array(vel)
    g = 1.0 / np.sqrt(1 - np.dot(vel, vel) / c ** 2)
    B = field.magB(np.concatenate([[t], pos]))
    return 2 * np.pi * g * mass / B / abs(charge)


def cyclotron_period2(t, pos, speed, field, mass, charge):
    """rapt/utils.py:68-104: from the speed."""
    g = 1.0 / np.sqrt(1 - (speed / c) ** 2)
    B = field.magB(np.concatenate([[t], pos]))
    return 2 * np.pi * g * mass / B / abs(charge)


def cyclotron_radius(t, pos, vel, field, mass, charge):
    """rapt/utils.py:106-145."""
    vsq = np.dot(vel, vel)
    g = 1.0 / np.sqrt(1 - vsq / c ** 2)
    B = field.B(np.concatenate([[t], pos]))
    Bmag = np.sqrt(np.dot(B, B))
    vpar = np.dot(vel, B) / Bmag
    vperp = np.sqrt(vsq - vpar ** 2)
    return g * mass * vperp / (abs(charge) * Bmag)


def cyclotron_radius2(t, pos, vpar, v, field, mass, charge):
    """rapt/utils.py:147-187."""
    g = 1.0 / np.sqrt(1 - (v / c) ** 2)
    B = field.B(np.concatenate([[t], pos]))
    Bmag = np.sqrt(np.dot(B, B))
    vperp = np.sqrt((v - vpar) * (v + vpar))
    return g * mass * vperp / (abs(charge) * Bmag)


def magnetic_moment(t, pos, vpar, v, field, mass):
    """rapt/utils.py:189-216: gamma^2 m v_perp^2 / (2 B)."""
    g = 1.0 / np.sqrt(1 - (v / c) ** 2)
    Bmag = field.magB(np.concatenate([[t], pos]))
    return g ** 2 * mass * (v - vpar) * (v + vpar) / (2 * Bmag)


def speedfromKE(KE, mass, unit="ev"):
    """rapt/utils.py:218-249."""
    mc2 = mass * c ** 2
    if unit.lower() == "ev":
        KE = KE * e
    if KE / mc2 < 1e-6:
        return np.sqrt(2 * KE / mass)
    return c * np.sqrt(1 - (mc2 / (mc2 + KE)) ** 2)


def guidingcenter(t, r, v, field, mass, charge, tol=1e-3, maxiter=20, debug=False):
    """rapt/utils.py:251-326: fixed point R = r - rho(R). Returns None (after a
    message) when it does not converge, as the reference does."""
    def gyrovector(rr):
        vsq = np.dot(v, v)
        g = 1 / np.sqrt(1 - vsq / c ** 2)
        B = field.B(np.concatenate([[t], rr]))
        Bsq = np.dot(B, B)
        return g * mass / (charge * Bsq) * np.cross(B, v)

    def norm(a):
        return np.sqrt(np.dot(a, a))

    GC_old = np.array(r) - gyrovector(r)
    GC_list = [GC_old]
    it = 1
    while it <= maxiter:
        GC = r - gyrovector(GC_old)
        GC_list.append(GC)
        if norm(GC - GC_old) / norm(GC) < tol:
            if debug:
                return GC_list
            B = field.B(np.concatenate([[t], GC]))
            return GC, np.dot(v, B) / norm(B), norm(v)
        GC_old = GC
        it += 1
    print("Could not reach the specified tolerance after ", it, " iterations.")


def getperp(v):
    """rapt/utils.py:328-374."""
    assert len(v) == 3
    if v[0] == 0.0 and v[1] == 0.0 and v[2] == 0.0:
        raise ValueError("Zero vector")
    if v[0] == 0:
        return np.array([1, 0, 0])
    if v[1] == 0:
        return np.array([0, 1, 0])
    if v[2] == 0:
        return np.array([0, 0, 1])
    cc = -1.0 * (v[0] + v[1]) / v[2]
    return np.array([1, 1, cc]) / np.sqrt(2 + cc ** 2)


def GCtoFP(t, R, vp, speed, field, mass, charge, gyrophase=0):
    """rapt/utils.py:376-433: particle position and velocity for a guiding centre."""
    B = field.B(np.concatenate([[t], R]))
    Bsq = np.dot(B, B)
    b = B / np.sqrt(Bsq)
    pa = np.arccos(vp / speed)
    rc = cyclotron_radius2(t, R, vp, speed, field, mass, charge)
    u = getperp(B)
    u = u / np.sqrt(np.dot(u, u))
    w = np.cross(b, u)
    s = np.sign(charge)
    pos = R + rc * (np.cos(gyrophase) * u + np.sin(gyrophase) * w)
    vel = speed * (np.cos(pa) * b + s * np.sin(pa) * np.sin(gyrophase) * u - s * np.sin(pa) * np.cos(gyrophase) * w)
    return pos, vel


def dipoleI(R0, Bm):
    """The second invariant I = integral of sqrt(1 - B/Bm) ds between the mirror
    points of the dipole line through the equator at R0 (rapt/utils.py:531-557):
    on r = R0 cos^2(lat), B = B0 (Re/R0)^3 sqrt(1 + 3 sin^2) / cos^6 and
    ds = R0 cos sqrt(1 + 3 sin^2) d(lat), integrated over latitude (host
    quadrature: a closed-form helper, not the stepping path)."""
    from scipy.integrate import quad
    from scipy.optimize import brentq
    Beq = B0 * (Re / R0) ** 3

    def Bratio(lat):
        s2 = np.sin(lat) ** 2
        return Beq * np.sqrt(1 + 3 * s2) / np.cos(lat) ** 6 / Bm

    if Beq >= Bm:
        return 0.0
    lat_m = brentq(lambda lat: Bratio(lat) - 1.0, 0.0, np.pi / 2 - 1e-9, xtol=1e-15, rtol=4 * np.finfo(float).eps)

    def integrand(lat):
        s2 = np.sin(lat) ** 2
        return np.sqrt(max(1.0 - Bratio(lat), 0.0)) * R0 * np.cos(lat) * np.sqrt(1 + 3 * s2)

    return 2 * quad(integrand, 0.0, lat_m, epsabs=0.0, epsrel=1e-12, limit=200)[0]


def dipole_gradI(x, y, Bm, h):
    """rapt/utils.py:559-581: central difference of dipoleI in the radial direction."""
    r0 = np.sqrt(x ** 2 + y ** 2)
    mag = (dipoleI(r0 + h, Bm) - dipoleI(r0 - h, Bm)) / (2 * h)
    return mag * np.array((x, y, 0)) / r0


def Bm(tpos, pa, field):
    """The mirror field |B| / sin^2(pa) at tpos for a pitch angle pa in degrees,
    first invariant conserved (rapt/utils.py:516-522); |B| from the device."""
    return field.magB(tpos) / np.sin(pa * np.pi / 180) ** 2


def dipoleBm(L, eqpa):
    """The mirror field B0 / L^3 / sin^2(eqpa) of the Earth dipole for the
    equatorial distance L (Re) and equatorial pitch angle eqpa in degrees
    (rapt/utils.py:524-529)."""
    return B0 / L ** 3 / np.sin(eqpa * np.pi / 180) ** 2


def dipole_bounce_period(L, v, eqpa):
    """Bounce period (s) in the Earth dipole, Walt's approximation
    0.117 L / beta (1 - 0.4635 sin(eqpa)^0.75) (M. Walt, Introduction to
    Geomagnetically Trapped Radiation, p. 49; rapt/utils.py:489-513)."""
    beta = v / c
    return 0.117 * L / beta * (1 - 0.4635 * np.sin(eqpa * np.pi / 180) ** 0.75)


def _walt_drift(k, L, v, eqpa):
    beta = v / c
    g = 1 / np.sqrt(1 - beta ** 2)
    return k / (L * g * beta ** 2) * (1 - np.sin(eqpa * np.pi / 180) ** 0.62 / 3)


def dipole_drift_period_p(L, v, eqpa):
    """Proton drift period (s) in the Earth dipole, Walt's approximation
    8.481 / (L gamma beta^2) (1 - sin(eqpa)^0.62 / 3) (Walt, p. 49;
    rapt/utils.py:435-460)."""
    return _walt_drift(8.481, L, v, eqpa)


def dipole_drift_period_e(L, v, eqpa):
    """Electron drift period (s) in the Earth dipole, Walt's approximation with
    1.557e4 in place of the proton's 8.481 (rapt/utils.py:462-487)."""
    return _walt_drift(1.557e4, L, v, eqpa)


def drift_error(b):
    """Relative deviation of each trajectory point of a BounceCenter from the
    distance of its first point, (|r| - |r0|) / |r0| (a dipole's drift path is
    a circle; rapt/utils.py:583-607)."""
    r = np.sqrt(np.sum(b.trajectory[:, 1:] ** 2, axis=1))
    return (r - r[0]) / r[0]

