"""Particle, GuidingCenter and Adaptive with RAPT's constructors, advance(),
params and getters; advance() runs on the GPU.

Mirrors rapt/Particle.py, rapt/GuidingCenter.py and rapt/Adaptive.py. Host-side
helpers (init, setke, setpa, isadiabatic, getters) follow the reference's
formulas, with field quantities evaluated by the GPU library. ``advance`` and
``advance_batch`` go through ``Ensemble`` (the C ABI); a field without a device
implementation raises ``NotImplementedError``.

Reference behaviours kept as they are: Particle.getB returns None
(Particle.py:456-461), Particle.getv uses sqrt(1 - gamma^2) (:427-431),
GuidingCenter.getp's relativistic branch returns m c (gamma^2 - 1) (:507) and
GuidingCenter.getv calls a missing method (:510-515).
"""
import pickle

import numpy as np

from . import _native as N
from . import utils as ru
from .ensemble import Ensemble

c = 299792458
_EOMS = {"TaoChanBrizardEOM": 0, "BrizardChanEOM": 1, "NorthropTellerEOM": 2}


def _params():
    from . import params
    return params


def _config(eom=0, tableau=0):
    p = _params()
    rtol, atol = p["solvertolerances"]
    return dict(rtol=rtol, atol=atol, cyclotronresolution=p["cyclotronresolution"], gctimestep=p["GCtimestep"],
                epss=p["epss"], epst=p["epst"], enforce_equatorial=int(bool(p["enforce equatorial"])),
                gc_eom=eom, tableau=tableau, bounceresolution=p["bounceresolution"],
                fieldlineresolution=p["fieldlineresolution"], dense_output=int(bool(p.get("dense output", False))),
                rkf_tol=float(p.get("rkf tolerance", 1e-3)), rkf_hmin=float(p.get("rkf minimum step", 1e-12)))


class _Pickle:
    def save(self, filename):
        with open(filename, "wb") as f:
            pickle.dump(self, f)

    def load(self, filename):
        with open(filename, "rb") as f:
            p = pickle.load(f)
        for k in p.__dict__.keys():
            self.__dict__[k] = p.__dict__[k]


# ============================================================== Particle
class Particle(_Pickle):
    """Relativistic full-orbit tracer, rapt/Particle.py:18-493."""

    def __init__(self, pos=[], vel=[], t0=0, mass=None, charge=None, field=None):
        self.pos = np.array(pos)
        self.vel = np.array(vel)
        self.t0 = t0
        self.tcur = t0
        self.mass = mass
        self.charge = charge
        self.field = field
        self.trajectory = np.zeros((1, 7))
        self.check_adiabaticity = False
        if not (len(self.pos) == 0 or len(self.vel) == 0 or self.mass is None):
            gamma = 1 / np.sqrt(1 - np.dot(self.vel, self.vel) / c ** 2)
            mom = self.mass * gamma * self.vel
            self.trajectory = np.concatenate(([self.tcur], self.pos, mom)).reshape(1, 7)

    def init(self, p, gyrophase=0):
        """Particle.py:111-166."""
        if isinstance(p, Particle):
            mom = p.trajectory[-1, 4:]
            gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2) if self.mass is not None else \
                np.sqrt(p.mass ** 2 + np.dot(mom, mom) / c ** 2)
            self.__init__(pos=p.trajectory[-1, 1:4], vel=p.trajectory[-1, 4:] / gm, t0=p.trajectory[-1, 0],
                          mass=p.mass, charge=p.charge, field=p.field)
        elif isinstance(p, GuidingCenter):
            B = p.field.magB(p.trajectory[-1, :4])
            gammasq = 1 + 2 * p.mu * B / (p.mass * c * c) + (p.trajectory[-1, 4] / p.mass / c) ** 2
            if np.sqrt(gammasq) - 1 < 1e-6:
                v = np.sqrt(2 * p.mu * B / p.mass + (p.trajectory[-1, 4] / p.mass) ** 2)
            else:
                v = c * np.sqrt(1 - 1 / gammasq)
            vpar = p.trajectory[-1, 4] / p.mass / np.sqrt(gammasq)
            pos, vel = ru.GCtoFP(self.tcur, p.trajectory[-1, 1:4], vpar, v, p.field, p.mass, p.charge, gyrophase)
            self.__init__(pos=pos, vel=vel, t0=p.trajectory[-1, 0], mass=p.mass, charge=p.charge, field=p.field)
        else:
            raise ValueError("Particle or GuidingCenter objects required.")

    def setke(self, ke, unit="ev"):
        assert ke > 0
        s = ru.speedfromKE(ke, self.mass, unit)
        mom = self.trajectory[-1, 4:]
        gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2)
        v = mom / gm
        v = v * (s / np.sqrt(np.dot(v, v)))
        self.__init__(self.pos, v, self.t0, self.mass, self.charge, self.field)

    def setpa(self, pa):
        tpos = self.trajectory[-1, 0:4]
        mom = self.trajectory[-1, 4:]
        gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2)
        v = mom / gm
        s = np.sqrt(np.dot(v, v))
        b = self.field.unitb(tpos)
        spar = np.dot(v, b)
        if abs(spar - s) < 1e-12:
            p = ru.getperp(b)
        else:
            vperp = v - spar * b
            p = vperp / np.sqrt(np.dot(vperp, vperp))
        w = s * np.sin(pa * np.pi / 180) * p + s * np.cos(pa * np.pi / 180) * b
        self.__init__(self.pos, w, self.t0, self.mass, self.charge, self.field)

    def advance(self, delta):
        """Particle.advance (Particle.py:230-309), on the GPU."""
        from . import Adiabatic
        res = advance_batch([self], delta)
        _raise_if_left_grid(res)
        if self.check_adiabaticity and res["raised"][0]:
            raise Adiabatic

    def isadiabatic(self):
        """Particle.py:345-384."""
        p = _params()
        tpos = self.trajectory[-1, :4]
        if self.field.static:
            return self.cycrad() / self.field.lengthscale(tpos) < p["epss"]
        return self.cycrad() / self.field.lengthscale(tpos) < p["epss"] and \
            self.cycper() / self.field.timescale(tpos) < p["epst"]

    def gett(self): return self.trajectory[:, 0]
    def getx(self): return self.trajectory[:, 1]
    def gety(self): return self.trajectory[:, 2]
    def getz(self): return self.trajectory[:, 3]
    def getpx(self): return self.trajectory[:, 4]
    def getpy(self): return self.trajectory[:, 5]
    def getpz(self): return self.trajectory[:, 6]

    def getp(self):
        return np.sqrt(self.getpx() ** 2 + self.getpy() ** 2 + self.getpz() ** 2)

    def getgamma(self):
        psq = self.trajectory[:, 4] ** 2 + self.trajectory[:, 5] ** 2 + self.trajectory[:, 6] ** 2
        return np.sqrt(1 + psq / (self.mass * c) ** 2)

    def getvx(self): return self.getpx() / self.getgamma() / self.mass
    def getvy(self): return self.getpy() / self.getgamma() / self.mass
    def getvz(self): return self.getpz() / self.getgamma() / self.mass

    def getv(self):
        psq = self.trajectory[:, 4] ** 2 + self.trajectory[:, 5] ** 2 + self.trajectory[:, 6] ** 2
        gammasq = 1 + psq / (self.mass * c) ** 2
        with np.errstate(invalid="ignore"):
            return np.sqrt(1 - gammasq) * c

    def getr(self): return np.sqrt(self.getx() ** 2 + self.gety() ** 2 + self.getz() ** 2)
    def gettheta(self): return np.arctan2(self.gety(), self.getx())
    def getphi(self): return np.arccos(self.getz() / self.getr())

    def getke(self):
        g = self.getgamma()
        ke_nr = 0.5 * (self.trajectory[:, 4] ** 2 + self.trajectory[:, 5] ** 2 + self.trajectory[:, 6] ** 2) / self.mass
        return np.where(g - 1 < 1e-6, ke_nr, (g - 1) * self.mass * c * c)

    def getB(self):
        self.field.magB(self.trajectory[:, :4])  # evaluated, not returned -- as the reference

    def guidingcenter(self):
        out = []
        for row in self.trajectory:
            t, r, mom = row[0], row[1:4], row[4:]
            gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2)
            rgc, vp, spd = ru.guidingcenter(t, r, mom / gm, self.field, self.mass, self.charge)
            out.append(list(rgc) + [vp, spd])
        return np.array(out)

    def mu(self):
        out = []
        for row in self.trajectory:
            t, r, mom = row[0], row[1:4], row[4:]
            gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2)
            rgc, vp, spd = ru.guidingcenter(t, r, mom / gm, self.field, self.mass, self.charge)
            out.append(ru.magnetic_moment(t, rgc, vp, spd, self.field, self.mass))
        return np.array(out)

    def cycrad(self):
        t, r, mom = self.trajectory[-1, 0], self.trajectory[-1, 1:4], self.trajectory[-1, 4:]
        gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2)
        return ru.cyclotron_radius(t, r, mom / gm, self.field, self.mass, self.charge)

    def cycper(self):
        t, r, mom = self.trajectory[-1, 0], self.trajectory[-1, 1:4], self.trajectory[-1, 4:]
        gm = np.sqrt(self.mass ** 2 + np.dot(mom, mom) / c ** 2)
        return ru.cyclotron_period(t, r, mom / gm, self.field, self.mass, self.charge)


# ============================================================== GuidingCenter
class GuidingCenter(_Pickle):
    """Relativistic guiding-centre tracer, rapt/GuidingCenter.py:18-624."""

    def __init__(self, pos=[], v=0, pa=None, ppar=None, t0=0, mass=None, charge=None, field=None):
        self.pos = pos
        self.v = v
        self.t0 = t0
        self.tcur = t0
        self.mass = mass
        self.charge = charge
        self.field = field
        self.trajectory = np.zeros((1, 5))
        self.check_adiabaticity = False
        if not (len(pos) == 0 or v == 0):
            gamma = 1 / np.sqrt(1 - (v / c) ** 2)
            if pa is not None:
                vpar = 0 if pa == 90 else v * np.cos(pa * np.pi / 180)
                ppar = gamma * mass * vpar
            self.mu = ru.magnetic_moment(self.tcur, self.pos, ppar / (mass * gamma), self.v, self.field, self.mass)
            self.trajectory[0, 0] = t0
            self.trajectory[0, 1:4] = pos[:]
            self.trajectory[0, 4] = ppar

    def init(self, p):
        """GuidingCenter.py:135-188."""
        if isinstance(p, GuidingCenter):
            B = p.field.magB(p.trajectory[-1, :4])
            gamma = np.sqrt(1 + 2 * p.mu * B / (p.mass * c * c) + (p.trajectory[-1, 4] / p.mass / c) ** 2)
            if gamma - 1 < 1e-6:
                v = np.sqrt(2 * p.mu * B / p.mass + (p.trajectory[-1, 4] / p.mass) ** 2)
            else:
                v = c * np.sqrt(1 - 1 / gamma ** 2)
            self.__init__(pos=p.trajectory[-1, 1:4], v=v, ppar=p.trajectory[-1, 4], t0=p.trajectory[-1, 0],
                          mass=p.mass, charge=p.charge, field=p.field)
            self.check_adiabaticity = p.check_adiabaticity
        elif isinstance(p, Particle):
            mom = p.trajectory[-1, 4:]
            gm = np.sqrt(p.mass ** 2 + np.dot(mom, mom) / c ** 2)
            res = ru.guidingcenter(p.trajectory[-1, 0], p.trajectory[-1, 1:4], mom / gm, p.field, p.mass, p.charge)
            pos, vp, v = res
            gamma = 1 / np.sqrt(1 - (v / c) ** 2)
            self.__init__(pos=pos, v=v, ppar=p.mass * gamma * vp, t0=p.trajectory[-1, 0], mass=p.mass,
                          charge=p.charge, field=p.field)
            self.check_adiabaticity = p.check_adiabaticity
        else:
            raise ValueError("Particle or GuidingCenter objects required.")

    def _speed_parts(self):
        mc = self.mass * c
        t, x, y, z, ppar = self.trajectory[-1]
        B = self.field.magB(self.trajectory[-1, :4])
        return mc, t, x, y, z, ppar, B

    def setke(self, ke, unit="ev"):
        mc, t, x, y, z, ppar, B = self._speed_parts()
        gm1 = 2 * self.mu * B / (mc * c) + (ppar / mc) ** 2
        ptot = np.sqrt(2 * self.mass * self.mu * B + ppar ** 2) if np.sqrt(gm1 + 1) - 1 < 1e-6 else np.sqrt(gm1) * mc
        pa_old = np.arccos(ppar / ptot)
        self.__init__(pos=[x, y, z], v=ru.speedfromKE(ke, self.mass, unit), pa=pa_old, t0=t, mass=self.mass,
                      charge=self.charge, field=self.field)

    def setpa(self, pa):
        mc, t, x, y, z, ppar, B = self._speed_parts()
        gammasq = 1 + 2 * self.mu * B / (mc * c) + (ppar / mc) ** 2
        v = np.sqrt(2 * self.mass * self.mu * B + ppar ** 2) / self.mass if np.sqrt(gammasq) - 1 < 1e-6 else \
            c * np.sqrt(1 - 1 / gammasq)
        self.__init__(pos=[x, y, z], v=v, pa=pa, t0=t, mass=self.mass, charge=self.charge, field=self.field)

    def isadiabatic(self):
        p = _params()
        tpos = self.trajectory[-1, :4]
        if self.field.static:
            return self.cycrad() / self.field.lengthscale(tpos) < p["epss"]
        return self.cycrad() / self.field.lengthscale(tpos) < p["epss"] and \
            self.cycper() / self.field.timescale(tpos) < p["epst"]

    def advance(self, delta, eom="TaoChanBrizardEOM"):
        """GuidingCenter.advance (GuidingCenter.py:397-458), on the GPU."""
        from . import NonAdiabatic
        res = advance_batch([self], delta, eom=eom)
        _raise_if_left_grid(res)
        if self.check_adiabaticity and res["raised"][0]:
            raise NonAdiabatic

    def bounceperiod(self):
        """GuidingCenter.bounceperiod (GuidingCenter.py:593-606) at the current
        state: field-line trace and half-bounce path on the GPU."""
        from . import _native
        ctx = _native.default_context()
        self.field.bind(ctx)
        ctx.set_config(**_config())
        row = self.trajectory[-1]
        return float(ctx.gc_bounce_period(np.r_[row[0:5], self.mu, self.mass])[0])

    def geteye(self, step=1):
        raise NotImplementedError("second invariant (field-line integrals) has no device implementation")

    def gett(self): return self.trajectory[:, 0]
    def getx(self): return self.trajectory[:, 1]
    def gety(self): return self.trajectory[:, 2]
    def getz(self): return self.trajectory[:, 3]
    def getpp(self): return self.trajectory[:, 4]
    def getr(self): return np.sqrt(self.getx() ** 2 + self.gety() ** 2 + self.getz() ** 2)
    def gettheta(self): return np.arctan2(self.gety(), self.getx())
    def getphi(self): return np.arccos(self.getz() / self.getr())

    def getB(self):
        return np.asarray(self.field.magB(self.trajectory[:, :4]), float).reshape(-1)

    def getgamma(self):
        mc = self.mass * c
        return np.sqrt(1 + 2 * self.mu * self.getB() / (mc * c) + (self.trajectory[:, 4] / mc) ** 2)

    def getp(self):
        g, B, pp = self.getgamma(), self.getB(), self.trajectory[:, 4]
        return np.where(g - 1 < 1e-6, np.sqrt(2 * self.mass * self.mu * B + pp ** 2), self.mass * c * (g ** 2 - 1))

    def getv(self):
        mom = self.getp()
        gamma = self.gamma()  # noqa: F841 -- GuidingCenter has no gamma method (GuidingCenter.py:513)
        return mom / gamma

    def getBm(self):
        mc = self.mass * c
        g, B, pp = self.getgamma(), self.getB(), self.trajectory[:, 4]
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(g - 1 < 1e-6, B + 0.5 * pp ** 2 / (self.mu * self.mass),
                            B / (1 - (pp / mc) ** 2 / ((g - 1) * (g + 1))))

    def getke(self):
        g, B, pp = self.getgamma(), self.getB(), self.trajectory[:, 4]
        return np.where(g - 1 < 1e-6, self.mu * B + 0.5 * pp ** 2 / self.mass, (g - 1) * self.mass * c * c)

    def cycrad(self):
        t, r, pp = self.trajectory[-1, 0], self.trajectory[-1, 1:4], self.trajectory[-1, 4]
        Bmag = self.field.magB(self.trajectory[-1, :4])
        gamma = np.sqrt(1 + 2 * self.mu * Bmag / (self.mass * c * c) + (pp / self.mass / c) ** 2)
        if gamma - 1 < 1e-6:
            vp = pp / self.mass
            v = np.sqrt(2 * self.mu * Bmag / self.mass + vp ** 2)
        else:
            vp = pp / self.mass / gamma
            v = c * np.sqrt(1 - 1 / gamma ** 2)
        return ru.cyclotron_radius2(t, r, vp, v, self.field, self.mass, self.charge)

    def cycper(self):
        t, r, pp = self.trajectory[-1, 0], self.trajectory[-1, 1:4], self.trajectory[-1, 4]
        Bmag = self.field.magB(self.trajectory[-1, :4])
        gamma = np.sqrt(1 + 2 * self.mu * Bmag / (self.mass * c * c) + pp ** 2)
        if gamma - 1 < 1e-6:
            vp = pp / self.mass
            v = np.sqrt(2 * self.mu * Bmag / self.mass + vp ** 2)
        else:
            v = c * np.sqrt(1 - 1 / gamma ** 2)
        return ru.cyclotron_period2(t, r, v, self.field, self.mass, self.charge)


# ============================================================== Adaptive
class Adaptive(_Pickle):
    """Particle <-> guiding-centre switching tracer, rapt/Adaptive.py:18-274."""

    def __init__(self, pos=None, vel=None, t0=0, mass=None, charge=None, field=None):
        self.pos = np.array(pos)
        self.vel = np.array(vel)
        self.tcur = t0
        self.mass = mass
        self.charge = charge
        self.field = field
        self.p = Particle(pos, vel, t0, mass, charge, field)
        self.p.check_adiabaticity = True
        self._pick_mode()

    def _pick_mode(self):
        if self.p.isadiabatic():
            g = GuidingCenter()
            g.check_adiabaticity = True
            g.init(self.p)
            self.trajlist = [g]
        else:
            self.trajlist = [self.p]

    def setke(self, ke, unit="ev"):
        self.p.setke(ke, unit)
        self.p.check_adiabaticity = True
        self._pick_mode()

    def setpa(self, pa):
        self.p.setpa(pa)
        self.p.check_adiabaticity = True
        self._pick_mode()

    def advance(self, delta):
        """Adaptive.advance (Adaptive.py:187-222), on the GPU."""
        assert self.trajlist[-1].check_adiabaticity
        _raise_if_left_grid(advance_batch([self], delta, verbose=True))

    def _cat(self, name):
        return np.concatenate([np.asarray(getattr(p, name)(), float) for p in self.trajlist])

    def gett(self): return self._cat("gett")
    def getx(self): return self._cat("getx")
    def gety(self): return self._cat("gety")
    def getz(self): return self._cat("getz")
    def getr(self): return self._cat("getr")
    def getphi(self): return self._cat("getphi")
    def gettheta(self): return self._cat("gettheta")
    def getke(self): return self._cat("getke")


# ============================================================== batch entry
def _estimate_rows(kind, tracers, delta):
    p = _params()
    n = 4
    if kind in (N.KIND_GC, N.KIND_ADAPTIVE):
        if p["GCtimestep"] > 0:
            n = max(n, int(np.ceil(np.max(delta) / p["GCtimestep"])) + 4)
    if kind in (N.KIND_PARTICLE, N.KIND_ADAPTIVE):
        dts = []
        for t in tracers:
            cur = t.trajlist[-1] if isinstance(t, Adaptive) else t
            dts.append(cur.cycper() / p["cyclotronresolution"] if isinstance(cur, Particle) else np.inf)
        dmin = min(dts)
        if np.isfinite(dmin):
            n = max(n, int(np.ceil(np.max(delta) / dmin)) + 4)
    n = min(n, 4096) if kind == N.KIND_ADAPTIVE else n
    if p.get("dense output", False) and kind != N.KIND_PARTICLE:
        n = max(n, 18)  # a dense-output step may cover 17 output times
    return n


# ============================================================== BounceCenter
class BounceCenter(_Pickle):
    """Bounce-averaged tracer, rapt/BounceCenter.py:15-316, advanced on the GPU.

    The drift gamma m v^2 / (q S_b |B|^2) (grad I x B) takes five field-line
    traces per right-hand side (the half-bounce path and four second-invariant
    integrals); the GPU runs one tracer per thread. Static fields only, as in the
    reference. Kept from the reference: the constructor hands the pitch angle in
    degrees to np.cos (BounceCenter.py:104), and advance() stamps each row with
    the time its interval began. The reference's second-invariant integral raises
    NameError below 70 degrees equatorial pitch angle (flutils.py:130); here that
    range is served by the same spline method. isequatorial=True fails in the
    reference (BounceCenter.py:238-239) and raises NotImplementedError here.
    """

    def __init__(self, pos=[], v=None, t0=0, pa=None, mass=None, charge=None, field=None):
        self.pos = pos
        self.v = v
        self.t0 = t0
        self.tcur = t0
        self.mass = mass
        self.charge = charge
        self.field = field
        self.isequatorial = False
        if not field.static:
            raise RuntimeError("BounceCenter does not work with nonstatic fields or electric fields.")
        self.pa = pa
        if not (len(pos) == 0 or v is None or pa is None):
            self.trajectory = np.reshape(np.concatenate(([t0], pos)), (1, 4))
            self.mu = ru.magnetic_moment(t0, pos, self.v * np.cos(self.pa), self.v, field, mass)
            assert self.mu > 0

    def _Bm(self):
        gamma = 1.0 / np.sqrt(1 - (self.v / c) ** 2)
        return self.mass * gamma ** 2 * self.v ** 2 / (2 * self.mu)

    def _v_grad(self, tpos):
        """BounceCenter.py:120-139."""
        gamma = 1.0 / np.sqrt(1 - (self.v / c) ** 2)
        Bvec = self.field.B(tpos)
        gB = self.field.gradB(tpos)
        return self.mu * np.cross(Bvec, gB) / (self.charge * gamma * np.dot(Bvec, Bvec))

    def _v_inert(self, tpos):
        """BounceCenter.py:141-172."""
        vg = self._v_grad(tpos)
        vgmag = np.sqrt(np.dot(vg, vg))
        vgdir = np.zeros(4)
        vgdir[0] = tpos[0]
        vgdir[1:] = vg / vgmag
        d = self.field.gradientstepsize
        v1 = self._v_grad(tpos - d * vgdir)
        v2 = self._v_grad(tpos + d * vgdir)
        Bvec = self.field.B(tpos)
        return self.mass * vgmag / (self.charge * np.dot(Bvec, Bvec) * 2 * d) * np.cross(Bvec, v2 - v1)

    def drift(self, tpos):
        """The bounce-averaged drift velocity (the right-hand side of advance)."""
        ctx = N.default_context()
        self.field.bind(ctx)
        ctx.set_config(**_config())
        return ctx.bc_eval("drift", tpos, self._Bm(), _params()["eyegradientstep"],
                           [self.v, self.mu, self.mass, self.charge])[0]

    def advance(self, delta):
        """BounceCenter.advance (BounceCenter.py:214-252), on the GPU."""
        advance_batch([self], delta)

    def gett(self):
        return self.trajectory[:, 0]

    def getx(self):
        return self.trajectory[:, 1]

    def gety(self):
        return self.trajectory[:, 2]

    def getz(self):
        return self.trajectory[:, 3]

    def getr(self):
        return np.sqrt(self.getx() ** 2 + self.gety() ** 2 + self.getz() ** 2)

    def gettheta(self):
        return np.arctan2(self.gety(), self.getx())

    def getphi(self):
        return np.arccos(self.getz() / self.getr())

    def getB(self):
        return np.asarray(self.field.magB(self.trajectory[:, :4]), float)


def _advance_bc(tracers, delta):
    if any(t.isequatorial for t in tracers):
        raise NotImplementedError("isequatorial bounce centres fail in the reference (BounceCenter.py:238-239)")
    p = _params()
    field = tracers[0].field
    ctx = N.default_context()
    field.bind(ctx)
    ctx.set_config(**_config())
    n = len(tracers)
    delta = np.broadcast_to(np.asarray(delta, float), (n,))
    if np.any(delta != delta[0]):
        raise ValueError("BounceCenter batches share one delta")
    st0 = np.array([[*t.trajectory[-1, :4], t.tcur] for t in tracers])
    cst = np.array([[t.v, t.mu, t.mass, t.charge] for t in tracers])
    max_rows = 64
    for _ in range(2):
        st, rows, nr, status, cnt = ctx.bc_advance(st0.copy(), cst, delta[0], p["BCtimestep"],
                                                   p["eyegradientstep"], max_rows)
        if nr.max() <= max_rows:
            break
        max_rows = int(nr.max())  # rerun from the same start with room for every row
    for i, t in enumerate(tracers):
        if nr[i]:
            t.trajectory = np.vstack((t.trajectory, rows[i, :nr[i]]))
        t.tcur = st[i, 4]
    return {"raised": np.zeros(n, bool), "stats": {"counters": cnt}, "status": status}


def _raise_if_left_grid(res):
    # a Grid field evaluated outside its grid: the reference's interpolator raises
    # ValueError from inside the step (fields.py:733-737); the RKF45 tableau below
    # its minimum step: rkf.py raises RuntimeError (rkf.py:136-139). The rows
    # before the failing interval stay.
    if res["status"] is not None and res["status"][0] == N.ST["OUT_OF_GRID"]:
        raise ValueError("One of the requested xi is out of bounds: the tracer left the Grid field's grid")
    if res["status"] is not None and res["status"][0] == N.ST["RKF_HMIN"]:
        raise RuntimeError("Error: Could not converge to the required tolerance with minimum stepsize (RKF45)")


def advance_batch(tracers, delta, eom="TaoChanBrizardEOM", tableau=0, verbose=False):
    """Advance a list of tracers of one class sharing one field, in place, as if
    ``advance(delta)`` had been called on each. ``delta``: scalar or per tracer.
    Returns {"raised": bool array (Adiabatic / NonAdiabatic raised), "stats": ...}."""
    if len(tracers) == 0:
        return {"raised": np.zeros(0, bool), "stats": None, "status": None}
    cls = type(tracers[0])
    field = tracers[0].field
    if any(type(t) is not cls or t.field is not field for t in tracers):
        raise ValueError("advance_batch needs tracers of one class sharing one field object")
    if cls is BounceCenter:
        return _advance_bc(tracers, delta)
    kind = {Particle: N.KIND_PARTICLE, GuidingCenter: N.KIND_GC, Adaptive: N.KIND_ADAPTIVE}[cls]
    n = len(tracers)
    delta = np.broadcast_to(np.asarray(delta, float), (n,)).copy()
    max_rows = _estimate_rows(kind, tracers, delta)
    ens = Ensemble(field, n, max_rows=max_rows, max_switch=64 if kind == N.KIND_ADAPTIVE else 0)
    ens.configure(**_config(_EOMS[eom], tableau))
    h = ens.h
    cur = [t.trajlist[-1] if kind == N.KIND_ADAPTIVE else t for t in tracers]
    for i, tr in enumerate(cur):
        row = tr.trajectory[-1]
        h["t_row"][i] = row[0]
        h["t_int"][i] = row[0]
        h["tcur"][i] = tr.tcur
        h["mass"][i] = tr.mass
        h["charge"][i] = tr.charge
        h["flags"][i] = N.FLAG_CHECK if tr.check_adiabaticity else 0
        if isinstance(tr, Particle):
            h["mode"][i] = N.MODE_PARTICLE
            h["s"][:, i] = row[1:7]
        else:
            h["mode"][i] = N.MODE_GC
            h["s"][:4, i] = row[1:5]
            h["s"][4:, i] = 0.0
            h["mu"][i] = tr.mu
            h["v"][i] = tr.v
    for k in ("status", "naccept", "nreject", "nfcn", "nswitch"):
        h[k][:] = 0
    ens.upload()
    chunks = [[] for _ in range(n)]
    stats = ens.advance(kind, delta)
    for _ in range(100000):
        hs = ens.download()
        rows, rmode, nr, swt, swm = ens.rows(reset=True)
        for i in range(n):
            if nr[i]:
                chunks[i].append((rows[i, :nr[i]].copy(), rmode[i, :nr[i]].copy()))
        if not np.any(hs["status"] == N.ST["ROWS_FULL"]):
            break
        stats = ens.advance_resume(kind)
    raised = (hs["flags"] & N.FLAG_RAISED) != 0
    for i, t in enumerate(tracers):
        rows = np.concatenate([r for r, _ in chunks[i]]) if chunks[i] else np.zeros((0, 7))
        modes = np.concatenate([m for _, m in chunks[i]]) if chunks[i] else np.zeros(0, np.int8)
        if kind == N.KIND_ADAPTIVE:
            _materialise_adaptive(t, rows, modes, hs, i, verbose)
        else:
            tr = t
            w = 7 if kind == N.KIND_PARTICLE else 5
            if len(rows):
                tr.trajectory = np.vstack((tr.trajectory, rows[:, :w]))
            tr.tcur = hs["tcur"][i]
    return {"raised": raised, "stats": stats, "status": hs["status"].copy()}


def _materialise_adaptive(a, rows, modes, hs, i, verbose):
    cur = a.trajlist[-1]
    mode = N.MODE_PARTICLE if isinstance(cur, Particle) else N.MODE_GC
    buf = []

    def flush():
        if buf:
            w = 7 if isinstance(cur, Particle) else 5
            cur.trajectory = np.vstack((cur.trajectory, np.array(buf)[:, :w]))
            buf.clear()

    for row, m in zip(rows, modes):
        if m == mode:
            buf.append(row)
            continue
        flush()
        if m == N.MODE_GC:
            g = GuidingCenter()
            g.mass, g.charge, g.field = a.mass, a.charge, a.field
            g.mu, g.v = row[5], row[6]
            g.t0 = g.tcur = row[0]
            g.pos = row[1:4].copy()
            g.trajectory = row[None, :5].copy()
            g.check_adiabaticity = True
            cur = g
            if verbose:
                print("Switched to guiding center mode at time", g.tcur, flush=True)
        else:
            p = Particle()
            p.mass, p.charge, p.field = a.mass, a.charge, a.field
            p.t0 = p.tcur = row[0]
            p.pos = row[1:4].copy()
            p.trajectory = row[None, :7].copy()
            p.check_adiabaticity = True
            cur = p
            if verbose:
                print("Switched to particle mode at time", p.tcur, flush=True)
        a.trajlist.append(cur)
        mode = m
    flush()
    cur.tcur = hs["tcur"][i]
    if isinstance(cur, GuidingCenter):
        cur.mu, cur.v = hs["mu"][i], hs["v"][i]
    a.tcur = cur.tcur
