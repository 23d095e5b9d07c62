"""Array-native batched entry: a device-resident ensemble of tracers.

``Ensemble`` holds N tracers as structure-of-arrays in GPU memory and advances
all of them with one call, with the semantics of calling ``advance(delta)`` on
each RAPT tracer (rapt/Particle.py:230-309, rapt/GuidingCenter.py:397-458,
rapt/Adaptive.py:187-222). The object classes in this package
(``Particle``, ``GuidingCenter``, ``Adaptive``) and ``advance_batch`` are built
on it.
"""
import numpy as np

from . import _native as N

c = 299792458.0


class Ensemble:
    """N tracers on the GPU.

    Parameters
    ----------
    field : field object of ``rapt_gb300.fields`` with a device implementation.
    n : number of tracers.
    max_rows : output rows kept per tracer between downloads (>= 2).
    max_switch : Adaptive switch-log entries kept per tracer.
    """

    ARRAYS = {"mode": np.int8, "status": np.int32, "flags": np.int32, "t_int": np.float64,
              "t_row": np.float64, "tcur": np.float64, "mu": np.float64, "v": np.float64,
              "mass": np.float64, "charge": np.float64, "naccept": np.int64, "nreject": np.int64,
              "nfcn": np.int64, "nswitch": np.int32}

    def __init__(self, field, n, max_rows=2, max_switch=0, ctx=None, pinned=False):
        self.ctx = ctx or N.default_context()
        self.field = field
        self.n = int(n)
        self.max_rows = int(max_rows)
        self.max_switch = int(max_switch)
        field.bind(self.ctx)
        self.ctx.check(self.ctx.L.rapt_ensemble_alloc(self.ctx.h, self.n, self.max_rows, self.max_switch),
                       "rapt_ensemble_alloc")
        self.h = {k: np.zeros(self.n, dt) for k, dt in self.ARRAYS.items()}
        self.h["s"] = np.zeros((6, self.n))
        self._pinned = []
        if pinned:
            self.pin()
        self.config = {}
        self.last_stats = None

    # ----------------------------------------------------------- host buffers
    def pin(self):
        """Page-lock the host SoA buffers (used by the end-to-end path)."""
        for a in list(self.h.values()):
            self.ctx.check(self.ctx.L.rapt_host_register(a.ctypes.data, a.nbytes), "rapt_host_register")
            self._pinned.append(a)

    def unpin(self):
        for a in self._pinned:
            self.ctx.L.rapt_host_unregister(a.ctypes.data)
        self._pinned = []

    def __del__(self):
        try:
            self.unpin()
        except Exception:
            pass

    def _hs(self, download=False):
        h = self.h
        st = N.RaptHostState()
        st.n = self.n
        for k in self.ARRAYS:
            setattr(st, k, h[k].ctypes.data)
        for i in range(6):
            st.s[i] = h["s"][i].ctypes.data
        return st

    def upload(self):
        st = self._hs()
        self.ctx.check(self.ctx.L.rapt_ensemble_upload(self.ctx.h, N.ctypes_byref(st)), "rapt_ensemble_upload")

    def download(self):
        st = self._hs()
        self.ctx.check(self.ctx.L.rapt_ensemble_download(self.ctx.h, N.ctypes_byref(st)), "rapt_ensemble_download")
        return self.h

    def rows(self, reset=True):
        """(rows[n,max_rows,7], row_mode[n,max_rows], nrows[n], sw_time[n,max_sw], sw_mode[n,max_sw])."""
        rows = np.zeros((self.n, self.max_rows, 7))
        rm = np.zeros((self.n, self.max_rows), np.int8)
        nr = np.zeros(self.n, np.int32)
        swt = np.zeros((self.n, max(self.max_switch, 1)))
        swm = np.zeros((self.n, max(self.max_switch, 1)), np.int8)
        self.ctx.check(self.ctx.L.rapt_rows_download(self.ctx.h, rows.ctypes.data, rm.ctypes.data, nr.ctypes.data,
                                                     swt.ctypes.data if self.max_switch else None,
                                                     swm.ctypes.data if self.max_switch else None, int(reset)),
                       "rapt_rows_download")
        return rows, rm, nr, swt[:, :self.max_switch], swm[:, :self.max_switch]

    # ----------------------------------------------------------- construction
    def set_particles(self, pos, vel, t0=0.0, mass=None, charge=None, check_adiabaticity=False):
        """Particle.__init__ for all tracers (rapt/Particle.py:95-109): p = gamma m v."""
        pos = np.asarray(pos, float).reshape(self.n, 3)
        vel = np.asarray(vel, float).reshape(self.n, 3)
        mass = np.broadcast_to(np.asarray(mass, float), (self.n,))
        h = self.h
        vsq = np.einsum("ij,ij->i", vel, vel)
        gamma = 1.0 / np.sqrt(1.0 - vsq / c ** 2)
        h["mode"][:] = N.MODE_PARTICLE
        h["s"][0:3] = pos.T
        h["s"][3:6] = (mass * gamma * vel.T)
        h["mass"][:] = mass
        h["charge"][:] = np.broadcast_to(np.asarray(charge, float), (self.n,))
        self._common(t0, check_adiabaticity)

    def set_guiding_centers(self, pos, v, pa=None, ppar=None, t0=0.0, mass=None, charge=None,
                            check_adiabaticity=False):
        """GuidingCenter.__init__ for all tracers (rapt/GuidingCenter.py:108-133):
        ppar from the pitch angle, mu = gamma^2 m v_perp^2 / (2 |B|)."""
        pos = np.asarray(pos, float).reshape(self.n, 3)
        v = np.broadcast_to(np.asarray(v, float), (self.n,)).copy()
        mass = np.broadcast_to(np.asarray(mass, float), (self.n,)).copy()
        t0a = np.broadcast_to(np.asarray(t0, float), (self.n,)).copy()
        gamma = 1.0 / np.sqrt(1.0 - (v / c) ** 2)
        if pa is not None:
            pa = np.broadcast_to(np.asarray(pa, float), (self.n,))
            vpar = np.where(pa == 90, 0.0, v * np.cos(pa * np.pi / 180))
            ppar = gamma * mass * vpar
        ppar = np.broadcast_to(np.asarray(ppar, float), (self.n,))
        Bmag = self.field.magB(np.column_stack([t0a, pos]))
        vpar = ppar / (mass * gamma)
        h = self.h
        h["mode"][:] = N.MODE_GC
        h["s"][0:3] = pos.T
        h["s"][3] = ppar
        h["s"][4:6] = 0.0
        h["mu"][:] = gamma ** 2 * mass * (v - vpar) * (v + vpar) / (2 * Bmag)
        h["v"][:] = v
        h["mass"][:] = mass
        h["charge"][:] = np.broadcast_to(np.asarray(charge, float), (self.n,))
        self._common(t0, check_adiabaticity)

    def _common(self, t0, check):
        h = self.h
        t0 = np.broadcast_to(np.asarray(t0, float), (self.n,))
        h["t_row"][:] = t0
        h["t_int"][:] = t0
        h["tcur"][:] = t0
        h["status"][:] = 0
        h["flags"][:] = np.where(np.broadcast_to(check, (self.n,)), N.FLAG_CHECK, 0)
        for k in ("naccept", "nreject", "nfcn", "nswitch"):
            h[k][:] = 0

    # ----------------------------------------------------------- running
    def configure(self, **cfg):
        """Set solver options; keys of rapt_config (rtol, atol, cyclotronresolution,
        gctimestep, epss, epst, enforce_equatorial, tableau, gc_eom, nsteps, form,
        collect, learned_scale, ...). Keys not given keep their earlier values."""
        merged = dict(self.config)
        merged.update(cfg)
        self.ctx.set_config(**merged)
        self.config = merged

    @classmethod
    def from_workload(cls, w, kind, max_rows=4, max_switch=0, ctx=None, pinned=False, **over):
        """Ensemble of a workload dict of ``rapt_gb300.workloads`` (field, params,
        positions and velocities or speeds and pitch angles), uploaded."""
        from . import fields as F
        name, kw = w["field"]
        ens = cls(getattr(F, name)(**kw), len(w["mass"]), max_rows=max_rows, max_switch=max_switch, ctx=ctx,
                  pinned=pinned)
        p = dict(w["params"])
        p.update(over)
        ens.configure(**p)
        if kind == "gc":
            ens.set_guiding_centers(w["pos"], w["v"], pa=w["pa"], t0=0.0, mass=w["mass"], charge=w["charge"])
        else:
            ens.set_particles(w["pos"], w["vel"], 0.0, w["mass"], w["charge"])
        ens.upload()
        if kind == "adaptive":
            ens.adaptive_init()
        return ens

    def adaptive_init(self):
        """Adaptive.__init__ mode pick on the device (rapt/Adaptive.py:95-104)."""
        self.ctx.check(self.ctx.L.rapt_adaptive_init(self.ctx.h), "rapt_adaptive_init")

    def advance(self, kind, delta):
        """Advance every tracer by ``delta`` (scalar or per-tracer array); returns stats."""
        kind = {"particle": N.KIND_PARTICLE, "gc": N.KIND_GC, "adaptive": N.KIND_ADAPTIVE}.get(kind, kind)
        self.field.bind(self.ctx)  # the context's field may have been changed by a field-method call
        st = N.RaptStats()
        if np.ndim(delta) == 0:
            rc = self.ctx.L.rapt_advance(self.ctx.h, int(kind), None, float(delta), N.ctypes_byref(st))
        else:
            d = np.ascontiguousarray(delta, dtype=np.float64)
            assert d.shape == (self.n,)
            rc = self.ctx.L.rapt_advance(self.ctx.h, int(kind), d.ctypes.data, 0.0, N.ctypes_byref(st))
        self.ctx.check(rc, "rapt_advance")
        self.last_stats = st.as_dict()
        return self.last_stats

    def advance_resume(self, kind):
        """Continue the last advance after tracers stopped with a full row buffer
        (drain it with ``rows(reset=True)`` first)."""
        kind = {"particle": N.KIND_PARTICLE, "gc": N.KIND_GC, "adaptive": N.KIND_ADAPTIVE}.get(kind, kind)
        self.field.bind(self.ctx)
        st = N.RaptStats()
        self.ctx.check(self.ctx.L.rapt_advance_resume(self.ctx.h, int(kind), N.ctypes_byref(st)), "rapt_advance_resume")
        self.last_stats = st.as_dict()
        return self.last_stats
