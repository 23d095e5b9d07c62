"""Field models (rapt/fields.py) with device implementations.

Each class keeps the reference constructor, its ``gradientstepsize``,
``timederivstepsize`` and ``static`` attributes and the ``_Field`` methods.
The methods are evaluated by the GPU library (``rapt_field_eval``) and accept
either one (t, x, y, z) point, as in the reference, or an (n, 4) array.

A field with no device implementation -- any subclass that overrides ``B``
or ``E`` -- raises ``NotImplementedError`` when a tracer is advanced with it;
there is no CPU fallback.
"""
import numpy as np

from . import _native as N

Re = 6378137
B0 = 3.07e-5


class _Field:
    """Base class, rapt/fields.py:5-280."""
    model_id = None
    _device_class = None

    def __init__(self):
        self.gradientstepsize = 1e-6
        self.timederivstepsize = 1e-3
        self.static = True

    # ---- device binding
    def device_params(self):
        raise NotImplementedError

    def has_device_impl(self):
        dc = self._device_class
        return (dc is not None and self.model_id is not None and type(self).B is dc.B and type(self).E is dc.E)

    def bind(self, ctx):
        """Load this field's model and parameters into a library context."""
        if not self.has_device_impl():
            raise NotImplementedError("%s has no device implementation; rapt_gb300 has no CPU fallback"
                                      % type(self).__name__)
        ctx.set_field(self.model_id, self.device_params(), self.gradientstepsize, self.timederivstepsize)

    def _eval(self, what, tpos):
        ctx = N.default_context()
        self.bind(ctx)
        tp = np.asarray(tpos, dtype=np.float64)
        single = tp.ndim == 1
        out = ctx.field_eval(what, tp.reshape(-1, 4))
        return out[0] if single else out

    # ---- _Field API
    def B(self, tpos):
        r = self._eval("B", tpos)
        return r[..., :3]

    def E(self, tpos):
        r = self._eval("E", tpos)
        return r[..., :3]

    def unitb(self, tpos):
        return self._eval("unitb", tpos)[..., :3]

    def magB(self, tpos):
        return self._eval("magB", tpos)[..., 0]

    def gradB(self, tpos):
        return self._eval("gradB", tpos)[..., :3]

    def jacobianB(self, tpos):
        r = self._eval("jacobianB", tpos)
        return r.reshape(r.shape[:-1] + (3, 3))

    def curvature(self, tpos):
        # fields.py:155-174; np.dot(gB, B) with the scalar |B| is elementwise there.
        Bv = self.B(tpos)
        Bm = np.sqrt(np.sum(Bv * Bv, axis=-1, keepdims=True))
        gB = self.gradB(tpos)
        gp = gB - (gB * Bm / Bm ** 2) * Bv
        return (np.sqrt(np.sum(gp * gp, axis=-1, keepdims=True)) / Bm)[..., 0]

    def curlb(self, tpos):
        return self._eval("curlb", tpos)[..., :3]

    def dBdt(self, tpos):
        if self.static:
            return 0
        return self._eval("dBdt", tpos)[..., 0]

    def dbdt(self, tpos):
        if self.static:
            return 0
        return self._eval("dbdt", tpos)[..., :3]

    def lengthscale(self, tpos):
        return self._eval("lengthscale", tpos)[..., 0]

    def timescale(self, tpos):
        if self.static:
            return None
        return self._eval("timescale", tpos)[..., 0]


class EarthDipole(_Field):
    """rapt/fields.py:282-317."""
    model_id = N.MODEL_IDS["EarthDipole"]

    def __init__(self, B0=B0):
        _Field.__init__(self)
        self.gradientstepsize = Re * 1e-6
        self.B0_ = B0
        self._coeff = -3 * B0 * Re ** 3

    def device_params(self):
        return [self.B0_]


class DoubleDipole(_Field):
    """rapt/fields.py:319-362."""
    model_id = N.MODEL_IDS["DoubleDipole"]

    def __init__(self, B0=B0, distance=20 * Re, imagestrength=1):
        _Field.__init__(self)
        self.gradientstepsize = Re / 1000
        self._dd = distance
        assert imagestrength >= 1
        self._k = imagestrength
        self.B0_ = B0
        self._coeff = -B0 * Re ** 3

    def device_params(self):
        return [self.B0_, self._dd, self._k]


class UniformBz(_Field):
    """rapt/fields.py:364-390."""
    model_id = N.MODEL_IDS["UniformBz"]

    def __init__(self, Bz=1):
        _Field.__init__(self)
        self.Bz = Bz

    def device_params(self):
        return [self.Bz]


class UniformCrossedEB(UniformBz):
    """rapt/fields.py:392-427."""
    model_id = N.MODEL_IDS["UniformCrossedEB"]

    def __init__(self, Ey=1, Bz=1):
        UniformBz.__init__(self)
        self.static = False
        self.Ey = Ey
        self.Bz = Bz

    def device_params(self):
        return [self.Ey, self.Bz]


class VarEarthDipole(_Field):
    """rapt/fields.py:429-470 (induced E ignored, as in the reference)."""
    model_id = N.MODEL_IDS["VarEarthDipole"]

    def __init__(self, amp=0.1, period=10):
        _Field.__init__(self)
        self.gradientstepsize = Re / 1000
        self.static = False
        self._amp = amp
        self._period = period

    def device_params(self):
        return [self._amp, self._period]


class Parabolic(_Field):
    """rapt/fields.py:472-511 (|z| > 1 uses the module-level B0, as in the reference)."""
    model_id = N.MODEL_IDS["Parabolic"]

    def __init__(self, B0=10.0, Bn=1.0, d=0.2):
        _Field.__init__(self)
        self.B0 = B0
        self.Bn = Bn
        self.d = d

    def device_params(self):
        return [self.B0, self.Bn, self.d]


class Harris(_Field):
    """Harris current sheet with a normal component and a uniform dawn-dusk E field:
    B = (B0 tanh(z/L), 0, Bn), E = (0, Ey, 0). Not in the reference.
    Finite-difference step L * 1e-4."""
    model_id = N.MODEL_IDS["Harris"]

    def __init__(self, B0=20e-9, L=0.5 * Re, Bn=2e-9, Ey=0.2e-3):
        _Field.__init__(self)
        self.static = False
        self.B0, self.L, self.Bn, self.Ey = B0, L, Bn, Ey
        self.gradientstepsize = L * 1e-4

    def device_params(self):
        return [self.B0, self.L, self.Bn, self.Ey]


class CompressedDipole(_Field):
    """Breathing dipole B0(t) = B0 (1 + amp sin(2 pi t / period)) in the
    VarEarthDipole form, with its induced azimuthal electric field
    E = -dB0/dt Re^3 (y, -x, 0) / r^3. Not in the reference."""
    model_id = N.MODEL_IDS["CompressedDipole"]

    def __init__(self, B0=B0, amp=0.1, period=60.0):
        _Field.__init__(self)
        self.gradientstepsize = Re / 1000
        self.static = False
        self.B0_, self._amp, self._period = B0, amp, period

    def device_params(self):
        return [self.B0_, self._amp, self._period]


class Grid(_Field):
    """Gridded fields, rapt/fields.py:513-814, interpolated on the device.

    Subclass and override ``parsefile`` as in the reference: it returns a dict
    with "time", the axes "x", "y", "z" and the 3-D arrays "Bx" .. "Ez" of one
    snapshot. The constructor parses every file of ``filelist`` (ordered in time)
    and uploads all snapshots to the device on first use; the reference keeps a
    window of three and re-parses as tracers move (fields.py:695-705), which gives
    the same interpolated values. One file: a time-independent field (3-D
    interpolation). Interpolation is SciPy's RegularGridInterpolator "linear",
    restated bit for bit in the device kernels.

    ``B``/``E`` (or ``Bgrid``/``Egrid``) outside the grid raise ValueError as the
    reference's interpolator does; a tracer that steps outside the grid stops
    with status OUT_OF_GRID. ``static`` stays True as in the reference
    (fields.py:41): set it to False for time-dependent data or a nonzero E.
    """
    model_id = N.MODEL_IDS["Grid"]
    _uids = iter(range(1, 1 << 62))

    def __init__(self, filelist):
        assert len(filelist) > 0
        _Field.__init__(self)
        self.gradientstepsize = 1e-3 * Re  # fields.py:578
        snaps = [self.parsefile(fn) for fn in filelist]
        g0 = snaps[0]
        self._x, self._y, self._z = (np.ascontiguousarray(g0[k], dtype=np.float64) for k in ("x", "y", "z"))
        for g in snaps[1:]:
            for k in ("x", "y", "z"):
                if not np.array_equal(np.asarray(g[k], dtype=np.float64), getattr(self, "_" + k)):
                    raise ValueError("grid coordinates must be the same in every file")
        self._t = np.array([float(g["time"]) for g in snaps])
        self._B = np.ascontiguousarray(np.stack([np.stack([g["Bx"], g["By"], g["Bz"]], -1) for g in snaps]),
                                       dtype=np.float64)
        E = np.ascontiguousarray(np.stack([np.stack([g["Ex"], g["Ey"], g["Ez"]], -1) for g in snaps]),
                                 dtype=np.float64)
        self._E = None if not np.any(E) else E  # all-zero E: the kernels skip the loads
        self._finite = bool(np.isfinite(self._B).all() and (self._E is None or np.isfinite(self._E).all()))
        self._time_indep = len(snaps) == 1
        self.t0 = self._t[0]
        if len(snaps) >= 2:
            self.t1 = self._t[1]
        if len(snaps) >= 3:
            self.t2 = self._t[2]
        self.files = []  # every file has been parsed
        self._uid = next(Grid._uids)

    def parsefile(self, filename):
        """Parse one snapshot file (fields.py:599-625); override when subclassing."""
        return dict()

    def bind(self, ctx):
        if not self.has_device_impl():
            raise NotImplementedError("%s overrides B or E; rapt_gb300 has no CPU fallback" % type(self).__name__)
        if getattr(ctx, "_grid_uid", None) != self._uid:
            ctx.grid_set(self._t, self._x, self._y, self._z, self._B, self._E)
            ctx._grid_uid = self._uid
        ctx.set_field(self.model_id, (), self.gradientstepsize, self.timederivstepsize)
        ctx.set_static(self.static)

    def _check_bounds(self, tpos):
        # RegularGridInterpolator's bounds check (bounds_error=True)
        tp = np.atleast_2d(np.asarray(tpos, dtype=np.float64))
        axes = [self._x, self._y, self._z]
        cols = [1, 2, 3]
        if not self._time_indep:
            axes, cols = [self._t] + axes, [0] + cols
        for d, (g, c) in enumerate(zip(axes, cols)):
            p = tp[:, c]
            if not np.logical_and(np.all(g[0] <= p), np.all(p <= g[-1])):
                raise ValueError("One of the requested xi is out of bounds in dimension %d" % d)

    def _eval(self, what, tpos):
        if what in ("B", "E"):
            self._check_bounds(tpos)
        out = _Field._eval(self, what, tpos)
        if self._finite and np.isnan(out).any():
            raise ValueError("One of the requested xi is out of bounds (a difference stencil left the grid)")
        return out

    def Bgrid(self, tpos):
        """fields.py:707-738."""
        return _Field.B(self, tpos)

    def Egrid(self, tpos):
        """fields.py:740-771."""
        return _Field.E(self, tpos)

    def B(self, tpos):
        return self.Bgrid(tpos)

    def E(self, tpos):
        return self.Egrid(tpos)


for _cls in (EarthDipole, DoubleDipole, UniformBz, UniformCrossedEB, VarEarthDipole, Parabolic, Harris,
             CompressedDipole, Grid):
    _cls._device_class = _cls
