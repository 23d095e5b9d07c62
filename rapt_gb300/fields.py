"""Field models (rapt/fields.py) with device implementations.

Each class keeps the reference constructor, its ``gradientstepsize``,
``timederivstepsize`` and ``static`` attributes and the ``_Field`` methods.
The methods are evaluated by the GPU library (``rapt_field_eval``) and accept
either one (t, x, y, z) point, as in the reference, or an (n, 4) array.

A field with no device implementation -- ``Grid``, or any subclass that
overrides ``B`` or ``E`` -- raises ``NotImplementedError`` when a tracer is
advanced with it; there is no CPU fallback.
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
    """Gridded fields (rapt/fields.py:513-814) have no device implementation."""
    model_id = None

    def __init__(self, *args, **kwargs):
        _Field.__init__(self)


for _cls in (EarthDipole, DoubleDipole, UniformBz, UniformCrossedEB, VarEarthDipole, Parabolic, Harris,
             CompressedDipole):
    _cls._device_class = _cls
