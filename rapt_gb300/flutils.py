"""Field-line utilities of rapt/flutils.py on the device.

``halfbouncepath``, ``bounceperiod``, ``eye`` and ``gradI`` trace the field
lines on the GPU (``rapt_bc_eval``; one thread per point, arrays of points
accepted). The half-bounce path and the second invariant integrate the
quadratic spline of |B| between its brentq mirror points to convergence; the
reference uses QUADPACK at epsrel 1e-4 and, for the second invariant below 70
degrees equatorial pitch angle, a Simpson branch that raises NameError
(flutils.py:130). ``usedipole=True`` uses the closed dipole forms of
``rapt_gb300.utils``. ``eye_error`` is the difference of the two.
``criticalpoints`` (flutils.py:21-63) and ``fl_error`` (flutils.py:318-352),
which need the traced points of a field line, are not provided.
"""
import numpy as np

from . import _native as N
from . import utils as ru


def _ctx(field):
    from .tracers import _config
    ctx = N.default_context()
    field.bind(ctx)
    ctx.set_config(**_config())
    return ctx


def _points(tpos):
    tp = np.asarray(tpos, dtype=np.float64)
    return tp.reshape(-1, 4), tp.ndim == 1


def halfbouncepath(tpos, field, Bm):
    """flutils.halfbouncepath (flutils.py:254-316)."""
    tp, single = _points(tpos)
    out = _ctx(field).bc_eval("halfbouncepath", tp, Bm, 1.0)[:, 0]
    return out[0] if single else out


def bounceperiod(tpos, field, Bm, v):
    """flutils.bounceperiod (flutils.py:231-252): 2 / v times the half-bounce path."""
    return (2 / v) * halfbouncepath(tpos, field, Bm)


def eye(tpos, field, Bm, usedipole=False):
    """flutils.eye (flutils.py:65-151): the second invariant I."""
    if usedipole:
        t = np.asarray(tpos, float)
        return ru.dipoleI(np.sqrt(np.dot(t[1:3], t[1:3])), Bm)
    tp, single = _points(tpos)
    out = _ctx(field).bc_eval("eye", tp, Bm, 1.0)[:, 0]
    return out[0] if single else out


def gradI(tpos, field, Bm, usedipole=False):
    """flutils.gradI (flutils.py:153-229), step params["eyegradientstep"]."""
    from . import params
    d = params["eyegradientstep"]
    if usedipole:
        t = np.asarray(tpos, float)
        return ru.dipole_gradI(t[1], t[2], Bm, d)
    tp, single = _points(tpos)
    out = _ctx(field).bc_eval("gradI", tp, Bm, d)
    return out[0] if single else out


def eye_error(tpos, field, Bm):
    """flutils.eye_error (flutils.py:354-377): the second invariant from the
    field line minus the closed dipole form."""
    return eye(tpos, field, Bm, usedipole=False) - eye(tpos, field, Bm, usedipole=True)


def criticalpoints(tpos, field, Bm):
    raise NotImplementedError("flutils.criticalpoints is not on the device path")


def fl_error(tpos, field, Bm):
    raise NotImplementedError("flutils.fl_error needs the traced field-line points, which the device path "
                              "does not return")
