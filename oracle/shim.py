"""Import the untouched RAPT reference for use as a test oracle.

TEST INFRASTRUCTURE ONLY. This module is imported by the golden-fixture
generator (tests/golden/make_golden.py) and by CPU tests that compare the C
restatement with the reference. It is never imported by the product package
``rapt_gb300``.

Two compatibility shims are applied, neither of which touches the reference
source tree:

* ``scipy.misc.derivative`` was removed in SciPy 1.12; ``rapt/flutils.py:19``
  imports it at module load, so a stand-in is installed first.
* ``Particle.__init__`` (``rapt/Particle.py:105``) and
  ``GuidingCenter.__init__`` (``rapt/GuidingCenter.py:123``) test
  ``pos == []``, which raises on numpy>=2 when ``pos`` is an ndarray. The
  wrappers below convert ndarray ``pos``/``vel`` to lists before calling the
  original constructors.
"""
import os
import sys
import types

import numpy as np

# The directory that holds the reference's ``rapt`` package; it must be named
# by the environment (the hosts that run the tests do not have it).
REFERENCE_ROOT = os.environ.get("RAPT_REFERENCE_ROOT", "")


def _install_scipy_misc():
    import scipy
    try:
        from scipy.misc import derivative  # noqa: F401
        return
    except Exception:
        pass

    def derivative(func, x0, dx=1.0, n=1, args=(), order=3):
        # Central difference, same contract as the removed scipy.misc.derivative
        # for the n=1, order=3 case used by rapt/flutils.py.
        if n != 1 or order != 3:
            raise NotImplementedError("shim supports n=1, order=3 only")
        return (func(x0 + dx, *args) - func(x0 - dx, *args)) / (2.0 * dx)

    mod = types.ModuleType("scipy.misc")
    mod.derivative = derivative
    sys.modules["scipy.misc"] = mod
    scipy.misc = mod


def load():
    """Return the reference ``rapt`` module, shimmed for numpy 2 / SciPy 1.18."""
    if "rapt" in sys.modules and getattr(sys.modules["rapt"], "_graft_shimmed", False):
        return sys.modules["rapt"]
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "rapt")):
        raise ImportError("RAPT reference not found: set RAPT_REFERENCE_ROOT to the directory holding rapt/ "
                          "(got %r)" % REFERENCE_ROOT)
    _install_scipy_misc()
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    sys.dont_write_bytecode = True
    import rapt  # noqa: E402

    P, G = rapt.Particle, rapt.GuidingCenter
    p_init, g_init = P.__init__, G.__init__

    def _aslist(a):
        return list(np.asarray(a, dtype=float)) if isinstance(a, np.ndarray) else a

    def p_init_shim(self, pos=[], vel=[], *a, **k):
        return p_init(self, _aslist(pos), _aslist(vel), *a, **k)

    def g_init_shim(self, pos=[], *a, **k):
        return g_init(self, _aslist(pos), *a, **k)

    P.__init__ = p_init_shim
    G.__init__ = g_init_shim
    rapt._graft_shimmed = True
    return rapt
