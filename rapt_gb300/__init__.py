"""rapt_gb300 -- GB300-native ensemble tracer for RAPT's hot path.

Mirrors the reference package ``rapt`` (mkozturk/rapt): constants and the
``params`` dict (rapt/__init__.py:5-34), the ``Adiabatic``/``NonAdiabatic``
switch exceptions (:14-17), field models, and the ``Particle``,
``GuidingCenter`` and ``Adaptive`` tracers, whose ``advance`` runs on the GPU
through librapt_gpu.so. ``Ensemble`` and ``advance_batch`` advance many
tracers at once.
"""
# Constants, rapt/__init__.py:5-10
e = 1.602176565e-19
m_pr = 1.672621777e-27
m_el = 9.10938291e-31
c = 299792458
B0 = 3.07e-5
re = Re = 6378137


class Adiabatic(Exception):
    pass


class NonAdiabatic(Exception):
    pass


# rapt/__init__.py:21-34
params = {
    "cyclotronresolution": 10,
    "Ptimestep": 0,
    "bounceresolution": 10,
    "GCtimestep": 0,
    "BCtimestep": 0.1,
    "solvertolerances": (1.49012e-8, 1.49012e-8),
    "fieldlineresolution": 50,
    "flsolver": "rkf",
    "eyegradientstep": 0.03 * Re,
    "epss": 5e-2,
    "epst": 5e-2,
    "enforce equatorial": False,
    # no reference counterpart: guiding centres integrate through each advance()
    # without restarting at the output times; rows from the continuous extension
    "dense output": False,
}

from . import fields, workloads  # noqa: E402
from .ensemble import Ensemble  # noqa: E402
from . import utils  # noqa: E402
from . import flutils  # noqa: E402
from .flutils import eye, gradI, halfbouncepath  # noqa: E402,F401  (rapt/__init__.py:42)
from .tracers import Adaptive, BounceCenter, GuidingCenter, Particle, advance_batch  # noqa: E402
