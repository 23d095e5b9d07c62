#!/usr/bin/env python3
"""Generate tests/golden/utils_golden.npz by running the unmodified RAPT
reference's closed-form helpers (rapt/utils.py: dipole_bounce_period,
dipole_drift_period_p, dipole_drift_period_e, dipoleBm, drift_error).

Run where the reference is checked out, with RAPT_REFERENCE_ROOT naming that
directory; the hosts that run the tests do not need it -- only the .npz
travels. The reference is imported through oracle/shim.py.
"""
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import shim  # noqa: E402

rapt = shim.load()
U = sys.modules["rapt.utils"]

rng = np.random.default_rng(21)
n = 64
L = rng.uniform(2, 9, n)
v = rapt.c * rng.uniform(0.05, 0.999, n)
eqpa = rng.uniform(5, 90, n)
out = {"L": L, "v": v, "eqpa": eqpa,
       "bounce": np.array([U.dipole_bounce_period(L[i], v[i], eqpa[i]) for i in range(n)]),
       "drift_p": np.array([U.dipole_drift_period_p(L[i], v[i], eqpa[i]) for i in range(n)]),
       "drift_e": np.array([U.dipole_drift_period_e(L[i], v[i], eqpa[i]) for i in range(n)]),
       "dipoleBm": np.array([U.dipoleBm(L[i], eqpa[i]) for i in range(n)])}
# drift_error reads only b.trajectory[:, 1:]: a stand-in object with a trajectory
traj = np.column_stack([np.arange(20.0), 5 * rapt.Re * (1 + 1e-3 * rng.standard_normal((20, 3)))])
out["drift_traj"] = traj
out["drift_error"] = U.drift_error(types.SimpleNamespace(trajectory=traj))
np.savez(os.path.join(os.path.dirname(os.path.abspath(__file__)), "utils_golden.npz"), **out)
print("wrote utils_golden.npz", {k: np.shape(v) for k, v in out.items()})
