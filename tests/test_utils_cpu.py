"""The host-side closed-form helpers of rapt/utils.py in rapt_gb300.utils
(Walt's dipole bounce and drift periods, the dipole mirror field, the
bounce-centre drift error) against values from the unmodified reference
(tests/golden/make_utils_golden.py)."""
import os
import types

import numpy as np

from rapt_gb300 import utils as U

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "utils_golden.npz"))


def test_dipole_periods_and_mirror_field_match_reference():
    L, v, pa = G["L"], G["v"], G["eqpa"]
    for name, fn in (("bounce", U.dipole_bounce_period), ("drift_p", U.dipole_drift_period_p),
                     ("drift_e", U.dipole_drift_period_e)):
        got = np.array([fn(L[i], v[i], pa[i]) for i in range(len(L))])
        np.testing.assert_allclose(got, G[name], rtol=1e-14, atol=0, err_msg=name)
    got = np.array([U.dipoleBm(L[i], pa[i]) for i in range(len(L))])
    np.testing.assert_allclose(got, G["dipoleBm"], rtol=1e-14, atol=0)


def test_drift_error_matches_reference():
    b = types.SimpleNamespace(trajectory=G["drift_traj"])
    np.testing.assert_allclose(U.drift_error(b), G["drift_error"], rtol=0, atol=1e-15)
