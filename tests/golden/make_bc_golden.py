#!/usr/bin/env python3
"""Generate tests/golden/bc_golden.npz from the unmodified RAPT reference:
the second invariant (flutils.eye), its gradient (flutils.gradI), the dipole
formula utils.dipoleI, and BounceCenter trajectories.

Run where the reference is checked out, with RAPT_REFERENCE_ROOT naming that
directory; only the .npz travels. The reference is imported through
oracle/shim.py and used unmodified.

Reference behaviour recorded here:
  * flutils.eye below 70 degrees equatorial pitch angle takes its Simpson
    branch, which calls the name simps that flutils.py never imports
    (flutils.py:18 imports simpson, :130 calls simps): NameError. Those cases
    are recorded as NaN; utils.dipoleI gives the dipole answer for them.
  * BounceCenter.__init__ passes the pitch angle in degrees to np.cos
    (BounceCenter.py:104), so pa = 80 means cos(80 rad).
  * BounceCenter.advance stamps each row with the time its interval began
    (np.arange(tcur, tcur + delta, dt), BounceCenter.py:249-251).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import shim  # noqa: E402

rapt = shim.load()
from rapt import flutils, utils  # noqa: E402

Re, m_pr, e = rapt.Re, rapt.m_pr, rapt.e


def main():
    out = {}
    F = rapt.fields
    fields = {"EarthDipole": F.EarthDipole(), "DoubleDipole": F.DoubleDipole()}
    # ---- eye: model id, L, equatorial pitch angle, Bm, I (NaN where it raises)
    rows = []
    for mid, name in ((0, "EarthDipole"), (1, "DoubleDipole")):
        fld = fields[name]
        for L in (4.0, 5.0, 6.5):
            tpos = np.array([0.0, L * Re, 0.0, 0.0])
            B0 = fld.magB(tpos)
            for eqpa in (40.0, 60.0, 72.0, 78.0, 85.0, 89.0):
                Bm = B0 / np.sin(np.deg2rad(eqpa)) ** 2
                try:
                    eye = flutils.eye(tpos, fld, Bm)
                except NameError:
                    eye = np.nan
                dip = utils.dipoleI(L * Re, Bm) if name == "EarthDipole" else np.nan
                rows.append([mid, L, eqpa, Bm, eye, dip])
    out["eye"] = np.array(rows)
    # ---- gradI at off-axis points (eyegradientstep 0.03 Re)
    rows = []
    for mid, name in ((0, "EarthDipole"), (1, "DoubleDipole")):
        fld = fields[name]
        for pos in ((6 * Re, 0, 0), (5 * Re, 2 * Re, 0), (-4 * Re, 3 * Re, 0.2 * Re)):
            tpos = np.r_[0.0, pos]
            Bm = fld.magB(tpos) / np.sin(np.deg2rad(80.0)) ** 2
            g = flutils.gradI(tpos, fld, Bm)
            rows.append([mid, *pos, Bm, *g])
    # a near-equatorial case: at one difference point the trimmed field line has
    # three samples (the spline branch on three points)
    fld = fields["DoubleDipole"]
    pos = (-38844185.468142495, 20985542.417829778, 0.0)
    tpos = np.r_[0.0, pos]
    Bm = fld.magB(tpos) * 1.0130884856
    rows.append([1, *pos, Bm, *flutils.gradI(tpos, fld, Bm)])
    out["gradI"] = np.array(rows)
    # ---- BounceCenter: 1 MeV protons, pa = 80 (cos of 80 rad), advance(0.35 bounce periods)
    rows = []
    for mid, name in ((0, "EarthDipole"), (1, "DoubleDipole")):
        fld = fields[name]
        v = utils.speedfromKE(1e6, m_pr)
        b = rapt.BounceCenter([6 * Re, 0, 0], v, 0, 80, m_pr, e, fld)
        gamma = 1 / np.sqrt(1 - (v / rapt.c) ** 2)
        Bm = m_pr * gamma ** 2 * v ** 2 / (2 * b.mu)
        bp = flutils.bounceperiod(b.trajectory[-1, :4], fld, Bm, v)
        b.advance(0.35 * bp)
        out["bc_%s_rows" % name] = b.trajectory
        rows.append([mid, v, 80.0, m_pr, e, b.mu, bp, 0.35 * bp, b.tcur])
    out["bc_cases"] = np.array(rows)  # model, v, pa, mass, charge, mu, bounce period, delta, tcur
    dst = os.path.join(HERE, "bc_golden.npz")
    np.savez_compressed(dst, **out)
    for k in sorted(out):
        print(k, np.shape(out[k]))


if __name__ == "__main__":
    main()
