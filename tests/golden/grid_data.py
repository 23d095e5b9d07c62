"""Synthetic Grid snapshots shared by the fixture generator and the tests.

The snapshots are computed, not stored: only +, -, *, / and sqrt (correctly
rounded IEEE operations) are used, so x86 and aarch64 hosts build bit-identical
arrays and the committed reference outputs in grid_golden.npz apply to both.

Field: a dipole B = -B0 Re^3 (3xz, 3yz, 2z^2 - x^2 - y^2) / r^5 scaled by
(1 + 0.05 k) in snapshot k, and a dawn-dusk E_y = 2e-4 (1 + 0.1 (x/Re - 6))
(1 + 0.25 k) V/m with a small E_x = -1e-5 (y/Re) V/m. Axes in metres: x from
2.5 to 9.5 Re and y from -4 to 4 Re in steps of Re/4; z non-uniform,
z = (u + u^3/27) Re for u from -3 to 3 in steps of 1/4.
"""
import numpy as np

Re = 6378137.0
B0 = 3.07e-5


def axes():
    x = (2.5 + 0.25 * np.arange(29)) * Re
    y = (-4.0 + 0.25 * np.arange(33)) * Re
    u = -3.0 + 0.25 * np.arange(25)
    z = (u + u * u * u / 27.0) * Re
    return x, y, z


def snapshot(k, x, y, z):
    """Arrays of snapshot k as Grid.parsefile returns them (3-D, indexing ij)."""
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    r2 = X * X + Y * Y + Z * Z
    r = np.sqrt(r2)
    r5 = r2 * r2 * r
    c = -B0 * (Re * Re * Re) * (1.0 + 0.05 * k)
    g = {"Bx": c * (3.0 * X * Z) / r5, "By": c * (3.0 * Y * Z) / r5,
         "Bz": c * (2.0 * Z * Z - X * X - Y * Y) / r5}
    s = 1.0 + 0.25 * k
    g["Ex"] = -1e-5 * (Y / Re) * s
    g["Ey"] = 2e-4 * (1.0 + 0.1 * (X / Re - 6.0)) * s
    g["Ez"] = np.zeros_like(X)
    return g


def snapshots(times):
    """parsefile results for snapshots at the given times."""
    x, y, z = axes()
    out = []
    for k, t in enumerate(times):
        g = snapshot(k, x, y, z)
        g.update(time=float(t), x=x, y=y, z=z)
        out.append(g)
    return out


def stacked(times):
    """(t, x, y, z, B, E) with B, E of shape [nt][nx][ny][nz][3]."""
    snaps = snapshots(times)
    x, y, z = axes()
    B = np.stack([np.stack([g["Bx"], g["By"], g["Bz"]], -1) for g in snaps])
    E = np.stack([np.stack([g["Ex"], g["Ey"], g["Ez"]], -1) for g in snaps])
    return np.array(times, float), x, y, z, B, E


# snapshot times of the time-dependent cases: five files, so that the
# reference's three-snapshot window moves twice over 0..8 s
TIMES = (0.0, 2.0, 4.0, 6.0, 8.0)
