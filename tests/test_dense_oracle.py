"""Dense output of the guiding-centre advance in the CPU oracle (an option of
the GPU library with no reference counterpart): the DOPRI5 continuous
extension's coefficients, and the dense advance against the reference's
restarting scheme and a tight-tolerance solution."""
import numpy as np

from rapt_gb300 import workloads as W
from tests._util import oracle_config, oracle_tracers, rel_state_error

# DOPRI5 tableau and the order-4 continuous extension (Hairer, Norsett & Wanner,
# Solving ODEs I, II.6), as the kernels and the oracle use them
A = [[], [1 / 5], [3 / 40, 9 / 40], [44 / 45, -56 / 15, 32 / 9],
     [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
     [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
     [35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]]
C = [0, 1 / 5, 3 / 10, 4 / 5, 8 / 9, 1, 1]
D = dict(d1=-12715105075.0 / 11282082432.0, d3=87487479700.0 / 32700410799.0,
         d4=-10690763975.0 / 1880347072.0, d5=701980252875.0 / 199316789632.0,
         d6=-1453857185.0 / 822651844.0, d7=69997945.0 / 29380423.0)


def _step(f, t, y, h):
    k = [f(t, y)]
    for s in range(1, 7):
        k.append(f(t + C[s] * h, y + h * sum(A[s][j] * k[j] for j in range(s))))
    return k, y + h * sum(A[6][j] * k[j] for j in range(6))


def _dense(y, y1, k, h, th):
    ydiff = y1 - y
    bspl = h * k[0] - ydiff
    r4 = ydiff - h * k[6] - bspl
    dd = h * (D["d1"] * k[0] + D["d3"] * k[2] + D["d4"] * k[3] + D["d5"] * k[4] + D["d6"] * k[5] + D["d7"] * k[6])
    th1 = 1 - th
    return y + th * (ydiff + th1 * (bspl + th * (r4 + th1 * dd)))


def test_continuous_extension_is_order_four():
    """The interpolant's local error at mid-step shrinks as h^5 (order 4), and it
    reproduces the step's end point and end slopes."""
    f = lambda t, y: np.array([y[1], -y[0] * (1 + 0.3 * np.sin(t))])  # noqa: E731
    y0 = np.array([1.0, 0.0])
    errs = []
    for h in (0.2, 0.1, 0.05):
        k, y1 = _step(f, 0.0, y0, h)
        yt, t = y0.copy(), 0.0
        for _ in range(200):  # fine reference to h/2
            _, yt = _step(f, t, yt, 0.5 * h / 200)
            t += 0.5 * h / 200
        errs.append(np.abs(_dense(y0, y1, k, h, 0.5) - yt).max())
        assert np.allclose(_dense(y0, y1, k, h, 1.0), y1, rtol=1e-15, atol=1e-15)
        eps = 1e-6
        slope0 = (_dense(y0, y1, k, h, eps) - y0) / (eps * h)
        assert np.allclose(slope0, k[0], rtol=1e-4, atol=1e-6)
    rate = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rate > 4.7), rate


def _run(oracle, w, delta, **over):
    f, cfg, tr = oracle_tracers(oracle, w, "gc")
    cfg = oracle_config(oracle, w, **over)
    for k, v in over.items():
        setattr(cfg, k, v)
    oracle.batch_advance(f, cfg, 1, tr, delta)
    return tr


def test_dense_advance_against_restarts_and_truth(oracle):
    """64 config-2 electrons for 5 s: at a 1 s cadence the dense advance is as
    accurate as the reference's restarting scheme; at a 0.01 s cadence it needs
    half the right-hand sides (the restarts force short steps) and stays within
    the tolerance-driven error. Rows land on the same times."""
    for cadence, max_ratio in ((1.0, 1.0), (0.01, 0.6)):
        w = W.subsample(W.config2(), np.arange(0, 65536, 1024))
        w["params"] = dict(w["params"], gctimestep=cadence)
        restart = _run(oracle, w, 5.0)
        dense = _run(oracle, w, 5.0, dense=1)
        truth = _run(oracle, w, 5.0, rtol=1e-11, atol=1e-11, nsteps=1000000)
        assert np.all(restart["status"] == 0) and np.all(dense["status"] == 0) and np.all(truth["status"] == 0)
        assert np.array_equal(dense["t"], restart["t"])
        er, _ = rel_state_error(restart["s"].T, truth["s"], 4)
        ed, _ = rel_state_error(dense["s"].T, truth["s"], 4)
        assert np.median(ed) < 3e-6 and ed.max() < 3e-5, (cadence, np.median(ed), ed.max())
        if cadence == 1.0:
            assert np.median(ed) < 2 * np.median(er), (np.median(ed), np.median(er))
        ratio = dense["nfcn"].sum() / restart["nfcn"].sum()
        assert ratio <= max_ratio, (cadence, ratio)


def test_dense_rows_and_adiabaticity_check(oracle):
    """Rows every cadence from the continuous extension; a NonAdiabatic check ends
    the call at the first failing row, in that row's state."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 4096))
    f, _, tr = oracle_tracers(oracle, w, "gc")
    cfg = oracle_config(oracle, w, gctimestep=0.05)
    cfg.dense = 1
    t = oracle.Tracer()
    import ctypes as C
    C.memmove(C.byref(t), tr[0:1].ctypes.data, C.sizeof(t))
    raised, rows = oracle.advance(f, cfg, t, 1.0)
    assert raised == 0 and len(rows) == 20
    assert np.allclose(rows[:, 0], 0.05 * np.arange(1, 21), rtol=1e-12)
    assert np.array_equal(rows[-1, 1:5], np.array(list(t.s)[:4])) and t.t == rows[-1, 0]
    # epss tiny: the first row is already non-adiabatic
    cfg.epss = 1e-12
    C.memmove(C.byref(t), tr[1:2].ctypes.data, C.sizeof(t))
    raised, rows = oracle.advance(f, cfg, t, 1.0, check=True)
    assert raised == 1 and len(rows) == 1 and t.t == rows[0, 0]
