"""The allocation-free entry point rapt_gc_advance_noalloc against the regular
context-based path (rapt_advance), through the C ABI.

rapt_gc_advance_noalloc exists for callers that cannot call cudaMalloc (for
example a running real-time loop, or a library that owns device memory through
its own pool): they hand in device buffers they already own and the library
allocates nothing, keeping its scratch in a fixed __device__ array. This test
gives it buffers allocated by the test itself and checks that two calls in a
row produce what two rapt_advance calls produce on the same inputs.
"""
import ctypes as C

import numpy as np
import pytest

from rapt_gb300 import _native as N
from rapt_gb300 import workloads as W
from tests._util import gpu_ensemble

pytestmark = pytest.mark.gpu

N_TRACERS = 1024
MAX_ROWS = 4


def _config(w):
    cfg = N.RaptConfig()
    N.lib().rapt_config_default(C.byref(cfg))
    for k, v in w["params"].items():
        setattr(cfg, k, v)
    return cfg


def test_noalloc_matches_context_path_twice():
    import torch
    w = W.subsample(W.config2(), np.arange(0, 65536, 65536 // N_TRACERS))
    ens = gpu_ensemble(w, "gc", max_rows=MAX_ROWS)
    h0 = {k: v.copy() for k, v in ens.h.items()}  # the initial state the ensemble uploaded
    dev = torch.device("cuda:0")

    def t(a, dtype=torch.float64):
        return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

    n = len(w["mass"])
    buf = {"t": t(h0["t_row"]), "x": t(h0["s"][0]), "y": t(h0["s"][1]), "z": t(h0["s"][2]),
           "ppar": t(h0["s"][3]), "mu": t(h0["mu"]), "v": t(h0["v"]), "mass": t(h0["mass"]),
           "charge": t(h0["charge"]), "status": torch.zeros(n, dtype=torch.int32, device=dev),
           "naccept": torch.zeros(n, dtype=torch.int64, device=dev),
           "nreject": torch.zeros(n, dtype=torch.int64, device=dev),
           "nfcn": torch.zeros(n, dtype=torch.int64, device=dev),
           "rows": torch.zeros((n, MAX_ROWS, 7), dtype=torch.float64, device=dev),
           "row_mode": torch.zeros((n, MAX_ROWS), dtype=torch.int8, device=dev),
           "nrows": torch.zeros(n, dtype=torch.int32, device=dev)}
    st = N.RaptGcDeviceState()
    st.n = n
    st.max_rows = MAX_ROWS
    for k, v in buf.items():
        setattr(st, k, v.data_ptr())
    cfg = _config(w)
    params = np.ascontiguousarray(ens.field.device_params(), dtype=np.float64)
    stream = torch.cuda.current_stream(dev).cuda_stream

    for call in range(2):
        ref_stats = ens.advance("gc", 1.0)
        ref = ens.download()
        rows, row_mode, nrows, _, _ = ens.rows(reset=True)
        stats = N.RaptStats()
        rc = N.lib().rapt_gc_advance_noalloc(0, ens.field.model_id, params.ctypes.data_as(N._DP), len(params),
                                             C.byref(cfg), C.byref(st), 1.0, stream, C.byref(stats))
        assert rc == N.RAPT_OK, rc
        torch.cuda.synchronize(dev)
        got = {k: v.cpu().numpy() for k, v in buf.items()}
        for k, j in (("x", 0), ("y", 1), ("z", 2), ("ppar", 3)):
            np.testing.assert_allclose(got[k], ref["s"][j], rtol=1e-12, atol=0, err_msg="call %d %s" % (call, k))
        np.testing.assert_allclose(got["t"], ref["t_row"], rtol=1e-12, atol=0)
        assert np.array_equal(got["status"], ref["status"])
        for k in ("naccept", "nreject", "nfcn"):
            assert np.array_equal(got[k], ref[k]), (call, k)
        assert np.array_equal(got["nrows"], nrows) and nrows.min() >= 1
        # every row this call produced (the end-of-interval rows included) and its mode
        for k in range(n):
            m = nrows[k]
            np.testing.assert_allclose(got["rows"][k, :m], rows[k, :m], rtol=1e-12, atol=1e-300,
                                       err_msg="call %d tracer %d" % (call, k))
            assert np.array_equal(got["row_mode"][k, :m], row_mode[k, :m]), (call, k)
        assert stats.accepted == ref_stats["accepted"] > 0


def test_noalloc_rejects_what_it_does_not_run():
    """The default configuration has GCtimestep = 0 (bounce-period cadence), which
    this path does not run: the call must refuse it, not report success with
    every tracer unadvanced. The same for the other forms."""
    st = N.RaptGcDeviceState()
    st.n = 16
    st.max_rows = MAX_ROWS
    cfg = N.RaptConfig()
    N.lib().rapt_config_default(C.byref(cfg))
    rc = N.lib().rapt_gc_advance_noalloc(0, 1, None, 0, C.byref(cfg), C.byref(st), 1.0, None, None)
    assert rc == N.RAPT_ERR_UNSUPPORTED
    cfg.gctimestep = 1.0
    cfg.form = 1
    rc = N.lib().rapt_gc_advance_noalloc(0, 1, None, 0, C.byref(cfg), C.byref(st), 1.0, None, None)
    assert rc == N.RAPT_ERR_UNSUPPORTED


def test_noalloc_rejects_too_many_tracers():
    st = N.RaptGcDeviceState()
    st.n = N.NOALLOC_MAX_TRACERS + 1
    st.max_rows = MAX_ROWS
    cfg = N.RaptConfig()
    N.lib().rapt_config_default(C.byref(cfg))
    rc = N.lib().rapt_gc_advance_noalloc(0, 1, None, 0, C.byref(cfg), C.byref(st), 1.0, None, None)
    assert rc == N.RAPT_ERR_INVALID
