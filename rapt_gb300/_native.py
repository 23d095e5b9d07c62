"""ctypes binding of librapt_gpu.so (declared in include/rapt_gpu.h).

The library is built in-tree by ``rapt_gb300/build.py``. There is no CPU
fallback: if the library is missing or no CUDA device is usable, the calls
raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librapt_gpu.so")

RAPT_OK, RAPT_ERR_INVALID, RAPT_ERR_CUDA, RAPT_ERR_NOMEM, RAPT_ERR_UNSUPPORTED, RAPT_ERR_STATE = range(6)
MODEL_IDS = {"EarthDipole": 0, "DoubleDipole": 1, "UniformBz": 2, "UniformCrossedEB": 3,
             "VarEarthDipole": 4, "Parabolic": 5, "Harris": 6, "CompressedDipole": 7, "Grid": 8}
MODE_PARTICLE, MODE_GC = 0, 1
KIND_PARTICLE, KIND_GC, KIND_ADAPTIVE = 0, 1, 2
FORMS = {"plain": 0, "fp32": 1, "learned": 2, "learned_fp32": 3}
ST = dict(OK=0, MAXSTEPS=2, HMIN=3, NONFINITE=4, GC_NOCONV=5, ROWS_FULL=6, BAD_INPUT=7, FIELDLINE=10,
          RKF_HMIN=8, ADAPTIVE_LIMIT=9, OUT_OF_GRID=11)
FLAG_CHECK, FLAG_RAISED, FLAG_DONE = 1, 2, 4
FIELD_QUANTITIES = {"B": 0, "E": 1, "gradB": 2, "curlb": 3, "magB": 4, "unitb": 5,
                    "lengthscale": 6, "dbdt": 7, "jacobianB": 8, "dBdt": 9, "timescale": 10}


class RaptConfig(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("cyclotronresolution", C.c_double),
                ("gctimestep", C.c_double), ("epss", C.c_double), ("epst", C.c_double),
                ("enforce_equatorial", C.c_int32), ("tableau", C.c_int32), ("gc_eom", C.c_int32),
                ("nsteps", C.c_int32), ("rkf_tol", C.c_double), ("rkf_hmin", C.c_double),
                ("form", C.c_int32), ("threads_per_block", C.c_int32),
                ("max_steps_per_launch", C.c_int64), ("blocks_per_sm", C.c_int32),
                ("use_graph", C.c_int32), ("collect", C.c_int32), ("learned_scale", C.c_double),
                ("learned_every", C.c_int32), ("per_tracer_launches", C.c_int32),
                ("bounceresolution", C.c_double), ("fieldlineresolution", C.c_double),
                ("dense_output", C.c_int32)]


class RaptHostState(C.Structure):
    _fields_ = [("n", C.c_int64), ("mode", C.c_void_p), ("status", C.c_void_p), ("flags", C.c_void_p),
                ("t_int", C.c_void_p), ("t_row", C.c_void_p), ("tcur", C.c_void_p),
                ("s", C.c_void_p * 6), ("mu", C.c_void_p), ("v", C.c_void_p), ("mass", C.c_void_p),
                ("charge", C.c_void_p), ("naccept", C.c_void_p), ("nreject", C.c_void_p),
                ("nfcn", C.c_void_p), ("nswitch", C.c_void_p)]


class RaptStats(C.Structure):
    _fields_ = [("accepted", C.c_int64), ("rejected", C.c_int64), ("rhs_evals", C.c_int64),
                ("switches", C.c_int64), ("done", C.c_int64), ("failed", C.c_int64),
                ("launches", C.c_int64), ("kernel_launches", C.c_int64), ("kernel_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol include/rapt_gpu.h declares, with its ctypes signature.
_VP, _D, _I, _I64 = C.c_void_p, C.c_double, C.c_int, C.c_int64
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "rapt_abi_version": (C.c_int, []),
    "rapt_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "rapt_ctx_destroy": (None, [_VP]),
    "rapt_last_error": (C.c_char_p, [_VP]),
    "rapt_field_set": (C.c_int, [_VP, C.c_int, _DP, C.c_int]),
    "rapt_field_set_steps": (C.c_int, [_VP, _D, _D]),
    "rapt_field_set_static": (C.c_int, [_VP, C.c_int]),
    "rapt_bc_advance": (C.c_int, [_VP, _I64, _VP, _VP, _D, _D, _D, _VP, C.c_int32, _VP, _VP, _VP]),
    "rapt_bc_eval": (C.c_int, [_VP, C.c_int, _I64, _VP, _VP, _D, _VP, _VP]),
    "rapt_grid_set": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, _VP, C.c_int32, _VP, C.c_int32, _VP, _VP, _VP]),
    "rapt_config_default": (None, [C.POINTER(RaptConfig)]),
    "rapt_config_set": (C.c_int, [_VP, C.POINTER(RaptConfig)]),
    "rapt_ensemble_alloc": (C.c_int, [_VP, _I64, C.c_int32, C.c_int32]),
    "rapt_ensemble_upload": (C.c_int, [_VP, C.POINTER(RaptHostState)]),
    "rapt_ensemble_download": (C.c_int, [_VP, C.POINTER(RaptHostState)]),
    "rapt_rows_download": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, C.c_int]),
    "rapt_advance": (C.c_int, [_VP, C.c_int, _VP, _D, C.POINTER(RaptStats)]),
    "rapt_advance_resume": (C.c_int, [_VP, C.c_int, C.POINTER(RaptStats)]),
    "rapt_adaptive_init": (C.c_int, [_VP]),
    "rapt_field_eval": (C.c_int, [_VP, C.c_int, _I64, _VP, _VP]),
    "rapt_rhs_eval": (C.c_int, [_VP, C.c_int, _I64, _VP, _VP, _VP, _VP, _VP]),
    "rapt_measure_peaks": (C.c_int, [_VP, _DP, _DP]),
    "rapt_host_register": (C.c_int, [_VP, C.c_uint64]),
    "rapt_host_unregister": (C.c_int, [_VP]),
    "rapt_gc_advance_noalloc": (C.c_int, [C.c_int, C.c_int, _DP, C.c_int, C.POINTER(RaptConfig), _VP, _D, _VP,
                                          C.POINTER(RaptStats)]),
    "rapt_gc_bounce_period": (C.c_int, [_VP, _I64, _VP, _VP]),
    "rapt_mlp_set_params": (C.c_int, [_VP, _VP, C.c_int32]),
    "rapt_mlp_get_params": (C.c_int, [_VP, _VP, C.c_int32]),
    "rapt_mlp_forward": (C.c_int, [_VP, _VP, _I64, _VP]),
    "rapt_mlp_grad": (C.c_int, [_VP, _VP, _I64, C.c_float, _VP, _DP]),
    "rapt_mlp_samples_reserve": (C.c_int, [_VP, _I64, C.c_uint64]),
    "rapt_mlp_samples_count": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "rapt_mlp_samples_download": (C.c_int, [_VP, _VP, _I64, _I64]),
    "rapt_mlp_samples_upload": (C.c_int, [_VP, _VP, _I64]),
    "rapt_mlp_samples_sort": (C.c_int, [_VP, _I64, _I64]),
    "rapt_mlp_train": (C.c_int, [_VP, _I64, C.c_int32, C.c_float, C.c_float, C.c_uint64, _DP]),
}

# Step-size MLP layout (include/rapt_gpu.h RAPT_MLP_*)
MLP_NPARAMS = 5816
MLP_NTRAIN = 5768
MLP_SAMPLE = 18

NOALLOC_MAX_TRACERS = 65536


class RaptGcDeviceState(C.Structure):
    """rapt_gc_device_state: device pointers of a caller-owned guiding-centre ensemble."""
    _fields_ = [("n", C.c_int64), ("t", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("ppar", C.c_void_p), ("mu", C.c_void_p), ("v", C.c_void_p), ("mass", C.c_void_p),
                ("charge", C.c_void_p), ("status", C.c_void_p), ("naccept", C.c_void_p),
                ("nreject", C.c_void_p), ("nfcn", C.c_void_p), ("rows", C.c_void_p), ("row_mode", C.c_void_p),
                ("nrows", C.c_void_p), ("max_rows", C.c_int32)]

_lib = None


class RaptError(RuntimeError):
    pass


def lib():
    """Load librapt_gpu.so; raises ImportError if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("librapt_gpu.so is not built (run `python rapt_gb300/build.py`); "
                              "rapt_gb300 has no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else a.ctypes.data


def ctypes_byref(obj):
    return C.byref(obj)


class Context:
    """One CUDA context + stream of the library (rapt_ctx_*)."""

    def __init__(self, device=0):
        self.L = lib()
        h = C.c_void_p()
        rc = self.L.rapt_ctx_create(int(device), C.byref(h))
        if rc != RAPT_OK or not h.value:
            raise RaptError("rapt_ctx_create(device=%d) failed with code %d (no usable CUDA device?)" % (device, rc))
        self.h = h
        self.device = device

    def check(self, rc, what):
        if rc != RAPT_OK:
            msg = self.L.rapt_last_error(self.h)
            raise RaptError("%s failed (code %d): %s" % (what, rc, msg.decode() if msg else ""))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.rapt_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_field(self, model_id, params=(), gradientstepsize=None, timederivstepsize=None):
        p = np.ascontiguousarray(params, dtype=np.float64)
        self.check(self.L.rapt_field_set(self.h, int(model_id), p.ctypes.data_as(_DP), len(p)), "rapt_field_set")
        if gradientstepsize is not None or timederivstepsize is not None:
            self.check(self.L.rapt_field_set_steps(self.h, float(gradientstepsize), float(timederivstepsize)),
                       "rapt_field_set_steps")

    def set_static(self, is_static):
        self.check(self.L.rapt_field_set_static(self.h, 1 if is_static else 0), "rapt_field_set_static")

    def grid_set(self, t, x, y, z, B, E=None):
        """Upload Grid snapshots (B, E: [nt][nx][ny][nz][3]) and select the Grid model."""
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (t, x, y, z)]
        nt, nx, ny, nz = (len(v) for v in a)
        B = np.ascontiguousarray(B, dtype=np.float64)
        if B.shape != (nt, nx, ny, nz, 3):
            raise ValueError("B must have shape %s, got %s" % ((nt, nx, ny, nz, 3), B.shape))
        if E is not None:
            E = np.ascontiguousarray(E, dtype=np.float64)
            if E.shape != B.shape:
                raise ValueError("E must have the shape of B")
        self.check(self.L.rapt_grid_set(self.h, nt, ptr(a[0]), nx, ptr(a[1]), ny, ptr(a[2]), nz, ptr(a[3]),
                                        ptr(B), ptr(E) if E is not None else None), "rapt_grid_set")

    def bc_advance(self, state, cst, delta, bctimestep, eyegradientstep, max_rows):
        """BounceCenter.advance for n bounce centres: state[n][5] (t, x, y, z, tcur)
        updated in place; returns (rows[n, max_rows, 4], nrows, status, counters)."""
        state = np.ascontiguousarray(state, dtype=np.float64)
        cst = np.ascontiguousarray(cst, dtype=np.float64)
        n = state.shape[0]
        rows = np.zeros((n, max_rows, 4))
        nrows = np.zeros(n, np.int32)
        status = np.zeros(n, np.int32)
        cnt = np.zeros((n, 4), np.int64)
        self.check(self.L.rapt_bc_advance(self.h, n, ptr(state), ptr(cst), float(delta), float(bctimestep),
                                          float(eyegradientstep), ptr(rows), int(max_rows), ptr(nrows), ptr(status),
                                          ptr(cnt)), "rapt_bc_advance")
        return state, rows, nrows, status, cnt

    def bc_eval(self, what, tpos, Bm, eyegradientstep, cst=None):
        tpos = np.ascontiguousarray(np.atleast_2d(tpos), dtype=np.float64)
        n = tpos.shape[0]
        Bm = np.ascontiguousarray(np.broadcast_to(np.asarray(Bm, float), (n,)))
        c = None if cst is None else np.ascontiguousarray(np.broadcast_to(np.asarray(cst, float), (n, 4)))
        out = np.zeros((n, 3))
        what = {"eye": 0, "gradI": 1, "drift": 2, "halfbouncepath": 3}.get(what, what)
        self.check(self.L.rapt_bc_eval(self.h, int(what), n, ptr(tpos), ptr(Bm), float(eyegradientstep), ptr(c),
                                       ptr(out)), "rapt_bc_eval")
        return out

    def set_config(self, **kw):
        cfg = RaptConfig()
        self.L.rapt_config_default(C.byref(cfg))
        for k, v in kw.items():
            if v is None:
                continue
            if not hasattr(cfg, k):
                raise KeyError(k)
            setattr(cfg, k, v)
        self.check(self.L.rapt_config_set(self.h, C.byref(cfg)), "rapt_config_set")
        return cfg

    def field_eval(self, quantity, tpos):
        tpos = np.ascontiguousarray(np.atleast_2d(tpos), dtype=np.float64)
        n = tpos.shape[0]
        out = np.zeros((n, 9))
        self.check(self.L.rapt_field_eval(self.h, FIELD_QUANTITIES[quantity], n, ptr(tpos), ptr(out)),
                   "rapt_field_eval")
        return out

    def rhs_eval(self, mode, state, mass, charge, v=None):
        state = np.ascontiguousarray(state, dtype=np.float64)
        n = state.shape[0]
        mass = np.ascontiguousarray(np.broadcast_to(mass, (n,)), dtype=np.float64)
        charge = np.ascontiguousarray(np.broadcast_to(charge, (n,)), dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(np.broadcast_to(v, (n,)), dtype=np.float64)
        out = np.zeros((n, 6))
        self.check(self.L.rapt_rhs_eval(self.h, int(mode), n, ptr(state), ptr(mass), ptr(charge), ptr(vv), ptr(out)),
                   "rapt_rhs_eval")
        return out

    def gc_bounce_period(self, state):
        """Bounce periods of GC states [n][7] = (t, x, y, z, ppar, mu, mass)."""
        st = np.ascontiguousarray(np.atleast_2d(state), dtype=np.float64)
        out = np.zeros(st.shape[0])
        self.check(self.L.rapt_gc_bounce_period(self.h, st.shape[0], ptr(st), ptr(out)), "rapt_gc_bounce_period")
        return out

    # ---- step-size MLP
    def mlp_set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self.check(self.L.rapt_mlp_set_params(self.h, ptr(p), p.size), "rapt_mlp_set_params")

    def mlp_get_params(self):
        p = np.zeros(MLP_NPARAMS, np.float32)
        self.check(self.L.rapt_mlp_get_params(self.h, ptr(p), p.size), "rapt_mlp_get_params")
        return p

    def mlp_forward(self, features):
        f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 16)
        out = np.zeros((f.shape[0], 2), np.float32)
        self.check(self.L.rapt_mlp_forward(self.h, ptr(f), f.shape[0], ptr(out)), "rapt_mlp_forward")
        return out

    def mlp_grad(self, samples, switch_weight=1.0):
        s = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1, MLP_SAMPLE)
        g = np.zeros(MLP_NTRAIN, np.float32)
        loss = (C.c_double * 2)()
        self.check(self.L.rapt_mlp_grad(self.h, ptr(s), s.shape[0], float(switch_weight), ptr(g),
                                        C.cast(loss, _DP)), "rapt_mlp_grad")
        return g, (loss[0], loss[1])

    def mlp_samples_reserve(self, capacity, mask=0):
        self.check(self.L.rapt_mlp_samples_reserve(self.h, int(capacity), int(mask)), "rapt_mlp_samples_reserve")

    def mlp_samples_count(self):
        k = C.c_int64()
        self.check(self.L.rapt_mlp_samples_count(self.h, C.byref(k)), "rapt_mlp_samples_count")
        return k.value

    def mlp_samples_download(self, first=0, n=None):
        if n is None:
            n = self.mlp_samples_count() - first
        out = np.zeros((n, MLP_SAMPLE), np.float32)
        self.check(self.L.rapt_mlp_samples_download(self.h, ptr(out), int(first), int(n)),
                   "rapt_mlp_samples_download")
        return out

    def mlp_samples_upload(self, samples):
        s = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1, MLP_SAMPLE)
        self.check(self.L.rapt_mlp_samples_upload(self.h, ptr(s), s.shape[0]), "rapt_mlp_samples_upload")

    def mlp_samples_sort(self, first=0, n=None):
        """Canonical order of samples [first, first + n) (rapt_mlp_samples_sort)."""
        if n is None:
            n = self.mlp_samples_count() - first
        self.check(self.L.rapt_mlp_samples_sort(self.h, int(first), int(n)), "rapt_mlp_samples_sort")

    def mlp_train(self, steps, batch=4096, lr=1e-3, switch_weight=1.0, seed=0):
        loss = (C.c_double * 2)()
        self.check(self.L.rapt_mlp_train(self.h, int(steps), int(batch), float(lr), float(switch_weight), int(seed),
                                         C.cast(loss, _DP)), "rapt_mlp_train")
        return loss[0], loss[1]

    def measure_peaks(self):
        a, b = C.c_double(), C.c_double()
        self.check(self.L.rapt_measure_peaks(self.h, C.byref(a), C.byref(b)), "rapt_measure_peaks")
        return a.value, b.value


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("RAPT_DEVICE", "0")))
    return _default_ctx
