"""CPU checks of the C ABI boundary: the library loads without a GPU, exports
every function include/rapt_gpu.h declares, and its ctypes layouts match the
header's structs. No compute call is made."""
import ctypes as C
import os
import re

import pytest

from rapt_gb300 import _native as N

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rapt_gpu.h")


def _declared():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rapt_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = _declared()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), name
    assert set(names) == set(N.SIGNATURES), set(names) ^ set(N.SIGNATURES)


def test_abi_version_and_defaults():
    L = N.lib()
    assert L.rapt_abi_version() == 1
    cfg = N.RaptConfig()
    L.rapt_config_default(C.byref(cfg))
    assert cfg.rtol == cfg.atol == 1.49012e-8   # rapt/__init__.py:27
    assert cfg.cyclotronresolution == 10 and cfg.nsteps == 500 and cfg.epss == cfg.epst == 0.05


def test_struct_layouts_match_header():
    # field order and sizes of rapt_config / rapt_host_state / rapt_stats / rapt_gc_device_state
    # ... collect, pad, learned_scale, learned_every, per_tracer_launches, bounce/fieldline res,
    # dense_output + tail padding
    assert C.sizeof(N.RaptConfig) == 8 * 6 + 4 * 4 + 8 * 2 + 4 * 2 + 8 + 4 * 2 + 4 + 4 + 8 + 4 + 4 + 8 + 8 + 8
    assert C.sizeof(N.RaptHostState) == 8 * 21
    assert C.sizeof(N.RaptStats) == 8 * 9
    assert C.sizeof(N.RaptGcDeviceState) == 8 * 18


def test_no_gpu_fails_loudly_without_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(N.RaptError):
        N.Context(0)


def test_noalloc_refuses_before_touching_the_device():
    """The allocation-free entry point validates its configuration before any
    CUDA call: the default configuration's bounce-period cadence, the FP32 and
    learned forms, dense output, sample collection and bad tolerances are refused
    with an error code (no GPU is needed to see that)."""
    L = N.lib()
    st = N.RaptGcDeviceState()
    st.n = 16
    st.max_rows = 4

    def call(**over):
        cfg = N.RaptConfig()
        L.rapt_config_default(C.byref(cfg))
        cfg.gctimestep = 1.0
        for k, v in over.items():
            setattr(cfg, k, v)
        return L.rapt_gc_advance_noalloc(0, 1, None, 0, C.byref(cfg), C.byref(st), 1.0, None, None)

    assert call(gctimestep=0.0) == N.RAPT_ERR_UNSUPPORTED
    for form in (1, 2, 3):
        assert call(form=form) == N.RAPT_ERR_UNSUPPORTED
    assert call(dense_output=1) == N.RAPT_ERR_UNSUPPORTED
    assert call(collect=1) == N.RAPT_ERR_UNSUPPORTED
    assert call(rtol=-1.0) == N.RAPT_ERR_INVALID
    assert call(gctimestep=-1.0) == N.RAPT_ERR_INVALID
    st.n = N.NOALLOC_MAX_TRACERS + 1
    assert call() == N.RAPT_ERR_INVALID


def test_object_api_raises_like_the_reference_on_stepper_failures():
    """A tracer that stopped because the RKF45 step fell below hmin raises
    RuntimeError (rkf.py:136-139); one that left a Grid raises ValueError."""
    from rapt_gb300 import tracers as T
    with pytest.raises(RuntimeError):
        T._raise_if_left_grid({"status": [N.ST["RKF_HMIN"]]})
    with pytest.raises(ValueError):
        T._raise_if_left_grid({"status": [N.ST["OUT_OF_GRID"]]})
    T._raise_if_left_grid({"status": [0]})
