"""Batching: graph replay of the launch rounds, the per-tracer launch pattern
and the autotuner give the same tracer results as the default persistent grid
(the arithmetic of a tracer does not depend on the launch shape)."""
import numpy as np
import pytest

from rapt_gb300 import autotune as A
from rapt_gb300 import workloads as W
from tests._util import gpu_ensemble

pytestmark = pytest.mark.gpu

KEYS = ("s", "t_row", "tcur", "naccept", "nreject", "nfcn", "status", "mode", "nswitch")


def _run(w, kind, delta, max_rows, **cfg):
    e = gpu_ensemble(w, kind, max_rows=max_rows, max_switch=64, **cfg)
    st = e.advance(kind, delta)
    return st, e.download(), e


def _same(ha, hb):
    for k in KEYS:
        assert np.array_equal(ha[k], hb[k]), k


def test_graph_replay_matches_rounds_adaptive():
    w = W.subsample(W.config3(), np.arange(0, 262144, 512))  # 512 protons
    d = w["delta"] / 5
    sa, ha, _ = _run(w, "adaptive", d, 1024)
    sb, hb, _ = _run(w, "adaptive", d, 1024, use_graph=1)
    _same(ha, hb)
    assert sa["accepted"] == sb["accepted"] and sa["switches"] == sb["switches"] > 0
    assert sb["launches"] % 4 == 0 and sb["launches"] >= sa["launches"]


def test_graph_replay_matches_rounds_gc_learned_shapes():
    w = W.subsample(W.config2(), np.arange(0, 65536, 64))
    sa, ha, _ = _run(w, "gc", 3.0, 8)
    sb, hb, _ = _run(w, "gc", 3.0, 8, use_graph=1, threads_per_block=64, blocks_per_sm=2)
    _same(ha, hb)


def test_per_tracer_launches_match_batched():
    w = W.subsample(W.config3(), np.arange(0, 262144, 4096))  # 64 protons
    d = w["delta"] / 10
    sa, ha, _ = _run(w, "adaptive", d, 1024)
    sb, hb, _ = _run(w, "adaptive", d, 1024, per_tracer_launches=1)
    _same(ha, hb)
    assert sb["kernel_launches"] >= 2 * len(w["mass"])


def test_autotune_picks_and_caches(tmp_path):
    w = W.subsample(W.config2(), np.arange(0, 65536, 16))
    e = gpu_ensemble(w, "gc", max_rows=8)
    cands = A.candidates(blocks=(64, 128), blocks_per_sm=(1, 2), graph=(0, 1))
    path = str(tmp_path / "tune.json")
    best, table = A.tune(e, "gc", 2.0, cands=cands, key="k", path=path)
    assert len(table) == 8 and best in [{k: r[k] for k in best} for r in table]
    assert all(r["ms"] > 0 for r in table)
    best2, _ = A.tune(e, "gc", 2.0, cands=cands, key="k", path=path)
    assert best2 == best
    # the ensemble is left at its start state and configuration
    st = e.advance("gc", 2.0)
    e2 = gpu_ensemble(w, "gc", max_rows=8)
    st2 = e2.advance("gc", 2.0)
    assert st["accepted"] == st2["accepted"]
