"""Host logic of the launch-shape autotuner (rapt_gb300.autotune): it times
every candidate from the same start state, picks the fastest, restores the
ensemble, and caches the winner per key -- exercised with a stand-in ensemble
whose device time depends on the launch shape (no GPU)."""
import numpy as np

from rapt_gb300 import autotune as A


class FakeEnsemble:
    """Duck-typed Ensemble: host state, configuration and an advance() whose
    'device time' is smallest at 64 threads x 4 blocks/SM with graph replay."""

    def __init__(self):
        self.h = {"s": np.arange(12.0).reshape(6, 2), "status": np.zeros(2, np.int32)}
        self.config = {"rtol": 1e-8, "threads_per_block": 0, "blocks_per_sm": 0, "use_graph": 0}
        self.uploads = self.inits = self.advances = 0
        self.starts = []

    def upload(self):
        self.uploads += 1

    def adaptive_init(self):
        self.inits += 1

    def configure(self, **kw):
        self.config.update(kw)

    def advance(self, kind, delta):
        self.advances += 1
        self.starts.append(self.h["s"].copy())
        self.h["s"] += delta  # the advance changes the host copy; tune must restore it
        c = self.config
        ms = abs(c["threads_per_block"] - 64) + abs(c["blocks_per_sm"] - 4) + (0 if c["use_graph"] else 0.5) + 1.0
        return {"kernel_ms": ms, "kernel_launches": 3}


def test_tune_picks_the_fastest_shape_from_the_same_start(tmp_path):
    ens = FakeEnsemble()
    s0 = ens.h["s"].copy()
    path = str(tmp_path / "autotune.json")
    best, table = A.tune(ens, "adaptive", 2.0, key="k", path=path)
    assert best == {"threads_per_block": 64, "blocks_per_sm": 4, "use_graph": 1}
    assert len(table) == len(A.candidates()) == ens.advances
    assert all(np.array_equal(s, s0) for s in ens.starts)  # every candidate from the start state
    assert np.array_equal(ens.h["s"], s0)                  # and the ensemble left at it
    assert ens.inits == len(table) + 1                     # Adaptive: mode picked again each time
    assert ens.config["rtol"] == 1e-8 and ens.config["threads_per_block"] == 0  # configuration restored
    # cached: a second call returns the stored result without timing anything
    ens2 = FakeEnsemble()
    best2, table2 = A.tune(ens2, "adaptive", 2.0, key="k", path=path)
    assert best2 == best and table2 == table and ens2.advances == 0
    assert A.load_cache(path)["k"]["best"] == best


def test_cache_survives_a_missing_or_corrupt_file(tmp_path):
    path = tmp_path / "autotune.json"
    assert A.load_cache(str(path)) == {}
    path.write_text("{not json")
    assert A.load_cache(str(path)) == {}
    A.save_cache({"a": {"best": {}, "table": []}}, str(tmp_path / "sub" / "t.json"))
    assert A.load_cache(str(tmp_path / "sub" / "t.json"))["a"]["table"] == []


def test_cache_key_and_candidates():
    assert A.cache_key(1, "gc", 3, 0) == "model1/gc/form3/tab0"
    c = A.candidates(blocks=(32,), blocks_per_sm=(1, 2), graph=(0,))
    assert c == [dict(threads_per_block=32, blocks_per_sm=1, use_graph=0),
                 dict(threads_per_block=32, blocks_per_sm=2, use_graph=0)]
