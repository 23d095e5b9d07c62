"""Autotuner of the persistent tracer kernels' launch shape.

The kernels run one persistent grid per mode in which every thread takes
tracers from a work queue in turn, so the launch shape decides how many tracers
each thread handles (threads per block x blocks per SM against the ensemble
size), how full the SMs are, and how much per-round host work remains (graph
replay of the rounds or one launch sequence per round). ``tune`` times the
candidate shapes on a sample of the caller's workload -- the arithmetic of every
tracer is the same under every shape, so device time alone decides -- and
caches the winner per (field model, run kind, form, tableau) in a JSON file.
"""
import json
import os

import numpy as np

CACHE = os.path.join(os.environ.get("XDG_CACHE_HOME", os.path.join(os.path.expanduser("~"), ".cache")),
                     "rapt_gb300", "autotune.json")
BLOCKS = (32, 64, 128)
BLOCKS_PER_SM = (1, 2, 4, 8, 16)


def cache_key(model, kind, form, tableau):
    return "model%d/%s/form%d/tab%d" % (int(model), kind, int(form), int(tableau))


def load_cache(path=CACHE):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(table, path=CACHE):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(blocks=BLOCKS, blocks_per_sm=BLOCKS_PER_SM, graph=(0, 1)):
    return [dict(threads_per_block=b, blocks_per_sm=m, use_graph=g) for b in blocks for m in blocks_per_sm
            for g in graph]


def tune(ens, kind, delta, cands=None, key=None, path=CACHE, use_cache=True):
    """Pick the fastest launch shape for advancing `ens` (an uploaded Ensemble
    holding a sample of the workload) by `delta`. The ensemble's host copy of
    the start state is restored (and, for Adaptive, its mode picked again)
    before each candidate. Returns (best shape,
    table of device ms per candidate); with a key, the best shape is cached."""
    if key is not None and use_cache:
        hit = load_cache(path).get(key)
        if hit:
            return hit["best"], hit["table"]
    cands = cands or candidates()
    init = {k: v.copy() for k, v in ens.h.items()}
    base = dict(ens.config)
    table = []

    def restore():
        for k, v in init.items():
            ens.h[k][...] = v
        ens.upload()
        if kind == "adaptive":
            ens.adaptive_init()

    for c in cands:
        restore()
        cfg = dict(base)
        cfg.update(c)
        ens.configure(**cfg)
        st = ens.advance(kind, delta)
        table.append(dict(c, ms=st["kernel_ms"], launches=st["kernel_launches"]))
    best = min(table, key=lambda r: r["ms"])
    best = {k: best[k] for k in ("threads_per_block", "blocks_per_sm", "use_graph")}
    restore()
    ens.configure(**base)
    if key is not None:
        t = load_cache(path)
        t[key] = {"best": best, "table": table}
        save_cache(t, path)
    return best, table


def sample(w, n):
    """An evenly spaced sample of n tracers of a workload dict."""
    from .workloads import subsample
    m = len(w["mass"])
    return subsample(w, np.linspace(0, m - 1, min(n, m)).astype(np.int64))
