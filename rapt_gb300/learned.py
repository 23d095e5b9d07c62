"""Host side of the learned forms: collect step-size samples from the plain
controller on the GPU, fit the feature normalisation, train the MLP with the
device kernels, and load it into a context.

The network (16 -> 64 -> 64 -> 2, BF16 weights, FP32 accumulation; layout in
include/rapt_gpu.h, RAPT_MLP_*) proposes a multiplicative correction of the
DOPRI5 controller's next step for guiding centres (the controller of
GuidingCenter.advance, rapt/GuidingCenter.py:450, SciPy dopri5). Its training
target for an accepted step n is log(h*_{n+1} / hnew_n), where hnew_n is the
plain controller's proposal and h*_{n+1} = h_{n+1} (1 / err_{n+1})^(1/5) the
step that would have put the error estimate of the attempt that followed
exactly at the acceptance threshold. A proposal is the network's output minus
a margin c calibrated on samples (``calibrate``): the c that maximises the
expected advance per attempt, E[(h / h*) 1(h <= h*)]. The error estimate
still judges every step; a rejected proposal falls back to the plain
controller. Steps that end an output interval give no sample; the learned form
starts the next interval with the step the controller wanted before the
interval-end clip instead of HINIT.

Features (computed on the device after each accepted step):
  0 log(|h| v / r)        1 log10 err_n           2 log10 err_{n-1}
  3 log(hnew / h)         4 mode (1: GC)          5 sign of the charge
  6 log10(m / m_e)        7 log10(gamma - 1)      8 cos(pitch) = ppar / (gamma m v)
  9 log(r / Re)          10 z / r                11 position in the output interval
 12 output interval / |h|                        13 step followed a rejection

Switch head: in Adaptive runs the guiding-centre kernels also record, at every
output row that gets an adiabaticity check, the features of the step that
ended the interval with label 1 if the check fails (the tracer switches to
particle mode) and no step target; the head is trained with a masked binary
cross-entropy and reported (``switch_metrics``). The kernels keep the exact
check at every row, so switching follows the reference either way.
"""
import numpy as np

from . import _native
from .ensemble import Ensemble

NFEAT = 14


def init_params(seed=0):
    """He-uniform weights, zero biases, identity normalisation."""
    rng = np.random.default_rng(seed)
    p = np.zeros(_native.MLP_NPARAMS, np.float32)
    o = 0

    def put(a):
        nonlocal o
        a = np.asarray(a, np.float32).ravel()
        p[o:o + a.size] = a
        o += a.size

    w1 = rng.uniform(-1, 1, (64, 16)) * np.sqrt(6.0 / NFEAT)
    w1[:, NFEAT:] = 0
    put(w1)
    put(np.zeros(64))
    put(rng.uniform(-1, 1, (64, 64)) * np.sqrt(6.0 / 64))
    put(np.zeros(64))
    w3 = np.zeros((8, 64))
    w3[:2] = rng.uniform(-1, 1, (2, 64)) * np.sqrt(3.0 / 64)
    put(w3)
    put(np.zeros(8))
    assert o == _native.MLP_NTRAIN
    put(np.zeros(16))   # xmu
    put(np.ones(16))    # xsig
    put(np.zeros(8))    # ymu
    put(np.ones(8))     # ysig
    return p


def set_normalisation(params, samples):
    """Feature mean / scale and step-target mean / scale from host samples [n][18]."""
    p = np.array(params, np.float32)
    s = np.asarray(samples, np.float64)
    n0 = _native.MLP_NTRAIN
    mu = np.zeros(16)
    sig = np.ones(16)
    mu[:NFEAT] = s[:, :NFEAT].mean(0)
    sd = s[:, :NFEAT].std(0)
    sig[:NFEAT] = np.where(sd > 1e-6, sd, 1.0)
    p[n0:n0 + 16] = mu
    p[n0 + 16:n0 + 32] = sig
    ymu = np.zeros(8)
    ysig = np.ones(8)
    t = s[:, 16][np.isfinite(s[:, 16])]  # switch-labelled samples have no step target
    if t.size:
        ymu[0] = t.mean()
        ysig[0] = max(t.std(), 1e-6)
    p[n0 + 32:n0 + 40] = ymu
    p[n0 + 40:n0 + 48] = ysig
    return p


def collect_gc(workload, seconds, capacity=1 << 21, mask=0, ctx=None, form=0):
    """Run guiding centres of `workload` for `seconds` with the plain controller
    and sample collection on; returns (ensemble, stats, sample count). The
    samples stay in the context's device buffer."""
    ctx = ctx or _native.default_context()
    ctx.mlp_samples_reserve(capacity, mask)
    rows = int(np.ceil(seconds / workload["params"]["gctimestep"])) + 4
    ens = Ensemble.from_workload(workload, "gc", max_rows=rows, ctx=ctx, form=form)
    ens.configure(collect=1)
    st = ens.advance("gc", float(seconds))
    ens.configure(collect=0)
    ctx.mlp_samples_sort()
    return ens, st, ctx.mlp_samples_count()


def train(ctx, steps=4000, batch=4096, lr=2e-3, seed=0, params=None, norm_sample=1 << 16, decay=True):
    """Train on the context's device samples with Adam steps on the device.
    Without `params`: fresh weights, normalisation from a host copy of the first
    `norm_sample` samples; with `params`: continue from them (normalisation
    kept). With decay, the last third of the steps run at lr / 10. Returns
    (params, losses)."""
    n = ctx.mlp_samples_count()
    if n == 0:
        raise RuntimeError("no training samples in the context")
    if params is None:
        host = ctx.mlp_samples_download(0, min(n, norm_sample))
        p = set_normalisation(init_params(seed), host)
    else:
        p = np.asarray(params, np.float32)
    ctx.mlp_set_params(p)
    losses = []
    if decay:
        s1 = (2 * steps) // 3
        losses.append(ctx.mlp_train(s1, batch, lr, 1.0, seed))
        losses.append(ctx.mlp_train(steps - s1, batch, lr / 10, 1.0, seed + 1))
    else:
        losses.append(ctx.mlp_train(steps, batch, lr, 1.0, seed))
    return ctx.mlp_get_params(), losses


def fit_gc(workload, seconds, ctx=None, rounds=2, steps=3000, batch=4096, lr=2e-3, capacity=1 << 22, mask=0,
           seed=0):
    """Train the step MLP for guiding centres of `workload`: samples from the
    plain controller, then `rounds` of on-policy samples from the learned
    controller itself (the proposals change the states and errors it sees),
    retraining on everything collected each time. Returns (params, info)."""
    ctx = ctx or _native.default_context()
    ctx.mlp_samples_reserve(capacity, mask)
    rows = int(np.ceil(seconds / workload["params"]["gctimestep"])) + 4
    info = {"collect": [], "losses": [], "calibration": []}

    def run(form, scale):
        n0 = ctx.mlp_samples_count()
        ens = Ensemble.from_workload(workload, "gc", max_rows=rows, ctx=ctx, form=form, collect=1,
                                     learned_scale=scale)
        st = ens.advance("gc", float(seconds))
        n1 = ctx.mlp_samples_count()
        ctx.mlp_samples_sort(n0, n1 - n0)  # canonical order: training is then reproducible
        info["collect"].append({"form": form, "accepted": st["accepted"], "rejected": st["rejected"],
                                "samples": n1 - n0})
        return n0, n1

    n0, n1 = run(0, 1.0)
    p, losses = train(ctx, steps, batch, lr, seed)
    info["losses"].append(losses)
    cal = calibrate(ctx, ctx.mlp_samples_download(n0, min(n1 - n0, 1 << 16)))
    info["calibration"].append(cal)
    for r in range(rounds):
        n0, n1 = run(2, cal["scale"])
        if n1 == n0:
            raise RuntimeError("sample buffer full: raise capacity or mask")
        p, losses = train(ctx, steps, batch, lr, seed + 10 * (r + 1), params=p)
        info["losses"].append(losses)
        cal = calibrate(ctx, ctx.mlp_samples_download(n0, min(n1 - n0, 1 << 16)))
        info["calibration"].append(cal)
    info["scale"] = cal["scale"]
    return p, info


def calibrate_global(workload, seconds, ctx=None, scales=(1.0, 0.95, 0.9, 0.85, 0.8, 0.75, 0.7, 0.65, 0.6),
                     form=3, every=1, quantile=0.99, slack=1.05):
    """Proposal scale calibrated on the global error, with the network loaded in
    ctx: guiding centres of `workload` are advanced `seconds` by the plain FP64
    controller, by a tight-tolerance run (rtol = atol = 1e-12, the exact
    solution) and by the learned form at each candidate scale, largest first.
    The chosen scale is the largest whose final-position error against the
    exact solution is no worse than the plain controller's, both at the given
    quantile and at the maximum over the tracers, up to `slack` (the sampling
    noise of a maximum over a few thousand tracers). Returns (scale, table);
    the scale is None if no candidate qualifies."""
    ctx = ctx or _native.default_context()
    rows = int(np.ceil(seconds / workload["params"]["gctimestep"])) + 4

    def final(**over):
        ens = Ensemble.from_workload(workload, "gc", max_rows=rows, ctx=ctx, **over)
        st = ens.advance("gc", float(seconds))
        h = ens.download()
        if np.any(h["status"] != 0):
            raise RuntimeError("calibration run stopped early: %s" % np.unique(h["status"]))
        return h["s"][:3].T.copy(), st

    exact, _ = final(rtol=1e-12, atol=1e-12, nsteps=1000000)
    norm = np.linalg.norm(exact, axis=1)

    def err_of(pos):
        e = np.linalg.norm(pos - exact, axis=1) / norm
        return {"median": float(np.median(e)), "q": float(np.quantile(e, quantile)), "max": float(e.max())}

    pos, st = final(form=0)
    plain = err_of(pos)
    table = [{"scale": None, "form": 0, "rhs": int(st["rhs_evals"]), **plain}]
    chosen = None
    for sc in sorted(scales, reverse=True):
        pos, st = final(form=form, learned_scale=float(sc), learned_every=int(every))
        e = err_of(pos)
        table.append({"scale": float(sc), "form": form, "rhs": int(st["rhs_evals"]), **e})
        if e["q"] <= slack * plain["q"] and e["max"] <= slack * plain["max"]:
            chosen = float(sc)
            break
    return chosen, table


def calibrate(ctx, samples, margins=np.linspace(0.0, 1.0, 201)):
    """Margin of the learned proposals from samples [n][18] with the network
    loaded in ctx. Efficiency = mean advance per attempt relative to the ideal
    step, (h / h*) 1(h <= h*), for the learned proposal exp(pred - c) hnew and
    for the plain controller's hnew. Returns a dict with the margin, the
    proposal scale exp(-c) for rapt_config.learned_scale and both efficiencies."""
    s = np.asarray(samples, np.float32)
    s = s[np.isfinite(s[:, 16])]
    pred = ctx.mlp_forward(s[:, :16])[:, 0].astype(np.float64)
    y = s[:, 16].astype(np.float64)
    eff = np.array([np.mean(np.exp(pred - c - y) * (pred - c <= y)) for c in margins])
    k = int(np.argmax(eff))
    c = float(margins[k])
    plain = float(np.mean(np.exp(-y) * (y >= 0)))
    return {"margin": c, "scale": float(np.exp(-c)), "eff_learned": float(eff[k]), "eff_plain": plain,
            "accept_learned": float(np.mean(pred - c <= y)), "accept_plain": float(np.mean(y >= 0)),
            "resid_std": float(np.std(pred - y)), "target_std": float(np.std(y))}


def switch_metrics(ctx, samples, threshold=0.5):
    """Switch head on switch-labelled samples [n][18] (label >= 0) with the
    network loaded in ctx: accuracy, recall and precision of the prediction
    sigmoid(logit) > threshold, against the base rate of switches."""
    s = np.asarray(samples, np.float32)
    s = s[s[:, 17] >= 0]
    if len(s) == 0:
        return {"n": 0}
    p = 1.0 / (1.0 + np.exp(-ctx.mlp_forward(s[:, :16])[:, 1].astype(np.float64)))
    y = s[:, 17] > 0.5
    pr = p > threshold
    tp = int(np.sum(pr & y))
    return {"n": int(len(s)), "base_rate": float(y.mean()), "accuracy": float(np.mean(pr == y)),
            "recall": tp / max(int(y.sum()), 1), "precision": tp / max(int(pr.sum()), 1)}


def save(path, params):
    np.save(path, np.asarray(params, np.float32))


def load(path, ctx=None):
    p = np.load(path).astype(np.float32)
    if ctx is not None:
        ctx.mlp_set_params(p)
    return p
