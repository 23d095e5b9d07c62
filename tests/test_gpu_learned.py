"""The learned form: the MLP's device forward and backward kernels against the
CPU oracle, device training, sample collection that leaves the plain path
unchanged, and an A/B comparison of the trained step proposals against the
plain DOPRI5 controller on held-out guiding centres."""
import numpy as np
import pytest

from rapt_gb300 import learned
from rapt_gb300 import workloads as W
from tests._util import gpu_ensemble, rel_state_error
from tests.test_mlp_oracle import _problem

pytestmark = pytest.mark.gpu

PLAIN, FP32, LEARNED, LEARNED_FP32 = 0, 1, 2, 3


def mo():
    from oracle import mlp_oracle
    return mlp_oracle


def test_forward_matches_oracle(ctx):
    p, s = _problem(5, n=1000)  # ragged: 1000 is not a multiple of 32
    ctx.mlp_set_params(p)
    got = ctx.mlp_forward(s[:, :16])
    ref, _ = mo().forward(p, s[:, :16])
    err = np.abs(got - ref) / (1 + np.abs(ref))
    # same BF16 rounding points; only FP32 accumulation order differs, which can
    # flip a BF16 rounding of a hidden activation
    assert np.median(err) < 1e-4 and err.max() < 2e-2, (np.median(err), err.max())
    assert np.array_equal(ctx.mlp_get_params(), p)


def test_gradient_matches_oracle(ctx):
    p, s = _problem(6, n=4000)
    ctx.mlp_set_params(p)
    g, (l0, l1) = ctx.mlp_grad(s, switch_weight=0.7)
    (r0, r1), gr = mo().loss_and_grad(p, s, switch_weight=0.7)
    assert abs(l0 - r0) < 1e-3 * r0 and abs(l1 - r1) < 1e-3 * r1, (l0, r0, l1, r1)
    rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
    assert rel < 1e-2, rel
    # every parameter block separately
    for a, b in [(0, 1024), (1024, 1088), (1088, 5184), (5184, 5248), (5248, 5376), (5760, 5762)]:
        rb = np.linalg.norm(g[a:b] - gr[a:b]) / np.linalg.norm(gr[a:b])
        assert rb < 2e-2, (a, b, rb)
    assert np.all(g[5376:5760] == 0) and np.all(g[5762:] == 0)


def test_device_training_fits_a_smooth_target(ctx):
    rng = np.random.default_rng(7)
    n = 1 << 16
    f = rng.normal(size=(n, 16)).astype(np.float32)
    f[:, 14:] = 0
    t = np.sin(f[:, 0]) + 0.5 * f[:, 3] * f[:, 5]
    lab = (f[:, 1] + f[:, 2] > 0).astype(np.float32)
    ctx.mlp_samples_upload(np.column_stack([f, t, lab]).astype(np.float32))
    p, losses = learned.train(ctx, steps=1500, batch=2048, lr=3e-3, seed=1)
    # normalised step loss: 0.5 for the mean predictor
    assert losses[-1][0] < 0.02, losses
    out = ctx.mlp_forward(f[:4096])
    assert np.sqrt(np.mean((out[:, 0] - t[:4096]) ** 2)) < 0.15 * np.std(t)
    acc = np.mean((out[:, 1] > 0) == (lab[:4096] > 0.5))
    assert acc > 0.97, acc


def test_collection_leaves_plain_results_unchanged(ctx):
    w = W.subsample(W.config2(), np.arange(0, 65536, 256))
    a = gpu_ensemble(w, "gc", max_rows=8)
    a.advance("gc", 5.0)
    ha = a.download()
    ctx.mlp_samples_reserve(1 << 18, 0)
    b = gpu_ensemble(w, "gc", max_rows=8, collect=1)
    b.advance("gc", 5.0)
    hb = b.download()
    for k in ("naccept", "nreject", "nfcn", "status"):
        assert np.array_equal(ha[k], hb[k]), k
    assert np.array_equal(ha["s"], hb["s"])
    n = ctx.mlp_samples_count()
    # one sample per accepted step except interval ends and steps followed by a clipped step
    assert 0.9 * ha["naccept"].sum() < n <= ha["naccept"].sum()
    s = ctx.mlp_samples_download(0, n)
    assert np.all(np.isfinite(s)) and np.all(s[:, 17] == -1) and np.all(s[:, 4] == 1)
    # the target is log(h*/hnew): mostly near the 0.6 error target, never wild
    assert np.abs(np.median(s[:, 16])) < 0.5 and np.all(np.abs(s[:, 16]) < 30)


def test_training_is_deterministic(ctx):
    """Sample collection (appended in an order set by device atomics), the
    canonical sort and device training repeated from scratch give the same
    samples and bit-identical parameters; the gradient is reduced without
    floating-point atomics."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 128))

    def once():
        ctx.mlp_samples_reserve(1 << 20, 1)
        b = gpu_ensemble(w, "gc", max_rows=8, collect=1)
        b.advance("gc", 3.0)
        ctx.mlp_samples_sort()
        s = ctx.mlp_samples_download()
        p, losses = learned.train(ctx, steps=300, batch=2048, lr=2e-3, seed=4)
        g, l = ctx.mlp_grad(s[:5000], switch_weight=1.0)
        return s, p, losses, g, l

    s1, p1, l1, g1, ll1 = once()
    s2, p2, l2, g2, ll2 = once()
    assert len(s1) > 10000 and np.array_equal(s1, s2)
    assert np.array_equal(p1, p2) and l1 == l2
    assert np.array_equal(g1, g2) and ll1 == ll2


def _train_on_config2(ctx, seconds=10.0):
    """Plain then on-policy samples from the even-indexed tracers of a config-2
    subsample (2048 electrons, 10 s each round)."""
    w = W.subsample(W.config2(), np.arange(0, 65536, 16))
    tr = W.subsample(w, np.arange(0, len(w["mass"]), 2))
    p, info = learned.fit_gc(tr, seconds, ctx=ctx, rounds=3, steps=3000, capacity=1 << 23, mask=1)
    assert info["collect"][0]["accepted"] > 2e6 and info["collect"][0]["samples"] > 1e6
    return w, p, info


@pytest.fixture(scope="module")
def trained(ctx):
    return _train_on_config2(ctx)


def test_learned_ab_against_plain(ctx, trained, oracle):
    """Held-out (odd-indexed) tracers, 10 s: what the trained network gains over
    the plain DOPRI5 controller, and at what price.

    At the proposal scale calibrated on samples (the largest expected advance
    per attempt) the network's proposals are far better predictions of the
    largest acceptable step than the controller's (residual spread of log h*
    a fraction of the controller's), so the learned form needs fewer
    right-hand sides and rejects fewer steps -- but its steps sit nearer the
    acceptance threshold and its global error (against a tight-tolerance run)
    is larger than the plain controller's. At the scale calibrated on the
    global error (learned.calibrate_global) the error is the plain
    controller's or smaller, and the right-hand sides are not fewer: on these
    orbits the trained proposals buy no work at matched accuracy."""
    w, p, info = trained
    print("fit", info)
    cal = info["calibration"][-1]
    assert info["losses"][0][-1][0] < 0.45, info  # below the mean predictor's 0.5
    # on samples, the calibrated proposals advance further per attempt than the
    # controller, and predict the largest acceptable step more tightly
    assert cal["eff_learned"] > cal["eff_plain"] and cal["resid_std"] < 0.5 * cal["target_std"], cal
    te = W.subsample(w, np.arange(1, len(w["mass"]), 2))
    ctx.mlp_set_params(p)
    scale_g, table = learned.calibrate_global(W.subsample(w, np.arange(0, len(w["mass"]), 2)), 10.0, ctx=ctx)
    assert scale_g is not None, table
    runs = {"plain": (PLAIN, 1.0), "learned": (LEARNED, cal["scale"]), "learned_fp32": (LEARNED_FP32, cal["scale"]),
            "matched": (LEARNED_FP32, scale_g)}
    res = {}
    for name, (form, scale) in runs.items():
        e = gpu_ensemble(te, "gc", max_rows=16, form=form, learned_scale=scale)
        st = e.advance("gc", 10.0)
        h = e.download()
        bad = np.nonzero(h["status"])[0]
        assert bad.size == 0, (name, st, np.unique(h["status"], return_counts=True), bad[:8])
        res[name] = (st, h)
    # a tight-tolerance run as the exact solution: the global error of each form
    e = gpu_ensemble(te, "gc", max_rows=16, rtol=1e-12, atol=1e-12, nsteps=1000000)
    e.advance("gc", 10.0)
    he = e.download()
    assert np.all(he["status"] == 0)
    exact = he["s"]
    report = {}
    for name, (st, h) in res.items():
        gpos, _ = rel_state_error(h["s"], exact.T, 4)
        report[name] = dict(rhs=st["rhs_evals"], rej_rate=st["rejected"] / max(st["accepted"], 1),
                            glob_med=float(np.median(gpos)), glob_p99=float(np.percentile(gpos, 99)),
                            glob_max=float(gpos.max()))
    report["scale_samples"], report["scale_global"] = cal["scale"], scale_g
    print("A/B", report)
    pl, le, lf, mt = report["plain"], report["learned"], report["learned_fp32"], report["matched"]
    # the gain at the sample-calibrated scale: fewer right-hand sides and rejections
    assert le["rhs"] < 0.95 * pl["rhs"] and le["rej_rate"] < pl["rej_rate"], report
    assert abs(lf["rhs"] - le["rhs"]) < 0.01 * le["rhs"], report
    # ... bought with accuracy: a larger global error than the plain controller's
    assert le["glob_med"] > pl["glob_med"], report
    # at the globally calibrated scale: the plain controller's accuracy (up to
    # the calibration sample's noise), and no saving of right-hand sides
    assert mt["glob_p99"] <= 1.25 * pl["glob_p99"] and mt["glob_max"] <= 1.25 * pl["glob_max"], report
    assert mt["rhs"] > 0.95 * pl["rhs"], report


BENCH_HORIZON = 25  # bench.py's advance(1.0) count in the standard run: 5 warm-up + 20 timed steps


def test_forms_error_at_bench_workload(ctx, oracle):
    """8,192 tracers of the 1M benchmark ensemble (evenly spaced), advanced by
    the benchmark's whole run, 25 x advance(1.0), with the step model trained and
    calibrated as bench.py does it: relative final-position error of every form
    against the FP64 oracle and against the exact solution (a GPU run at rtol =
    atol = 1e-12).

    The plain form takes the oracle's step sequence; its difference is rounding,
    amplified on a few sensitive orbits. The other forms take other step
    sequences (the FP32 form occasionally, where rounding flips an accept/reject
    decision; the learned forms always), and two valid rtol = 1e-8 solutions
    differ by their integration errors: over 25 s the oracle's own global error
    reaches ~4e-5 (max over the sample), so the learned forms' difference from
    it cannot stay below 1e-6 there. What the learned forms keep is accuracy:
    their global error against the exact solution is no worse than the plain
    FP64 controller's (the scale is calibrated for that). After one benchmark
    step (1 s) the learned + FP32 form is within 1e-6 of the oracle."""
    import bench
    from tests._util import oracle_tracers
    params, fit = bench.train_step_model(ctx)
    ctx.mlp_set_params(params)
    scale = fit["scale"]
    w = W.gc_bench(1 << 20)
    idx = bench.sample_indices(1 << 20, 8192)
    ws = W.subsample(w, idx)
    f, cfg, tr = oracle_tracers(oracle, ws, "gc")
    oracle.batch_advance(f, cfg, 1, tr, 1.0)
    orc1 = tr["s"][:, :3].copy()
    oracle.batch_advance(f, cfg, 1, tr, float(BENCH_HORIZON - 1))
    orc = tr["s"][:, :3]
    exact, bad = bench.exact_positions(w, idx, BENCH_HORIZON, ctx)
    assert bad == 0
    res = {}
    for form in (PLAIN, FP32, LEARNED, LEARNED_FP32):
        e = gpu_ensemble(ws, "gc", max_rows=4, form=form, learned_scale=scale, learned_every=bench.LEARNED_EVERY)
        e.advance("gc", 1.0)
        one = e.download()["s"][:3].T.copy()
        for _ in range(BENCH_HORIZON - 1):
            e.advance("gc", 1.0)
            e.rows(reset=True)
        h = e.download()
        assert np.all(h["status"] == 0)
        pos = h["s"][:3].T
        res[form] = {"oracle_1s": bench.pos_errors(one, orc1), "oracle": bench.pos_errors(pos, orc),
                     "exact": bench.pos_errors(pos, exact)}
    res["oracle_vs_exact"] = bench.pos_errors(orc, exact)
    print("errors at the bench horizon", res, "scale", scale)
    pl = res[PLAIN]
    # plain: rounding-level differences from the oracle
    assert pl["oracle"]["median"] < 1e-11 and pl["oracle"]["max"] < 1e-6, pl
    assert pl["oracle_1s"]["max"] < 1e-8, pl
    # FP32: the plain controller's steps except where rounding flips a decision
    assert res[FP32]["oracle"]["median"] < 1e-6 and res[FP32]["oracle_1s"]["max"] < 1e-6, res[FP32]
    # the learned forms: global error no worse than the plain form's (25 %
    # allowance for the sample: the scale was calibrated on other tracers)
    for form in (LEARNED, LEARNED_FP32):
        r = res[form]["exact"]
        assert r["p99"] <= 1.25 * pl["exact"]["p99"] and r["max"] <= 1.25 * pl["exact"]["max"], (form, res)
    # one benchmark step: the learned + FP32 form within 1e-6 of the oracle
    assert res[LEARNED_FP32]["oracle_1s"]["max"] <= 1e-6, res[LEARNED_FP32]


def test_switch_head_on_harris_adaptive(ctx):
    """Switch-labelled samples from Adaptive runs in the Harris sheet (even
    tracers train, odd tracers test): the trained switch head against the
    majority-class predictor. The kernels keep the exact check either way."""
    w = W.subsample(W.config3(), np.arange(0, 262144, 32))
    tr = W.subsample(w, np.arange(0, len(w["mass"]), 2))
    te = W.subsample(w, np.arange(1, len(w["mass"]), 2))
    ctx.mlp_samples_reserve(1 << 21, 0)
    e = gpu_ensemble(tr, "adaptive", max_rows=4096, max_switch=64, collect=1)
    e.advance("adaptive", tr["delta"] / 3)
    s = ctx.mlp_samples_download()
    lab = s[:, 17]
    assert np.all(np.isnan(s[lab >= 0, 16])) and np.all(np.isfinite(s[lab < 0, 16]))
    n_sw = int(np.sum(lab >= 0))
    assert n_sw > 1000 and 0 < np.mean(lab[lab >= 0]) < 1, (n_sw, np.mean(lab[lab >= 0]))
    p, losses = learned.train(ctx, steps=2000, batch=4096, lr=2e-3, seed=3)
    ctx.mlp_samples_reserve(1 << 21, 0)
    e = gpu_ensemble(te, "adaptive", max_rows=4096, max_switch=64, collect=1)
    e.advance("adaptive", te["delta"] / 3)
    m = learned.switch_metrics(ctx, ctx.mlp_samples_download())
    print("switch head", m, "losses", losses)
    majority = max(m["base_rate"], 1 - m["base_rate"])
    assert m["accuracy"] > majority, m
