#!/usr/bin/env python3
"""Benchmark: accepted RK steps/s of the 1M-tracer guiding-centre ensemble.

Workload (``gc_doubledipole_1M``): 1,048,576 electrons in the double-dipole
field, config-2 distributions (L 4-7, MLT 0-24 h, KE log-uniform 0.1-10 MeV,
equatorial pitch 15-85 deg, seed 0), Tao-Chan-Brizard guiding-centre
equations, DOPRI5 at rtol = atol = 1e-8, GCtimestep 1 s. One step = one
``GuidingCenter.advance(1.0)`` of every tracer (one output interval).

Four forms run on the same start state: plain FP64, FP32 stages, learned
(FP64 with MLP step proposals) and learned+FP32. The step MLP is trained first
(untimed) on guiding centres of an independent config-2 draw, and its proposal
scale is calibrated so that its global error matches the plain controller's.
``value`` is the learned+FP32 form's whole-job accepted steps / device time
with the state resident in HBM; ``forms`` holds every form's accepted steps/s,
rejections, right-hand sides, simulated tracer-seconds/s and gyro-periods/s.
``e2e`` is the learned+FP32 metric through the public API with the state copied
from pinned host memory and back inside the timed region. ``accuracy``
compares the final positions of an evenly spaced sample of the ensemble after
the whole run (warm-up + timed steps) with the FP64 oracle (the CPU leg below)
and with a tight-tolerance GPU run (the exact solution). ``--impl reference``
times the CPU restatement of the reference algorithm (the oracle) on all host
cores over a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "accepted RK steps/s at 1M particles, learned+FP32 vs plain FP64 GPU at rtol 1e-8"
UNIT = "accepted steps/s"

# Algorithmic FP64 work of one accepted DOPRI5 step of the Tao-Chan-Brizard
# guiding-centre equations in the double-dipole field: 6 right-hand sides of
# 446 flops (7-point stencil of 7 B evaluations) + 275 flops of stage
# combination, error norm and control; rsqrt/sqrt/div/pow count as one flop each.
FLOPS_PER_ACCEPTED_STEP = 6 * 446 + 275 + 6 * 23 + 4
# FP32-pipe thread instructions (FFMA + FADD + FMUL) per accepted step of the
# learned + FP32 guiding-centre kernel k_gc32<DoubleDipole, learned> (the
# headline form): the float-float stages and centre field, the FP32 stencil
# differences, the equations and the step learner, from one ncu capture of the
# 262,144-tracer case (sm__sass_thread_inst_executed_op_{ffma,fadd,fmul}_pred_on.sum
# over the launch's accepted steps; profiles/k_gc32_learned_doubledipole_262k_full.md).
FP32_OPS_PER_ACCEPTED_STEP = 9575
# DRAM traffic of one k_gc32 launch per tracer and simulated second
# (dram__bytes_read.sum + dram__bytes_write.sum of the same capture: local-memory
# traffic; the algorithmic state traffic is ~464 B per tracer and launch).
TRAFFIC_PER_TRACER_SECOND = 1.532e5
# Pipe and issue utilisation of the same capture: the headline kernel saturates
# neither pipe, and instruction fetch is its top stall (the bound it is on).
HEADLINE_NCU = {"issue_active": 0.482, "fp32_pipe_active": 0.354, "fp64_pipe_active": 0.303,
                "top_stall": "no_instruction"}
# FP64 FMA issue rate of a GB300 SM (thread-instructions per clock; ncu's FP64
# pipe peak, 304 per clock over the 152 SMs).
FP64_FMA_PER_CLK_PER_SM = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=None,
                    help="tracers per GPU (default: 2^20 for the headline workload, the workload's own size otherwise)")
    ap.add_argument("--bc-delta", type=float, default=2.0, help="bc_drift_65k: BounceCenter.advance(delta) per step")
    ap.add_argument("--cpu-sample", type=int, default=0, help="tracers in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="gc_doubledipole_1M",
                    choices=["gc_doubledipole_1M", "harris_adaptive_262k", "earthdipole_particles", "compressed_adaptive",
                             "gc_grid_262k", "gc_dense_cadence", "bc_drift_65k"],
                    help="gc_doubledipole_1M: the headline metric; harris_adaptive_262k: the batching comparison; "
                         "earthdipole_particles (config 4) and compressed_adaptive (config 5): form comparisons "
                         "on --n tracers")
    ap.add_argument("--forms", default="plain,fp32,learned,learned_fp32",
                    help="comma-separated forms to time (plain, fp32, learned, learned_fp32); the headline is "
                         "learned_fp32 when listed")
    ap.add_argument("--learned-every", type=int, default=LEARNED_EVERY,
                    help="learned forms: the network runs on every k-th step-loop iteration of a warp "
                         "(rapt_config.learned_every)")
    ap.add_argument("--acc-sample", type=int, default=8192,
                    help="tracers in the accuracy sample (evenly spaced; 0: no accuracy check)")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    # the package's default context (field evaluations) on this rank's GPU
    os.environ.setdefault("RAPT_DEVICE", os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return rank, ws, dist
    return 0, 1, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.p is None:
            return out
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if sm:
            hi = [s for s in sm if s > 0.5 * max(sm)] or sm
            out = {"sm_mhz": statistics.median(hi), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def sample_indices(n, n_sample):
    return np.unique(np.linspace(0, n - 1, n_sample).astype(np.int64))


def cpu_baseline(w, n_sample, horizon, threads):
    """The oracle (CPU restatement of the reference algorithm) on host cores:
    an evenly spaced sample of the guiding centres of workload `w` advanced
    `horizon` seconds. Returns (accepted steps/s, accepted, seconds, final
    states)."""
    from oracle import oracle as O
    from rapt_gb300 import workloads as W
    idx = sample_indices(len(w["mass"]), n_sample)
    w = W.subsample(w, idx)
    f = O.field("DoubleDipole")
    cfg = O.config(rtol=1e-8, atol=1e-8, gctimestep=1.0)
    tr = O.tracers_from_structs([O.gc_new_pa(f, w["pos"][i], w["v"][i], w["pa"][i], 0.0, w["mass"][i],
                                             w["charge"][i]) for i in range(len(idx))])
    t = time.perf_counter()
    O.batch_advance(f, cfg, 1, tr, float(horizon), nthreads=threads)
    dt = time.perf_counter() - t
    acc = int(tr["naccept"].sum())
    return acc / dt, acc, dt, tr


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    from rapt_gb300 import workloads as W
    threads = os.cpu_count() or 1
    n = args.cpu_sample or 16384
    w = W.gc_bench(1 << 20)
    vals = []
    for i in range(args.warmup + args.steps):
        v, acc, dt, _ = cpu_baseline(w, n, 1.0, threads)
        if i >= args.warmup:
            vals.append((acc, dt))
    acc = sum(a for a, _ in vals)
    dt = sum(d for _, d in vals)
    value = acc / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, config-2 distributions)",
            "config": {"workload": "gc_doubledipole_1M", "sample_tracers_per_step": n,
                       "step": "GuidingCenter.advance(1.0) of each sampled tracer"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d of the 1,048,576 tracers (evenly spaced), 1 s each" % n},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


FORMS = (("plain", 0), ("fp32", 1), ("learned", 2), ("learned_fp32", 3))
HEADLINE = "learned_fp32"
LEARNED_EVERY = 4  # the network runs on every k-th step-loop iteration of a warp (rapt_config.learned_every)


def gyro_frequency_sum(w, magB):
    """Sum over tracers of 1 / cyclotron period (utils.cyclotron_period) at the start."""
    c = 299792458.0
    gamma = 1.0 / np.sqrt(1.0 - (w["v"] / c) ** 2)
    return float(np.sum(np.abs(w["charge"]) * magB / (2 * np.pi * gamma * w["mass"])))


def train_step_model(ctx, every=None):
    """Trains the step MLP on guiding centres drawn from the config-2
    distributions (8,192 electrons, an independent draw from the benchmark's):
    plain-controller samples then three on-policy rounds, 10 s each; then the
    proposal scale is calibrated on the global error of 2,048 other config-2
    electrons over 10 s (learned.calibrate_global). Deterministic."""
    from rapt_gb300 import learned, workloads as W
    w = W.subsample(W.config2(), np.arange(0, 65536, 8))
    t = time.perf_counter()
    p, info = learned.fit_gc(w, 10.0, ctx=ctx, rounds=3, steps=3000, capacity=1 << 23, mask=7)
    ctx.mlp_set_params(p)
    wc = W.subsample(W.config2(), np.arange(4, 65536, 32))
    scale, table = learned.calibrate_global(wc, 10.0, ctx=ctx, every=every or LEARNED_EVERY)
    info["scale_samples"] = info["scale"]
    info["calibration_global"] = table
    info["scale"] = scale if scale is not None else min(r["scale"] for r in table if r["scale"] is not None)
    info["seconds"] = time.perf_counter() - t
    info["accepted_steps_generated"] = int(sum(c["accepted"] for c in info["collect"]))
    return p, info


def hbm_peak_gbs():
    """Measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json),
    else 6,800 GB/s, an earlier measurement of the same copy."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def pos_errors(pos, ref):
    e = np.linalg.norm(pos - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)), "max": float(e.max())}


def exact_positions(w, idx, horizon, ctx):
    """Final positions of the sample tracers from a tight-tolerance run
    (rtol = atol = 1e-12): the exact solution the forms' global errors are
    measured against."""
    from rapt_gb300 import Ensemble, workloads as W
    ws = W.subsample(w, idx)
    e = Ensemble.from_workload(ws, "gc", max_rows=int(horizon) + 4, ctx=ctx, rtol=1e-12, atol=1e-12,
                               nsteps=1000000)
    e.advance("gc", float(horizon))
    h = e.download()
    return h["s"][:3].T.copy(), int(np.count_nonzero(h["status"]))


def run_ours(args, rank, ws, dist):
    import torch
    from rapt_gb300 import Ensemble, workloads as W, fields as F
    args.n = args.n or (1 << 20)
    from rapt_gb300 import _native as N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = N.Context(dev)
    fp64_peak, fp32_peak = ctx.measure_peaks()
    forms = [(nm, f) for nm, f in FORMS if nm in args.forms.split(",")]
    names = dict(forms)
    if "plain" not in names:
        raise SystemExit("--forms must include plain")
    head = HEADLINE if HEADLINE in names else ("fp32" if "fp32" in names else "plain")
    fit = None
    every = args.learned_every
    if "learned" in names or "learned_fp32" in names:
        params, fit = train_step_model(ctx, every)
        ctx.mlp_set_params(params)
    if ws > 1:
        # one ensemble of ws x n tracers, split into contiguous shards of equal
        # estimated cost; rank r advances shard r
        from rapt_gb300 import shard
        w_all = W.gc_bench(args.n * ws)
        field = F.DoubleDipole()
        field.bind(ctx)
        magB = field.magB(np.column_stack([np.zeros(len(w_all["mass"])), w_all["pos"]]))
        costs = shard.cost_estimate(1, w_all["pos"], w_all["v"], w_all["mass"], w_all["charge"], magB, 1.0)
        a, b = shard.shard(costs, rank, ws)
        w = W.subsample(w_all, np.arange(a, b))
        del w_all
    else:
        w = W.gc_bench(args.n)
    n = len(w["mass"])
    ens = Ensemble(F.DoubleDipole(), n, max_rows=4, ctx=ctx, pinned=not args.no_e2e)
    ens.configure(**w["params"])
    ens.set_guiding_centers(w["pos"], w["v"], pa=w["pa"], t0=0.0, mass=w["mass"], charge=w["charge"])
    init = {k: (v.copy()) for k, v in ens.h.items()}
    fgyro = gyro_frequency_sum(w, ens.field.magB(np.column_stack([np.zeros(n), w["pos"]])))
    idx = sample_indices(n, args.acc_sample) if args.acc_sample > 0 else None
    horizon = args.warmup + args.steps
    scale = fit["scale"] if fit else 1.0

    def reset():
        for k, v in init.items():
            ens.h[k][...] = v
        ens.upload()

    results, finals = {}, {}
    barrier(dist)
    clk = Clocks(dev) if rank == 0 else None
    t_all = time.perf_counter()
    for name, form in forms:
        reset()
        ens.configure(form=form, learned_scale=scale, learned_every=every, collect=0)
        for _ in range(args.warmup):
            ens.advance("gc", 1.0)
            ens.rows(reset=True)
        # ---- device-resident timed region (a profiler range: ncu --profile-from-start off
        # captures these launches only)
        barrier(dist)
        acc = rej = rhs = launches = 0
        dev_ms = 0.0
        torch.cuda.cudart().cudaProfilerStart()
        for _ in range(args.steps):
            st = ens.advance("gc", 1.0)
            acc += st["accepted"]
            rej += st["rejected"]
            rhs += st["rhs_evals"]
            dev_ms += st["kernel_ms"]
            launches += st["kernel_launches"]
            ens.ctx.check(ens.ctx.L.rapt_rows_download(ens.ctx.h, None, None, None, None, None, 1), "reset rows")
        torch.cuda.cudart().cudaProfilerStop()
        barrier(dist)
        # after the timed steps: tracers that ended with a failure status (RAPT_ST_*)
        h = ens.download()
        bad = h["status"] != 0
        codes, counts = np.unique(h["status"][bad], return_counts=True)
        failed = {"tracers": int(np.count_nonzero(bad)), "status": {int(c): int(k) for c, k in zip(codes, counts)},
                  "first": [int(i) for i in np.flatnonzero(bad)[:4]]}
        if idx is not None:
            finals[name] = (h["s"][:3, idx].T.copy(), failed)
        dev_s = allmax(dist, dev_ms * 1e-3)
        acc_all = allsum(dist, acc)
        sim = allsum(dist, float(n * args.steps))
        results[name] = {"accepted_per_s": acc_all / dev_s, "ms_per_step": dev_s * 1e3 / args.steps,
                         "accepted": int(acc), "rejected": int(rej), "rhs_evals": int(rhs),
                         "reject_rate": rej / max(acc, 1), "rhs_per_tracer_second": rhs / (n * args.steps),
                         "tracer_seconds_per_s": sim / dev_s,
                         "gyro_periods_per_s": allsum(dist, fgyro * args.steps) / dev_s,
                         "kernel_launches": int(launches), "device_ms": dev_ms, "failed": failed}
    wall = time.perf_counter() - t_all
    clocks = clk.stop() if clk else None
    headr = results[head]
    plain = results["plain"]
    for r in results.values():
        r["accepted_per_s_vs_plain"] = r["accepted_per_s"] / plain["accepted_per_s"]
        r["tracer_seconds_per_s_vs_plain"] = r["tracer_seconds_per_s"] / plain["tracer_seconds_per_s"]
    # ---- end to end through the public API with pinned host buffers (headline form)
    e2e = None
    if not args.no_e2e:
        reset()
        ens.configure(form=names[head], learned_scale=scale, learned_every=every)
        h2d = sum(ens.h[k].nbytes for k in ens.h)
        d2h = h2d + n * ens.max_rows * 8 * 8  # state back + rows buffer
        barrier(dist)
        t1 = time.perf_counter()
        acc_e = 0
        for _ in range(args.steps):
            ens.upload()
            st = ens.advance("gc", 1.0)
            acc_e += st["accepted"]
            ens.download()
            ens.rows(reset=True)
        e2e_s = allmax(dist, time.perf_counter() - t1)
        e2e = {"value": allsum(dist, acc_e) / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "form": head}
    gathered = None
    if ws > 1:
        # the host gather of every shard's final state (untimed)
        from rapt_gb300 import shard
        h = ens.download()
        g = shard.gather(dist, {"s": h["s"][:4].T.copy(), "status": h["status"].copy(),
                                "naccept": h["naccept"].copy()})
        tot = shard.sum_counters(dist, {"tracers": n, "accepted": int(h["naccept"].sum())})
        if rank == 0:
            gathered = {"tracers": int(len(g["status"])), "failed": int(np.count_nonzero(g["status"])),
                        "accepted_last_form": int(g["naccept"].sum()), "counters": tot,
                        "shards": "contiguous, balanced by estimated cost (rapt_gb300.shard)"}
    if rank != 0:
        return
    # ---- roofline: each kernel against the pipe it runs on
    import torch
    num_sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    fp64_spec = num_sms * FP64_FMA_PER_CLK_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    plain_tf = FLOPS_PER_ACCEPTED_STEP * plain["accepted"] / (plain["device_ms"] * 1e-3) / 1e12
    roof_plain = {"kernel": "k_gc<DoubleDipole> (plain FP64)", "bound": "fp64", "unit": "TFLOP/s",
                  "achieved": plain_tf, "peak": fp64_spec, "frac": plain_tf / fp64_spec,
                  "peak_note": "%d SMs x %d FP64 FMA/clk x 2 flops x %.0f MHz (sampled SM clock)" % (
                      num_sms, FP64_FMA_PER_CLK_PER_SM, sm_mhz),
                  "peak_microbench": fp64_peak, "frac_microbench": plain_tf / fp64_peak,
                  "flops_per_accepted_step": FLOPS_PER_ACCEPTED_STEP,
                  "flops_note": "algorithmic FP64 flops of one DOPRI5 step (FMA = 2, rsqrt/div/pow = 1)"}
    line = {"metric": METRIC, "value": headr["accepted_per_s"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": headr["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 stages (float-float) + f64 control" if head != "plain" else "f64",
            "data": "synthetic (seeded, config-2 distributions at 2^20 tracers per GPU)",
            "config": {"workload": "gc_doubledipole_1M", "tracers_per_gpu": n, "form": head,
                       "eom": "TaoChanBrizard", "method": "DOPRI5", "rtol": 1e-8, "atol": 1e-8,
                       "step": "GuidingCenter.advance(1.0) of every tracer",
                       "l2": "state 1M x 232 B > L2 (compute bound; no flush)",
                       "parallelism": "%d cost-balanced shards of one ensemble" % ws if ws > 1 else "single GPU"},
            "forms": results, "gpu_launches": int(headr["kernel_launches"]), "clocks": clocks, "wall_s": wall}
    if head in ("fp32", "learned_fp32"):
        ops = FP32_OPS_PER_ACCEPTED_STEP * headr["accepted"] / (headr["device_ms"] * 1e-3) / 1e12
        fp32_ops_peak = fp32_peak / 2  # the microbenchmark counts an FMA as 2 flops
        traffic = TRAFFIC_PER_TRACER_SECOND * n
        line["roofline"] = {"kernel": "k_gc32<DoubleDipole> (%s)" % head, "bound": "fp32", "unit": "Tops/s",
                            "achieved": ops, "peak": fp32_ops_peak, "frac": ops / fp32_ops_peak,
                            "ops_per_accepted_step": FP32_OPS_PER_ACCEPTED_STEP,
                            "ops_note": "FP32-pipe thread instructions (FFMA/FADD/FMUL) per accepted step, from ncu",
                            "peak_source": "measured in-run: FP32 FMA chains (rapt_measure_peaks)",
                            "traffic": traffic, "traffic_note": "DRAM bytes per launch (local memory), "
                            "scaled from a 262,144-tracer ncu capture",
                            "traffic_frac_hbm": traffic / (headr["ms_per_step"] * 1e-3) / (hbm_peak_gbs() * 1e9),
                            "hbm_peak": hbm_peak_gbs(),
                            "ncu_262k": HEADLINE_NCU,
                            "plain_kernel": roof_plain}
    else:
        line["roofline"] = dict(roof_plain)
    if fit:
        line["step_model"] = {"scale": fit["scale"], "scale_from_samples": fit["scale_samples"],
                              "learned_every": every, "train_seconds": fit["seconds"],
                              "accepted_steps_generated": fit["accepted_steps_generated"],
                              "samples": int(sum(c["samples"] for c in fit["collect"])),
                              "calibration": fit["calibration"][-1], "calibration_global": fit["calibration_global"],
                              "losses": fit["losses"][-1]}
    if e2e:
        line["e2e"] = e2e
    if gathered:
        line["gather"] = gathered
    if not args.no_cpu_baseline:
        v, a, dt, tr = cpu_baseline(w, len(idx) if idx is not None else 4096, horizon, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d of the %d tracers (evenly spaced), %d s each (%.1f s)" % (
                                    len(tr), n, horizon, dt)}
        if idx is not None:
            exact, bad = exact_positions(w, idx, horizon, ctx)
            orc = tr["s"][:, :3]
            line["accuracy"] = {
                "sample_tracers": int(len(idx)), "horizon_s": horizon,
                "measure": "relative final-position error |dx| / |x| after warm-up + timed steps",
                "vs_oracle": {k: pos_errors(v[0], orc) for k, v in finals.items()},
                "vs_exact": {k: pos_errors(v[0], exact) for k, v in finals.items()},
                "oracle_vs_exact": pos_errors(orc, exact),
                "exact": "GPU plain FP64 at rtol = atol = 1e-12", "failed": {k: v[1] for k, v in finals.items()},
                "exact_failed": bad}
    print(json.dumps(line), flush=True)


def advance_all(ens, kind, delta):
    """Advance and resume tracers stopped by a full row buffer until all are
    done (rows are reset on the device, not downloaded); returns summed stats."""
    tot = {"accepted": 0, "rejected": 0, "kernel_ms": 0.0, "kernel_launches": 0, "switches": 0, "done": 0}
    st = ens.advance(kind, delta)
    while True:
        for k in tot:
            tot[k] += st[k]
        if tot["done"] >= ens.n:
            return tot
        ens.ctx.check(ens.ctx.L.rapt_rows_download(ens.ctx.h, None, None, None, None, None, 1), "reset rows")
        st = ens.advance_resume(kind)


def run_config3(args, rank, ws, dist):
    """Batching comparison on the Harris-sheet Adaptive ensemble (262,144
    protons, durations log-uniform 1-300 s): the default persistent grid, the
    autotuned launch shape with graph replay, and the unbatched pattern (one
    launch sequence per tracer) on an evenly spaced sample."""
    from rapt_gb300 import Ensemble, workloads as W, autotune as A, _native as N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = N.Context(dev)
    w = W.config3(seed=rank)
    n = len(w["mass"])
    sim = float(np.sum(w["delta"]))
    # autotune on a 16k sample advanced by a tenth of its durations
    ws_ = A.sample(w, 16384)
    es = Ensemble.from_workload(ws_, "adaptive", max_rows=1024, max_switch=64, ctx=ctx)
    best, table = A.tune(es, "adaptive", ws_["delta"] / 10, use_cache=False)
    del es
    ens = Ensemble.from_workload(w, "adaptive", max_rows=1024, max_switch=64, ctx=ctx)
    init = {k: v.copy() for k, v in ens.h.items()}
    res = {}
    for name, shape in (("default", {}), ("tuned", best)):
        cfg = dict(w["params"])
        cfg.update(shape)
        ens.configure(**{k: 0 for k in ("threads_per_block", "blocks_per_sm", "use_graph")})
        ens.configure(**cfg)
        for k, v in init.items():
            ens.h[k][...] = v
        ens.upload()
        ens.adaptive_init()
        barrier(dist)
        st = advance_all(ens, "adaptive", w["delta"])
        dev_s = allmax(dist, st["kernel_ms"] * 1e-3)
        res[name] = {"shape": shape or "128 threads, max blocks/SM, no graph", "device_s": dev_s,
                     "accepted_per_s": allsum(dist, st["accepted"]) / dev_s,
                     "tracer_seconds_per_s": allsum(dist, sim) / dev_s, "switches": int(st["switches"]),
                     "kernel_launches": int(st["kernel_launches"])}
    # unbatched: one launch sequence per tracer, on a 256-tracer sample
    sm = A.sample(w, 256)
    e1 = Ensemble.from_workload(sm, "adaptive", max_rows=1024, max_switch=64, ctx=ctx, per_tracer_launches=1)
    st = advance_all(e1, "adaptive", sm["delta"])
    sim1 = float(np.sum(sm["delta"]))
    res["per_tracer_launches"] = {"sample_tracers": len(sm["mass"]), "device_s": st["kernel_ms"] * 1e-3,
                                  "accepted_per_s": st["accepted"] / (st["kernel_ms"] * 1e-3),
                                  "tracer_seconds_per_s": sim1 / (st["kernel_ms"] * 1e-3),
                                  "kernel_launches": int(st["kernel_launches"])}
    if rank != 0:
        return
    line = {"metric": "Adaptive tracer-seconds/s, batched graph vs per-tracer launches", "workload": "harris_adaptive_262k",
            "value": res["tuned"]["tracer_seconds_per_s"], "unit": "tracer-seconds/s", "n_gpus": ws,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded, config-3 distributions)",
            "config": {"workload": "harris_adaptive_262k", "tracers_per_gpu": n, "sim_tracer_seconds": sim,
                       "gctimestep": 0.5, "rtol": 1e-8, "atol": 1e-8},
            "results": res, "autotune": {"best": best, "table": table},
            "speedup_batched_vs_per_tracer": res["tuned"]["tracer_seconds_per_s"] /
            res["per_tracer_launches"]["tracer_seconds_per_s"]}
    print(json.dumps(line), flush=True)


def run_forms_workload(args, rank, ws, dist):
    """Form comparison on config 4 (particles in the Earth dipole, 50
    gyro-periods, DOP853) or config 5 (Adaptive in the compressed dipole with its
    induced E, 200 s), on --n tracers: device time, accepted and rejected steps,
    simulated tracer-seconds/s of each form. For config 5 the step MLP is
    trained first (guiding-centre segments use it; particle segments run the
    plain controller)."""
    from rapt_gb300 import Ensemble, workloads as W, _native as N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = N.Context(dev)
    if args.n:
        n = args.n
    else:
        n = (1 << 18) if args.workload == "earthdipole_particles" else (1 << 16)
    if args.workload == "earthdipole_particles":
        w = W.subsample(W.config4(seed=rank), np.arange(0, 1 << 20, max(1, (1 << 20) // n))[:n])
        kind, delta, rows = "particle", w["delta"], 520
        forms = [("plain", 0), ("fp32", 1)]
        scale = 1.0
    else:
        w = W.subsample(W.config5(seed=rank), np.arange(0, 1 << 20, max(1, (1 << 20) // n))[:n])
        kind, delta, rows = "adaptive", 200.0, 1024
        forms = [(nm, f) for nm, f in FORMS if nm in args.forms.split(",")]
        if any(f >= 2 for _, f in forms):
            params, fit = train_step_model(ctx, args.learned_every)
            ctx.mlp_set_params(params)
            scale = fit["scale"]
        else:
            scale = 1.0
    ens = Ensemble.from_workload(w, kind, max_rows=rows, max_switch=64, ctx=ctx)
    init = {k: v.copy() for k, v in ens.h.items()}
    sim = float(np.sum(np.broadcast_to(delta, (len(w["mass"]),))))
    res, finals = {}, {}
    if kind == "particle":
        p0 = np.linalg.norm(init["s"][3:6].T, axis=1)
    for name, form in forms:
        for k, v in init.items():
            ens.h[k][...] = v
        ens.upload()
        if kind == "adaptive":
            ens.adaptive_init()
        ens.configure(form=form, learned_scale=scale, learned_every=args.learned_every)
        barrier(dist)
        st = advance_all(ens, kind, delta)
        h = ens.download()
        finals[name] = (h["s"][:3].T.copy(), h["status"].copy(), h["mode"].copy())
        if kind == "particle":
            # kinetic-energy drift: |p| is conserved in the static dipole
            p1 = np.linalg.norm(h["s"][3:6].T, axis=1)
            drift = np.abs(p1 / p0 - 1.0)[h["status"] == 0]
            energy_drift = {"median": float(np.median(drift)), "p99": float(np.percentile(drift, 99)),
                            "max": float(drift.max())}
        dev_s = allmax(dist, st["kernel_ms"] * 1e-3)
        res[name] = {"device_s": dev_s, "accepted": int(st["accepted"]), "rejected": int(st["rejected"]),
                     "reject_rate": st["rejected"] / max(st["accepted"], 1),
                     "accepted_per_s": allsum(dist, st["accepted"]) / dev_s,
                     "tracer_seconds_per_s": allsum(dist, sim) / dev_s, "switches": int(st["switches"]),
                     "failed": int(np.count_nonzero(h["status"])),
                     "status_counts": {int(k): int(v) for k, v in zip(*np.unique(h["status"], return_counts=True))},
                     "naccept_per_tracer": {"median": float(np.median(h["naccept"])),
                                            "p99": float(np.percentile(h["naccept"], 99)),
                                            "max": int(h["naccept"].max())}}
        if kind == "particle":
            res[name]["energy_drift"] = energy_drift
    if rank != 0:
        return
    plain = res["plain"]
    for r in res.values():
        r["tracer_seconds_per_s_vs_plain"] = r["tracer_seconds_per_s"] / plain["tracer_seconds_per_s"]
    # error against the plain FP64 form on the same ensemble (tracers that both
    # finished without a failure status)
    p_pos, p_st, p_mode = finals["plain"]
    for name, (pos, st_, mode) in finals.items():
        if name == "plain":
            continue
        ok = (st_ == 0) & (p_st == 0)
        e = np.linalg.norm(pos[ok] - p_pos[ok], axis=1) / np.linalg.norm(p_pos[ok], axis=1)
        res[name]["error_vs_plain"] = {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)),
                                       "max": float(e.max()), "compared": int(ok.sum()),
                                       "same_final_mode": int(np.sum(ok & (mode == p_mode)))}
    print(json.dumps({"workload": args.workload, "tracers_per_gpu": len(w["mass"]), "n_gpus": ws,
                      "kind": kind, "sim_tracer_seconds": sim, "results": res}), flush=True)


def grid_cpu_baseline(g, w, n_sample, threads):
    """The oracle on a sample of the gridded-field guiding centres, 1 s each."""
    from oracle import oracle as O
    idx = np.linspace(0, len(w["mass"]) - 1, n_sample).astype(np.int64)
    f = O.grid_field(g._t, g._x, g._y, g._z, g._B, g._E, static=g.static)
    p = w["params"]
    cfg = O.config(rtol=p["rtol"], atol=p["atol"], gctimestep=p["gctimestep"])
    tr = O.tracers_from_structs([O.gc_new_pa(f, w["pos"][i], w["v"][i], w["pa"][i], w["t0"], w["mass"][i],
                                             w["charge"][i]) for i in idx])
    t = time.perf_counter()
    O.batch_advance(f, cfg, 1, tr, 1.0, nthreads=threads)
    dt = time.perf_counter() - t
    acc = int(tr["naccept"].sum())
    return acc / dt, acc, dt


def run_grid_workload(args, rank, ws, dist):
    """Guiding centres in a gridded field (Grid, fields.py:513-814): 262,144
    electrons in a 241 x 241 x 121 x 3-snapshot dipole grid (1.0 GB of B and E
    resident in HBM), GuidingCenter.advance(1.0) per step, plain FP64 and FP32
    forms; accepted steps/s against the oracle on host cores."""
    from rapt_gb300 import Ensemble, workloads as W, _native as N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = N.Context(dev)
    n = args.n or (1 << 18)
    w = W.gc_grid(n, seed=rank)
    t_build = time.perf_counter()
    g = W.dipole_grid()
    t_build = time.perf_counter() - t_build
    ens = Ensemble(g, n, max_rows=8, ctx=ctx)
    ens.configure(**w["params"])
    ens.set_guiding_centers(w["pos"], w["v"], pa=w["pa"], t0=w["t0"], mass=w["mass"], charge=w["charge"])
    init = {k: v.copy() for k, v in ens.h.items()}
    steps, warmup = min(args.steps, 12), max(3, min(args.warmup, 6))  # the snapshots span 20 s
    res = {}
    clk = Clocks(dev) if rank == 0 else None
    for name, form in (("plain", 0), ("fp32", 1)):
        for k, v in init.items():
            ens.h[k][...] = v
        ens.upload()
        ens.configure(form=form)
        for _ in range(warmup):
            ens.advance("gc", 1.0)
            ens.rows(reset=True)
        barrier(dist)
        acc = rej = launches = 0
        dev_ms = 0.0
        for _ in range(steps):
            st = ens.advance("gc", 1.0)
            acc += st["accepted"]
            rej += st["rejected"]
            dev_ms += st["kernel_ms"]
            launches += st["kernel_launches"]
            ens.rows(reset=True)
        barrier(dist)
        h = ens.download()
        dev_s = allmax(dist, dev_ms * 1e-3)
        res[name] = {"accepted_per_s": allsum(dist, acc) / dev_s, "ms_per_step": dev_s * 1e3 / steps,
                     "accepted": int(acc), "rejected": int(rej), "reject_rate": rej / max(acc, 1),
                     "tracer_seconds_per_s": allsum(dist, float(n * steps)) / dev_s,
                     "kernel_launches": int(launches),
                     "status_counts": {int(k): int(v) for k, v in zip(*np.unique(h["status"], return_counts=True))}}
    clocks = clk.stop() if clk else None
    if rank != 0:
        return
    grid_bytes = int(g._B.nbytes + (g._E.nbytes if g._E is not None else 0))
    line = {"metric": "accepted RK steps/s, guiding centres in a gridded field", "workload": "gc_grid_262k",
            "value": res["plain"]["accepted_per_s"], "unit": UNIT, "n_gpus": ws, "steps": steps, "warmup": warmup,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded, config-2 distributions; "
            "gridded dipole with E, 3 snapshots)",
            "config": {"workload": "gc_grid_262k", "tracers_per_gpu": n, "grid": list(g._B.shape[:4]),
                       "grid_bytes": grid_bytes, "gctimestep": 0.5, "rtol": w["params"]["rtol"],
                       "atol": w["params"]["atol"],
                       "static": False, "grid_build_s": t_build,
                       "l2": "grid 1.0 GB > L2; tracers spread over it"},
            "forms": res, "clocks": clocks}
    if not args.no_cpu_baseline:
        n_s = args.cpu_sample or 2048
        v, a, dt = grid_cpu_baseline(g, w, n_s, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": "%d of the %d tracers, 1 s each (%.1f s)" % (n_s, n, dt)}
    print(json.dumps(line), flush=True)


def run_dense_workload(args, rank, ws, dist):
    """Output cadence against cost: 262,144 config-2 electrons with rows every
    0.01 s, GuidingCenter.advance(0.5) per step, the reference's restart per row
    against dense output (one integration per advance, rows from the continuous
    extension); simulated tracer-seconds/s and right-hand sides per
    tracer-second of each, plain FP64."""
    from rapt_gb300 import Ensemble, workloads as W, fields as F, _native as N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = N.Context(dev)
    n = args.n or (1 << 18)
    w = W.subsample(W.gc_bench(1 << 20, seed=rank), np.arange(0, 1 << 20, (1 << 20) // n)[:n])
    cadence, span = 0.01, 0.5
    # 50 rows per step, plus the 17 a dense-output step may cover
    ens = Ensemble(F.DoubleDipole(), n, max_rows=128, ctx=ctx)
    ens.configure(rtol=1e-8, atol=1e-8, gctimestep=cadence)
    ens.set_guiding_centers(w["pos"], w["v"], pa=w["pa"], t0=0.0, mass=w["mass"], charge=w["charge"])
    init = {k: v.copy() for k, v in ens.h.items()}
    steps, warmup = args.steps, max(3, args.warmup)
    res = {}
    clk = Clocks(dev) if rank == 0 else None
    for name, dense in (("restart", 0), ("dense", 1)):
        for k, v in init.items():
            ens.h[k][...] = v
        ens.upload()
        ens.configure(dense_output=dense)
        for _ in range(warmup):
            ens.advance("gc", span)
            ens.rows(reset=True)
        barrier(dist)
        acc = rhs = launches = 0
        dev_ms = 0.0
        for _ in range(steps):
            st = ens.advance("gc", span)
            acc += st["accepted"]
            rhs += st["rhs_evals"]
            dev_ms += st["kernel_ms"]
            launches += st["kernel_launches"]
            ens.rows(reset=True)
        barrier(dist)
        h = ens.download()
        dev_s = allmax(dist, dev_ms * 1e-3)
        sim = allsum(dist, float(n * steps * span))
        res[name] = {"tracer_seconds_per_s": sim / dev_s, "accepted_per_s": allsum(dist, acc) / dev_s,
                     "ms_per_step": dev_s * 1e3 / steps, "rhs_per_tracer_second": rhs / (n * steps * span),
                     "accepted": int(acc), "kernel_launches": int(launches),
                     "failed": int(np.count_nonzero(h["status"])),
                     "status_counts": {int(k): int(v) for k, v in zip(*np.unique(h["status"], return_counts=True))}}
    clocks = clk.stop() if clk else None
    if rank != 0:
        return
    line = {"metric": "simulated tracer-seconds/s at a 0.01 s output cadence", "workload": "gc_dense_cadence",
            "value": res["dense"]["tracer_seconds_per_s"], "unit": "tracer-seconds/s", "n_gpus": ws,
            "steps": steps, "warmup": warmup, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded, config-2 distributions)",
            "config": {"workload": "gc_dense_cadence", "tracers_per_gpu": n, "gctimestep": cadence,
                       "step": "GuidingCenter.advance(0.5)", "rtol": 1e-8, "atol": 1e-8},
            "results": res, "dense_vs_restart": res["dense"]["tracer_seconds_per_s"] /
            res["restart"]["tracer_seconds_per_s"], "clocks": clocks}
    print(json.dumps(line), flush=True)


def _bc_inputs(w, magB):
    c = 299792458.0
    gamma = 1.0 / np.sqrt(1.0 - (w["v"] / c) ** 2)
    mu = gamma ** 2 * w["mass"] * (w["v"] * np.sin(np.deg2rad(w["eqpa"]))) ** 2 / (2 * magB)
    st = np.column_stack([np.zeros(len(mu)), w["pos"], np.zeros(len(mu))])
    cst = np.column_stack([w["v"], mu, w["mass"], w["charge"]])
    return st, cst


def bc_cpu_baseline(w, st, cst, delta, n_sample, threads):
    """The oracle's BounceCenter.advance (same algorithm: converged integrals) on
    a sample, one tracer per host thread."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    idx = np.linspace(0, len(cst) - 1, n_sample).astype(np.int64)
    f = O.field("DoubleDipole")
    p = w["params"]

    def one(i):
        cfg = O.config(rtol=p["rtol"], atol=p["atol"])
        s = st[i].copy()
        _, rows, cnt = O.bc_advance(f, cfg, s, cst[i, 0], cst[i, 1], cst[i, 2], cst[i, 3], delta, p["bctimestep"],
                                    p["eyegradientstep"], quad=1)
        return len(rows), int(cnt[0])

    t = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:  # ctypes releases the GIL during each call
        res = list(ex.map(one, idx))
    dt = time.perf_counter() - t
    return sum(r[1] for r in res) / dt, n_sample * delta / dt, dt


def run_bc_workload(args, rank, ws, dist):
    """Bounce centres (BounceCenter.advance): 65,536 protons in the DoubleDipole
    field advanced 2 s per step; each right-hand side traces five field lines
    (the half-bounce path and four second invariants for grad I). Simulated
    tracer-seconds/s and right-hand sides/s, against the oracle on host cores."""
    from rapt_gb300 import workloads as W, fields as F, _native as N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = N.Context(dev)
    n = args.n or (1 << 16)
    w = W.bc_drift(1 << 16, seed=rank)
    if n < (1 << 16):  # an evenly spaced subset of the 65,536
        w = W.subsample(w, np.arange(0, 1 << 16, (1 << 16) // n)[:n])
    F.DoubleDipole().bind(ctx)
    ctx.set_config(rtol=w["params"]["rtol"], atol=w["params"]["atol"])
    magB = ctx.field_eval("magB", np.column_stack([np.zeros(n), w["pos"]]))[:, 0]
    st0, cst = _bc_inputs(w, magB)
    delta = args.bc_delta
    p = w["params"]
    steps, warmup = max(1, min(args.steps, 3)), min(args.warmup, 1)
    st = st0.copy()
    for _ in range(warmup):
        st, rows, nr, status, cnt = ctx.bc_advance(st, cst, delta, p["bctimestep"], p["eyegradientstep"], 32)
    clk = Clocks(dev) if rank == 0 else None
    barrier(dist)
    t0 = time.perf_counter()
    rhs = acc = nrows = 0
    for _ in range(steps):
        st, rows, nr, status, cnt = ctx.bc_advance(st, cst, delta, p["bctimestep"], p["eyegradientstep"], 32)
        rhs += int(cnt[:, 0].sum())
        acc += int(cnt[:, 2].sum())
        nrows += int(nr.sum())
    barrier(dist)
    wall = allmax(dist, time.perf_counter() - t0)
    clocks = clk.stop() if clk else None
    if rank != 0:
        return
    line = {"metric": "simulated bounce-centre seconds/s", "workload": "bc_drift_65k",
            "value": allsum(dist, float(n * steps * delta)) / wall, "unit": "tracer-seconds/s", "n_gpus": ws,
            "steps": steps, "warmup": warmup, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded; protons L 4-7, 0.5-5 MeV, equatorial pitch angle 70-88 deg)",
            "config": {"workload": "bc_drift_65k", "tracers_per_gpu": n, "field": "DoubleDipole",
                       "step": "BounceCenter.advance(%g)" % delta, "bctimestep": p["bctimestep"],
                       "eyegradientstep_re": 0.03, "timing": "host wall clock around rapt_bc_advance "
                       "(copies and per-row launches included)"},
            "rhs_per_s": allsum(dist, rhs) / wall, "accepted_per_s": allsum(dist, acc) / wall,
            "field_line_traces_per_s": 5 * allsum(dist, rhs) / wall, "rows": nrows,
            "status_counts": {int(k): int(v) for k, v in zip(*np.unique(status, return_counts=True))},
            "clocks": clocks}
    if not args.no_cpu_baseline:
        n_s = args.cpu_sample or 256
        v, ts, dt = bc_cpu_baseline(w, st0, cst, delta, n_s, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": ts, "unit": "tracer-seconds/s", "rhs_per_s": v, "cores": os.cpu_count(),
                                "kind": "port", "sample": "%d of the %d bounce centres, %g s each (%.1f s)" % (
                                    n_s, n, delta, dt)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, ws, dist = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
    elif args.workload == "harris_adaptive_262k":
        run_config3(args, rank, ws, dist)
    elif args.workload in ("earthdipole_particles", "compressed_adaptive"):
        run_forms_workload(args, rank, ws, dist)
    elif args.workload == "gc_grid_262k":
        run_grid_workload(args, rank, ws, dist)
    elif args.workload == "gc_dense_cadence":
        run_dense_workload(args, rank, ws, dist)
    elif args.workload == "bc_drift_65k":
        run_bc_workload(args, rank, ws, dist)
    else:
        run_ours(args, rank, ws, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
