#!/usr/bin/env python
"""Benchmark: logL evaluations per second of the batched GB300 likelihood.

Workload (default ``config2``): a 256x256 float32 mock, SIE + external shear
lens, Sersic bulge + exponential disk sources, sky foreground, 25x25
Gaussian-plus-wings PSF, 25-point (5x5) pixel quadrature, 10% random mask,
1024 candidate parameter vectors per launch.  One step = one evaluation of
the whole batch (set_params -> render -> convolve + chi^2 -> logL).

Arms
  default            the CUDA path in the default (exact) floating-point
                     mode, whose logL equals the FP32 oracle's (elementary
                     functions correctly rounded, no contraction).  ``value``:
                     device-resident parameters, CUDA-event timing of K steps
                     on the launching stream.  ``e2e``: the public C-ABI call
                     ``lg_eval_batch`` with host parameters and host logL
                     (H2D + D2H inside the timing).  ``parity``: the first
                     --parity-n timed candidates against the FP32 oracle on
                     the host.  ``fast_mode``: the same batch timed with
                     LG_FLAG_FAST_MATH (hardware-approximate functions, FMA
                     contraction) and its parity.
  --impl reference   the reference algorithm on the host CPU: the
                     reference's own sources compiled here if that build is
                     present (oracle/_ref), else the C++ restatement (oracle),
                     with all host threads, one candidate per step as the
                     reference's callback does.

Multi-GPU: one process per GPU under torchrun; each rank evaluates its own
batch (replicas, weak scaling; no collective on the data path); the JSON
``value`` is the total over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "logL evals/s"
UNIT = "evals/s"

# Source-level FP32 operation count per ray of each plugin's evaluation
# (add/sub/mul/div/sqrt = 1, each libm-class call = 1), counted from the
# plugin formulas; plus per-ray overheads of compute() and the quadrature
# loop.  Used for the algorithmic FLOPs of the render kernel.
# DRAM bytes (read + write) of one launch of the dominant kernel, measured
# with ncu on the GB300 for the default workload (the kernel's time under ncu
# matched the bench's CUDA events): the render writes the raw models
# (268 MB algorithmic; about 60 MB are still in L2 when it ends) and the
# convolution reads them once (268 MB) -- no re-reads.
MEASURED_TRAFFIC = {("config2", 1024, "render", "fast"): 208.45e6, ("config2", 1024, "convolve", "fast"): 269.2e6,
                    ("config2", 1024, "render", "exact"): 210.09e6, ("config2", 1024, "convolve", "exact"): 270.17e6}
# Thread instructions per ray of the render kernel (ncu smsp__inst_executed.sum
# x 32 / rays of the launch) per floating-point mode, config2 workload: the
# render is bound by instruction issue (4 warp instructions per SM and cycle),
# so its issue rate against that peak is the second roofline it reports.
MEASURED_INSTR_PER_RAY = {("config2", "exact"): 406.5, ("config2", "fast"): 90.8}

RAY_FLOPS = {
    "sis": 12, "sis_plus_shear": 20, "nsis": 10, "sie": 26, "sie_plus_shear": 34, "nsie": 30,
    "point_mass": 9, "epl": 172, "epl_plus_shear": 180, "sersic": 17, "sersic_old": 17, "exponential": 15,
    "devauc": 16, "gauss": 16, "sky": 6,
}
RAY_OVERHEAD = 4 + 8  # x + qq, ww*f + acc; per lens plane: a += .., finiteness test and y -= a


def ray_flops(plugins):
    return sum(RAY_FLOPS[p] for p in plugins) + RAY_OVERHEAD + sum(1 for p in plugins if p not in RAY_FLOPS)


def workload(name):
    from lensed_gb300 import workloads

    if name == "config2":
        return workloads.config2(), 1024
    if name == "small":
        return workloads.small(), 1
    if name == "large":
        return workloads.large(), 256
    if name == "systems":
        return workloads.systems(), 256
    raise SystemExit(f"unknown workload {name}")


def run_sampler(args):
    """Nested sampling of the small workload (128^2 SIE + Sersic + sky, 9-point
    rule, 13 free parameters), nlive = 1000: plain ellipsoidal proposal vs the
    learned coupling-flow proposal retrained every 1000 replacements.  Reports
    exact-likelihood calls, wall time, ln Z and posterior means of both."""
    import lensed_gb300 as lg
    from lensed_gb300 import workloads

    s = workloads.small()
    ctx = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=1024, flags=args.flags)
    out = {}
    seeds = [11 + 7 * k for k in range(max(1, args.sampler_seeds))]
    flow = {"layers": args.flow_layers, "width": args.flow_width, "epochs": args.flow_epochs}
    if args.train_tc >= 0:
        flow["train_tc"] = args.train_tc
    arms = [("plain", {}), ("flow", {"proposal": lg.PROPOSAL_FLOW, "flow_every": 1000})]
    if args.max_ellipsoids > 1:
        arms.append(("plain_multi", {"max_ellipsoids": args.max_ellipsoids}))
    for name, kw in arms:
        if name == "plain" and args.skip_plain:
            continue
        runs = [ctx.nested(nlive=1000, batch=1024, tol=0.1, seed=sd, flow=flow, **kw) for sd in seeds]
        r = runs[0]
        w = np.exp(r["logwt"])
        _, phys = ctx.eval_cube(r["samples"])
        mean_phys = (w[:, None] * phys).sum(0) / w.sum()
        std_phys = np.sqrt(np.maximum((w[:, None] * (phys - mean_phys) ** 2).sum(0) / w.sum(), 0.0))
        out[name] = {"logz": r["logz"], "logz_err": r["logz_err"], "ncall": r["ncall"], "wall_s": r["wall_s"],
                     "eval_s": r["eval_s"], "train_s": r["train_s"], "propose_s": r["propose_s"],
                     "niter": r["niter"], "flow_proposals": r["n_flow_proposals"],
                     "ellipsoid_proposals": r["n_ellipsoid_proposals"],
                     "posterior_mean": dict(zip(ctx.ids, [float(v) for v in mean_phys])),
                     "posterior_std": dict(zip(ctx.ids, [float(v) for v in std_phys])),
                     # every seed: ln Z, calls, wall time
                     "seeds": {str(sd): {"logz": x["logz"], "ncall": x["ncall"], "wall_s": x["wall_s"],
                                         "flow_proposals": x["n_flow_proposals"]} for sd, x in zip(seeds, runs)},
                     "mean_ncall": float(np.mean([x["ncall"] for x in runs])),
                     "mean_wall_s": float(np.mean([x["wall_s"] for x in runs])),
                     "mean_logz": float(np.mean([x["logz"] for x in runs])),
                     # standard error of the mean ln Z from the seeds' spread
                     "mean_logz_se": float(np.std([x["logz"] for x in runs], ddof=1) / np.sqrt(len(runs)))
                     if len(runs) > 1 else float(r["logz_err"])}
    line = {"metric": "calls & wall-time to lnZ (learned vs plain sampler)", "unit": "calls, s",
            "value": out["flow"]["mean_ncall"], "higher_is_better": False, "n_gpus": 1, "dtype": "f32 (f64 evidence)",
            "data": "synthetic", "config": {"workload": s.name, "nlive": 1000, "batch": 1024, "tol": 0.1,
                                            "flow": flow},
            "plain": out.get("plain"), "flow": out["flow"], "plain_multi_ellipsoid": out.get("plain_multi"),
            # mean ln Z of the learned runs minus that of the plain runs, and
            # its standard error (a single run's ln Z scatters by about its
            # quoted error, 0.23 here, so single-seed differences say little)
            "dlogz": out["flow"]["mean_logz"] - out["plain"]["mean_logz"] if "plain" in out else None,
            "dlogz_se": float(np.hypot(out["flow"]["mean_logz_se"], out["plain"]["mean_logz_se"]))
            if "plain" in out else None,
            "seeds": seeds,
            # largest difference of the learned and plain posterior means, in
            # posterior standard deviations (free parameters)
            "max_mean_shift_in_std": max(
                abs(out["flow"]["posterior_mean"][k] - out["plain"]["posterior_mean"][k])
                / out["plain"]["posterior_std"][k]
                for k in out["plain"]["posterior_std"] if out["plain"]["posterior_std"][k] > 0) if "plain" in out
            else None,
            "truth": dict(zip(ctx.ids, [float(v) for v in ctx.to_map_order(s.truth)]))}
    print(json.dumps(line), flush=True)


def run_flow_inverse(args):
    """The learned proposal's inverse flow (d = 13, 8 coupling layers, width
    128) on M latent points with random weights: device time per launch of
    the tcgen05 kernel and of the FP32 kernel (CUDA events, 20 launches after
    warm-up), and their largest differences on the same points."""
    import ctypes as C

    import lensed_gb300 as lg

    d, layers, width, hidden = 13, 8, 128, 2
    M = args.batch or 65536
    rng = np.random.Generator(np.random.PCG64(7))
    npar = lg.lib().lg_flow_nparams(d, layers, width, hidden)
    params = (rng.normal(size=npar) * 0.08).astype(np.float32)
    z = rng.normal(size=(M, d)).astype(np.float32)
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    out = {}
    for tc in (1, 0):
        u = np.zeros((M, d), np.float32)
        ld = np.zeros(M, np.float32)
        rc = lg.lib().lg_flow_inverse_check(0, d, layers, width, hidden, 1, tc, P(params), P(z), M, P(u), P(ld))
        ms = np.zeros(1, np.float32)
        rct = lg.lib().lg_flow_inverse_time(0, d, layers, width, hidden, tc, P(params), P(z), M, 20, P(ms))
        out["tc" if tc else "fp32"] = {"rc": rc, "rc_time": rct, "ms": float(ms[0]), "u": u, "ld": ld}
    # dense FLOPs per point: 8 layers x 2 x (6.5 x 128 + 128 x 128 + 128 x 13)
    flop = 2.0 * sum(a * b for a, b in [(d // 2 + d % 2, width), (width, width), (width, 2 * (d // 2 + d % 2))]) * layers
    line = {"metric": "learned-proposal inverse flow", "M": M, "flow": [d, layers, width, hidden],
            "ms_per_launch": {k: v["ms"] for k, v in out.items()},
            "latent_points_per_s": {k: M / (v["ms"] * 1e-3) for k, v in out.items() if v["ms"] > 0},
            "tflops": {k: M * flop / (v["ms"] * 1e-3) / 1e12 for k, v in out.items() if v["ms"] > 0},
            "rc": {k: [v["rc"], v["rc_time"]] for k, v in out.items()},
            "max_abs_diff_u": float(np.abs(out["tc"]["u"] - out["fp32"]["u"]).max()),
            "max_abs_diff_logdet": float(np.abs(out["tc"]["ld"] - out["fp32"]["ld"]).max())}
    print(json.dumps(line), flush=True)


def run_flow_train(args):
    """Training steps of the learned proposal's flow (d = 13, 8 coupling
    layers, width 128, 2 hidden layers) on minibatches of `--batch` rows
    (default 256, the sampler's) of 1024 points with random weights: device
    time per step (forward + backward + Adam) of the tcgen05 step and of the
    FP32-weight step (CUDA events, 50 steps after warm-up), and the
    tensor-core step's dense FLOPs per second (forward, recomputed forward
    and the two backward products of every dense)."""
    import ctypes as C

    import lensed_gb300 as lg

    d, layers, width, hidden = 13, 8, 128, 2
    batch = args.batch or 256
    n = max(1024, batch)
    rng = np.random.Generator(np.random.PCG64(7))
    npar = lg.lib().lg_flow_nparams(d, layers, width, hidden)
    params = (rng.normal(size=npar) * 0.05).astype(np.float32)
    x = rng.normal(size=(n, d)).astype(np.float32)
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    out = {}
    for tc in (1, 0):
        ms = np.zeros(1, np.float32)
        rc = lg.lib().lg_flow_train_time(0, d, layers, width, hidden, tc, P(params), P(x), n, batch, 50, P(ms))
        out["tc" if tc else "fp32"] = {"rc": rc, "ms": float(ms[0])}
    # dense multiply-adds per row and layer: 16 x 128 + 128 x 128 + 128 x 16
    # (K and N padded to 16); 4 passes (forward, recomputed forward, dX, dW)
    flop = 2.0 * (16 * width + width * width + width * 16) * layers * 4
    line = {"metric": "learned-proposal training step", "batch": batch, "flow": [d, layers, width, hidden],
            "ms_per_step": {k: v["ms"] for k, v in out.items()},
            "rows_per_s": {k: batch / (v["ms"] * 1e-3) for k, v in out.items() if v["ms"] > 0},
            "tc_tflops": batch * flop / (out["tc"]["ms"] * 1e-3) / 1e12 if out["tc"]["ms"] > 0 else None,
            "rc": {k: v["rc"] for k, v in out.items()}}
    print(json.dumps(line), flush=True)


def run_systems(args):
    """16 systems of uneven sizes, 256 candidates each, one batch per step
    through lg_systems_eval (host buffers in and out: value = e2e)."""
    import lensed_gb300 as lg
    from lensed_gb300 import workloads

    syst, per = workload("systems")
    t_create = time.perf_counter()
    S = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], syst[0].objects, capacity=[per] * len(syst),
                   rule="g3k7", flags=args.flags | (0 if args.no_autotune else lg.LG_FLAG_AUTOTUNE))
    t_create = time.perf_counter() - t_create
    params = []
    for s in syst:
        ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=1)
        params.append(ctx.to_map_order(workloads.draw_candidates(s, per, seed=1)))
        ctx.close()
    for _ in range(args.warmup):
        S.eval(params)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = S.eval(params)
    dt = (time.perf_counter() - t0) / args.steps
    total = per * len(syst)
    assert all(np.all(np.isfinite(o)) for o in out)
    pix = sum(s.width * s.height for s in syst) / len(syst)
    line = {"metric": METRIC, "value": total / dt, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (f64 chi^2 reduction)", "data": "synthetic",
            "config": {"workload": f"{len(syst)} systems, sizes " + ",".join(str(s.width) for s in syst)
                       + f" (mean {pix:.0f} px), epl_plus_shear+sersic+sky, odd PSFs 15-31, rule g3k7",
                       "batch": total, "per_system": per, "launch_shape": S.launch_shape,
                       "autotune": (S.tune_report.splitlines() or ["off"])[0]
                                   + f" (creation {t_create:.1f} s)"},
            "gpu_launches": 4 * args.steps,
            "e2e": {"value": total / dt, "unit": UNIT,
                    "h2d_bytes_per_step": int(sum(p.nbytes for p in params)), "d2h_bytes_per_step": 8 * total}}
    print(json.dumps(line), flush=True)


def describe(s, B):
    return {
        "workload": f"{s.name}: {s.width}x{s.height} float32, objects " + "+".join(s.plugins)
                    + (f", {s.psf.shape[0]}x{s.psf.shape[1]} PSF" if s.psf is not None else ", no PSF")
                    + f", rule {s.rule}" + (", 10% mask" if s.mask is not None else ""),
        "batch": B,
        "params": int(s.truth.size),
        "l2": "per-step working set larger than L2 (raw model images B x N x 4 B = "
              f"{B * s.width * s.height * 4 / 2**20:.0f} MiB written and re-read)" if s.psf is not None
              else "inputs resident; no L2 flush (compute-bound)",
        "data": "synthetic seeded mock (no public dataset)",
    }


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle(s, threads, precision=32):
    from lensed_gb300 import quadrature
    from oracle.oracle import Oracle

    # the C library's float functions per ray: the natural CPU implementation
    return Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image,
                  weight=s.weight, precision=precision, threads=threads, math="libm")


def Oracle_for(s, threads):
    """The FP32 oracle of a workload (correctly rounded elementary
    functions: the reference's semantics the parity bound is stated for)."""
    from lensed_gb300 import quadrature
    from oracle.oracle import Oracle

    return Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), psf=s.psf, image=s.image,
                  weight=s.weight, precision=32, threads=threads)


def parity_block(got, want, mode):
    d = np.abs(np.asarray(got) - np.asarray(want))
    return {"mode": mode, "n": int(d.size), "max_abs_dlogL": float(d.max()), "median_abs_dlogL": float(np.median(d)),
            "bound": 1e-3, "within_bound": bool(d.max() <= 1e-3),
            "abs_logL_range": [float(np.abs(want).min()), float(np.abs(want).max())],
            "oracle": "FP32 restatement, elementary functions evaluated in double and rounded once"}


def mode_name(flags):
    return "strict" if flags & 1 else ("fast" if flags & 16 else "exact")


def ref_impl(s):
    """The reference's own code built for the host (oracle/_ref) if present
    for this workload, else the C++ restatement."""
    try:
        from lensed_gb300 import quadrature
        from oracle import ref as R

        psf = (0, 0) if s.psf is None else (s.psf.shape[1], s.psf.shape[0])
        if R.available([(p, 0) for p in s.plugins], s.width, s.height, psf, quadrature.rule(s.rule).size, "libm"):
            return "reference", R
    except Exception:
        pass
    return "port", None


def cpu_rate(s, cand, threads, budget_s=12.0, kind="port", ref=None):
    """Evaluate candidates one at a time on the host until the budget is spent."""
    o = ref.Reference.for_system(s, threads) if ref is not None else cpu_oracle(s, threads)
    o.loglike(cand[:1])  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        o.loglike(cand[n % len(cand): n % len(cand) + 1])
        n += 1
        dt = time.perf_counter() - t0
        if (dt > budget_s and n >= 2) or n >= 200:
            break
    return n / dt, n, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from lensed_gb300 import workloads

    s, B = workload(args.workload)
    cand = workloads.draw_candidates(s, 64, seed=1)
    threads = os.cpu_count() or 1
    kind, R = ref_impl(s)
    o = R.Reference.for_system(s, threads) if R is not None else cpu_oracle(s, threads)
    for i in range(args.warmup):
        o.loglike(cand[i % 64: i % 64 + 1])
    t0 = time.perf_counter()
    for i in range(args.steps):
        o.loglike(cand[i % 64: i % 64 + 1])
    dt = time.perf_counter() - t0
    v = args.steps / dt
    sample = (f"{args.steps} candidates, one logL per step, {threads} threads (OpenMP over pixels); "
              + ("the reference's own kernels compiled for the host" if kind == "reference"
                 else "the C++ restatement"))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 chi^2 sum)", "data": "synthetic",
            "config": describe(s, B),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="config2")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU baseline and the oracle parity check of the timed results")
    ap.add_argument("--flags", type=int, default=0,
                    help="lg_options.flags: 0 exact (default), 1 strict, 16 fast, 16|4 fast with IEEE div/sqrt")
    ap.add_argument("--no-fast", action="store_true", help="do not time the fast mode beside the exact one")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-candidate-per-call measurement")
    ap.add_argument("--plain-only", action="store_true", help="only the one-candidate-per-call measurement")
    ap.add_argument("--parity-n", type=int, default=128,
                    help="timed candidates checked against the FP32 oracle (CPU) for the parity block")
    ap.add_argument("--flow-layers", type=int, default=8)
    ap.add_argument("--flow-width", type=int, default=128)
    ap.add_argument("--flow-epochs", type=int, default=200)
    ap.add_argument("--train-tc", type=int, default=-1,
                    help="sampler workload: 1 tensor-core training steps, 0 the FP32-weight ones (-1: the default)")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--sampler-seeds", type=int, default=16,
                    help="sampler workload: runs (seeds) per sampler (one run's ln Z scatters by about 0.2)")
    ap.add_argument("--max-ellipsoids", type=int, default=8,
                    help="sampler workload: also run the plain sampler with this many bounding ellipsoids (1: skip)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shape instead of timing the tuner's candidates at creation")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "systems":
        return run_systems(args)
    if args.workload == "sampler":
        return run_sampler(args)
    if args.workload == "flow-inverse":
        return run_flow_inverse(args)
    if args.workload == "flow-train":
        return run_flow_train(args)

    import torch

    import lensed_gb300 as lg
    from lensed_gb300 import workloads

    from lensed_gb300 import replicas

    rank, world, local, dist = replicas.init()
    torch.cuda.set_device(local)
    s, B = workload(args.workload)
    if args.batch:
        B = args.batch
    # a dedicated stream: the context's kernels and the timing events share it
    stream = torch.cuda.Stream(device=f"cuda:{local}")
    cand_obj = workloads.draw_candidates(s, B, seed=replicas.candidate_seed(rank))

    def timed(flags, clocks=None):
        """Create a context in the given floating-point mode and time K steps
        of the device-resident batch evaluation (CUDA events on the launching
        stream, barrier and max over ranks)."""
        t_create = time.perf_counter()
        ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, device=local, max_batch=B,
                         flags=flags | (0 if args.no_autotune else lg.LG_FLAG_AUTOTUNE))
        t_create = time.perf_counter() - t_create
        cand = ctx.to_map_order(cand_obj)
        d_params = torch.from_numpy(np.ascontiguousarray(cand)).to(f"cuda:{local}")
        d_logL = torch.empty(B, dtype=torch.float64, device=f"cuda:{local}")
        sh = stream.cuda_stream

        def step():
            ctx.eval_batch_device(d_params.data_ptr(), B, d_logL.data_ptr(), sh)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if not np.all(np.isfinite(d_logL.cpu().numpy())):
            raise SystemExit("non-finite logL in warm-up")
        if clocks:
            clocks.start()
            time.sleep(0.3)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1)
        clk = clocks.stop() if clocks else None
        ms = replicas.max_over_ranks(ms, dist, device=f"cuda:{local}")
        value = replicas.aggregate(B * args.steps, ms / 1e3, world)
        logL = d_logL.cpu().numpy()
        # per-stage device times (the reference's --profile stages), averaged
        stage = np.zeros(4)
        nprof = 5
        for _ in range(nprof):
            stage += ctx.profile(d_params.data_ptr(), B, d_logL.data_ptr())
        stage /= nprof
        return {"ctx": ctx, "cand": cand, "value": value, "ms": ms, "clocks": clk, "logL": logL, "stage": stage,
                "t_create": t_create}

    # the headline: the default (exact) mode unless --flags asks otherwise
    # plain mode: one candidate per call with a host sync (the reference
    # flow, e.g. MultiNest's callback), on a context created for it
    # (max_batch = 1; its launch shape tuned for one candidate)
    def plain_leg(flags):
        ctx1 = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, device=local, max_batch=1,
                          flags=flags | (0 if args.no_autotune else lg.LG_FLAG_AUTOTUNE))
        shape = ctx1.launch_shape
        # through the C ABI as a C caller makes it (lg_eval_batch, B = 1),
        # the argument pointers prepared once
        import ctypes as C

        hp1 = ctx1.to_map_order(cand_obj[:64])
        rows = [np.ascontiguousarray(hp1[i:i + 1]) for i in range(len(hp1))]
        ptrs = [r.ctypes.data_as(C.POINTER(C.c_double)) for r in rows]
        one = np.zeros(1)
        pone = one.ctypes.data_as(C.POINTER(C.c_double))
        call = lg.lib().lg_eval_batch
        for i in range(20):
            if call(ctx1.h, ptrs[i % len(ptrs)], 1, pone):
                raise SystemExit("plain evaluation failed")
        n1 = 1000
        t0 = time.perf_counter()
        for i in range(n1):
            call(ctx1.h, ptrs[i % len(ptrs)], 1, pone)
        rate = n1 / (time.perf_counter() - t0)
        if not np.isfinite(one[0]):
            raise SystemExit("non-finite plain logL")
        # the reference-signature callback loglike(cube, ndim, npar, lnew,
        # ctx) (src/nested.h:3): unit cube in, physical values written back
        cb = lg.lib().loglike
        cb.restype = None
        cb.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                       C.c_void_p]
        nd, npar, lnew = C.c_int(ctx1.ndims), C.c_int(ctx1.npars), C.c_double()
        cubes = np.random.Generator(np.random.PCG64(3)).random((64, ctx1.npars))
        work = np.empty(ctx1.npars)
        pw = work.ctypes.data_as(C.POINTER(C.c_double))
        for i in range(20):
            work[:] = cubes[i % 64]
            cb(pw, C.byref(nd), C.byref(npar), C.byref(lnew), ctx1.h)
        t0 = time.perf_counter()
        for i in range(n1):
            work[:] = cubes[i % 64]
            cb(pw, C.byref(nd), C.byref(npar), C.byref(lnew), ctx1.h)
        rate_cb = n1 / (time.perf_counter() - t0)
        ctx1.close()
        return rate, shape, rate_cb

    if args.plain_only:
        # one-candidate calls alone (for profiling the plain path)
        if rank == 0:
            r = plain_leg(args.flags)
            line = {"metric": METRIC + " (one candidate per call)", "value": r[0], "unit": UNIT,
                    "n_gpus": 1, "higher_is_better": True, "data": "synthetic", "config": describe(s, 1),
                    "fp_mode": mode_name(args.flags), "plain_launch_shape": r[1],
                    "plain_loglike_callback_per_s": r[2]}
            print(json.dumps(line), flush=True)
        return

    head = timed(args.flags, Clocks(local))
    ctx, cand, value, ms, clk, logL_gpu, stage, t_create = (head[k] for k in (
        "ctx", "cand", "value", "ms", "clocks", "logL", "stage", "t_create"))
    # the fast mode beside it (hardware-approximate functions, FMA contraction)
    fast = None
    if args.flags == 0 and not args.no_fast:
        fast = timed(lg.LG_FLAG_FAST_MATH)
        fast["ctx"].close()

    # end to end through the public C ABI with host buffers
    hp = np.ascontiguousarray(cand)
    for _ in range(2):
        ctx.eval_batch(hp)
    ne2e = max(3, min(args.steps, 50))
    t0 = time.perf_counter()
    for _ in range(ne2e):
        ll_host = ctx.eval_batch(hp)
    e2e_dt = (time.perf_counter() - t0) / ne2e
    e2e = replicas.aggregate(B, replicas.max_over_ranks(e2e_dt, dist, device=f"cuda:{local}"), world)

    plain, plain_shape, plain_loglike = None, None, None
    fast_plain = None
    if rank == 0 and not args.no_plain:
        plain, plain_shape, plain_loglike = plain_leg(args.flags)
        if fast is not None:
            fast_plain = plain_leg(lg.LG_FLAG_FAST_MATH)

    # roofline of the dominant kernel (headline mode)
    N, Q = s.width * s.height, len(lg.quad_rules()[s.rule][1])
    render_flops = B * N * Q * ray_flops(s.plugins)
    conv_flops = 2.0 * B * N * (s.psf.size if s.psf is not None else 0)
    try:
        peak_fp32 = lg.measure_fp32_peak(local)
    except Exception:
        peak_fp32 = None
    nominal = 152 * 128 * 2 * 2070e6 / 1e12
    dom = "render" if stage[1] >= stage[2] else "convolve"
    if dom == "render":
        ach = render_flops / (stage[1] * 1e-3) / 1e12
    else:
        ach = conv_flops / (stage[2] * 1e-3) / 1e12
    peak = peak_fp32 or nominal
    roof = {"kernel": "lg_render_raw" if dom == "render" and s.psf is not None else
            ("lg_render_chi2" if dom == "render" else "lg_conv_chi2"),
            "bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "peak_source": "measured FP32 FMA probe (lg_measure_fp32_peak) on this GPU" if peak_fp32 else
                           "nominal 152 SM x 128 lanes x 2 flop x 2070 MHz",
            "nominal_peak": nominal, "traffic": MEASURED_TRAFFIC.get((args.workload, B, dom, mode_name(args.flags))),
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch of this workload and mode"
                              if (args.workload, B, dom, mode_name(args.flags)) in MEASURED_TRAFFIC else None,
            "algorithmic_flops_per_launch": render_flops if dom == "render" else conv_flops,
            "stage_ms": {"set_params": float(stage[0]), "render": float(stage[1]), "convolve": float(stage[2]),
                         "finish": float(stage[3])},
            "convolve_tflops": (conv_flops / (stage[2] * 1e-3) / 1e12) if stage[2] > 0 else None,
            "rays_per_s": B * N * Q / (stage[1] * 1e-3)}
    ipr = MEASURED_INSTR_PER_RAY.get((args.workload, mode_name(args.flags)))
    if dom == "render" and ipr and clk and clk.get("sm_mhz"):
        # issue roofline: thread instructions per second against 152 SMs x 4
        # warp instructions x 32 threads per cycle at the sampled SM clock
        ach_i = ipr * B * N * Q / (stage[1] * 1e-3) / 1e12
        peak_i = 152 * 4 * 32 * clk["sm_mhz"] * 1e6 / 1e12
        roof["issue"] = {"thread_instructions_per_ray": ipr, "achieved": ach_i, "peak": peak_i,
                         "unit": "T thread-instructions/s", "frac": ach_i / peak_i,
                         "source": "instructions per ray from ncu smsp__inst_executed.sum (one launch, "
                                   "this workload and mode); time from this run's render stage"}

    config = describe(s, B)
    config["fp_mode"] = mode_name(args.flags)
    config["launch_shape"] = ctx.launch_shape
    config["autotune"] = (ctx.tune_report.splitlines() or ["off"])[0] + f" (context creation {t_create:.1f} s)"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (f64 chi^2 reduction)", "data": "synthetic",
            "config": config, "gpu_launches": 3 * args.steps,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(hp.nbytes), "d2h_bytes_per_step": 8 * B},
            "plain_evals_per_s": plain, "plain_loglike_callback_per_s": plain_loglike,
            "plain_launch_shape": plain_shape, "roofline": roof}
    if fast is not None:
        fst = fast["stage"]
        line["fast_mode"] = {"value": fast["value"], "unit": UNIT, "ms_per_step": fast["ms"] / args.steps,
                             "flags": "LG_FLAG_FAST_MATH",
                             "stage_ms": {"set_params": float(fst[0]), "render": float(fst[1]),
                                          "convolve": float(fst[2]), "finish": float(fst[3])}}
        if fast_plain:
            line["fast_mode"].update({"plain_evals_per_s": fast_plain[0], "plain_launch_shape": fast_plain[1],
                                      "plain_loglike_callback_per_s": fast_plain[2]})
    if clk:
        line["clocks"] = clk
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        kind, R = ref_impl(s)
        v, n, dt = cpu_rate(s, workloads.draw_candidates(s, 8, seed=1), threads, kind=kind, ref=R)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                                "sample": f"{n} candidates of the same workload, one at a time, {dt:.1f} s"}
        # parity of the timed results: the first n of the timed candidates
        # against the FP32 oracle (the checker; the reference's semantics
        # with correctly rounded elementary functions)
        npar = min(B, args.parity_n)
        o32 = Oracle_for(s, threads)
        want = o32.loglike(cand_obj[:npar])
        line["parity"] = parity_block(logL_gpu[:npar], want, mode_name(args.flags))
        if fast is not None:
            line["fast_mode"]["parity"] = parity_block(fast["logL"][:npar], want, "fast")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    ctx.close()


if __name__ == "__main__":
    main()
