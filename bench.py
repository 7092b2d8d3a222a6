#!/usr/bin/env python
"""Benchmark: batched FP64 forward + adjoint of the amalgamated reconciliation
likelihood on one GB300 (families·(logL+grad)/s).

Workload (one step = one likelihood + gradient evaluation over the batch, as
one NUTS leapfrog evaluation): 17-taxon Yule species tree (root age 1) with 3
WGDs, Δt = 0.02, branch-wise log-normal DLWGD rates, 5,000 synthetic families
whose CCDs have log-uniform clade counts in [10, 2000].  Each step perturbs
the log-rates by N(0, 0.01²).

  value     families / device time per step (CUDA events around the step's
            device work on the library's stream: parameter upload, forward,
            adjoint, group reduction), families resident in HBM
  e2e       families / wall time per step of the C-ABI calls a host caller
            makes with host buffers (wg_model_set_rates: slice tables on the
            host; wg_logpdf_grad: H2D from pinned memory, kernels, D2H of
            per-family logL and the gradient, host chain rule)
  --impl reference   the CPU restatement of the reference (forward-mode duals,
            as ForwardDiff) on the host cores, on a bounded sample per step

Multi-GPU: one process per GPU (torchrun); every rank evaluates its own
5,000-family workload (weak scaling, no collective in the timed region).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "families·(logL+grad)/s FP64 @17 taxa: batched adjoint vs plain GPU, rel err ≤1e-10"
METRIC4 = "families·(logL+grad)/s FP64 @40 taxa (50,000 families, 10 WGDs, Δt=0.01), rel err ≤1e-10"
UNIT = "families/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


LAUNCH_PROFILE = os.path.join(ROOT, "profiles", "launches_cfg1_5000fam.txt")


def ncu_traffic():
    """DRAM bytes per evaluation of the 5,000-family workload by kernel
    family, read from the committed ncu launch-list summary (its line
    ``dram_bytes_per_evaluation: adjoint=<bytes> forward=<bytes>
    commit=<sha>``); DRAM traffic cannot be measured inside the timed run."""
    try:
        with open(LAUNCH_PROFILE) as fh:
            for line in fh:
                if line.startswith("dram_bytes_per_evaluation:"):
                    kv = dict(x.split("=", 1) for x in line.split(":", 1)[1].split())
                    return {"adjoint": int(kv["adjoint"]), "forward": int(kv["forward"]),
                            "commit": kv.get("commit")}
    except (OSError, ValueError, KeyError):
        pass
    return None


def workload(nf, config=1):
    if config == 4:
        return (f"cfg4: {nf:,} families, 40-taxon Yule tree + 10 WGDs, Δt=0.01, DLWGD log-normal rates, CCDs from "
                "500 NNI-perturbed trees (heavy-tailed clade counts, widest rows in device memory); "
                "log-likelihood + gradient (169 parameters) per step")
    return (f"cfg1: {nf:,} families, 17-taxon Yule tree + 3 WGDs, Δt=0.02, DLWGD log-normal rates; "
            "log-likelihood + gradient (70 parameters) per step")


def make_workload(synth, config, families, rank):
    if config == 4:
        return synth.config4(n_families=families)
    return synth.config1(seed=1 + rank, n_families=families)


def perturbed(W, wm, rng, scale=0.01):
    r = wm.rates
    return wm(W.DLWGD(λ=r.λ + rng.normal(0, scale, r.λ.size), μ=r.μ + rng.normal(0, scale, r.μ.size), q=r.q,
                      η=r.η))


def cpu_reference(W, wl, ccds_idx, steps, warmup, threads):
    """The oracle (C++ restatement, forward-mode duals) on host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    wm = wl.model
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt, minn=wm.minn, maxn=wm.maxn)
    occ = O.parse_texts(om, [wl.ale[i] for i in ccds_idx], threads)
    r = wm.rates
    rng = np.random.default_rng(123)
    times = []
    for s in range(warmup + steps):
        lam = r.λ + rng.normal(0, 0.01, r.λ.size)
        mu = r.μ + rng.normal(0, 0.01, r.μ.size)
        t0 = time.perf_counter()
        om.gradient(occ, lam, mu, q=r.q, eta=r.η, nthreads=threads)
        dt = time.perf_counter() - t0
        if s >= warmup:
            times.append(dt)
    return len(occ) / float(np.mean(times)), times


PARITY_LOGL = 1e-10  # per-family relative, as the benchmark spec states
PARITY_GRAD = 1e-8   # relative to max(|g|, 1), against forward-mode duals


def parity_check(W, wl, wm, batch, per_family, threads, n_grad=200):
    """The timed workload checked against the oracle after the timed region:
    every family's log L from the last timed step against the oracle's
    value-only logpdf at the same rates, and the gradient of a seeded
    n_grad-family sample (the same batch, weights 1 on the sample and 0
    elsewhere, the condition scaled by the sample size) against the oracle's
    forward-mode duals.  Returns the parity object of the bench line."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from whale_gb300.core import map_gradient

    O.build()
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt, minn=wm.minn, maxn=wm.maxn)
    occ = O.parse_texts(om, wl.ale, threads)
    r = wm.rates
    _, oper = om.logpdf(occ, r.λ, r.μ, q=r.q, eta=r.η, nthreads=threads)
    a, b = np.asarray(per_family, float), np.asarray(oper, float)
    both_inf = np.isneginf(a) & np.isneginf(b)
    rel = np.where(both_inf, 0.0, np.abs(a - b) / np.maximum(np.abs(b), 1e-300))
    # the gradient sample among families whose likelihood is representable
    # (an underflowing family contributes nothing to the gradient)
    fin = np.where(np.isfinite(b))[0]
    sample = np.sort(np.random.default_rng(11).choice(fin, size=min(n_grad, len(fin)), replace=False))
    w = np.zeros(len(occ))
    w[sample] = 1.0
    _, _, dl, dm, dq, de = batch.grad_nodes_weighted(wm, w, float(len(sample)))
    g = map_gradient(wm, dl, dm, dq, de)
    flat = np.concatenate([g["λ"], g["μ"], g["q"], [g["η"]]])
    _, og = om.gradient([occ[i] for i in sample], r.λ, r.μ, q=r.q, eta=r.η, nthreads=threads)
    grel = np.abs(flat - og) / np.maximum(np.abs(og), 1.0)
    out = {"max_rel_logl": float(np.max(rel)), "max_rel_grad": float(np.max(grel)),
           "families_checked": int(len(occ)), "families_grad_checked": int(len(sample)),
           "minus_inf_families": int(np.sum(both_inf)),
           "bars": {"logl": PARITY_LOGL, "grad": PARITY_GRAD},
           "against": "oracle/whale_oracle.cpp (value-only logpdf on all families; duals of chunk 12 on the "
                      "sample) at the rates of the last timed step"}
    out["ok"] = bool(out["max_rel_logl"] <= PARITY_LOGL and out["max_rel_grad"] <= PARITY_GRAD)
    return out


def pick_cpu_sample(W, wl, budget_s, threads):
    """A bounded, size-representative sample of the workload for the CPU leg."""
    n = len(wl.ale)
    order = np.random.default_rng(7).permutation(n)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    wm = wl.model
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt, minn=wm.minn, maxn=wm.maxn)
    r = wm.rates
    # time a probe of 32 families, then scale the sample to the budget
    probe = list(order[:32])
    occ = O.parse_texts(om, [wl.ale[i] for i in probe], threads)
    t0 = time.perf_counter()
    om.gradient(occ, r.λ, r.μ, q=r.q, eta=r.η, nthreads=threads)
    per = (time.perf_counter() - t0) / len(probe)
    k = int(max(32, min(n, budget_s / max(per, 1e-6))))
    return list(order[:k])


def run_track(args, W):
    """TreeTracker sampling of one pick, 1 tree per family of the workload,
    timed both ways after one batched logpdf! (tables in device memory):
    device (wg_track_device + wg_track_nodes: one thread per tree, node
    arrays back) and host (wg_batch_tables download per family +
    wg_backtrack_tables on every host core).  Both give the same trees."""
    import ctypes as C
    from concurrent.futures import ThreadPoolExecutor

    import torch
    from whale_gb300 import synth
    from whale_gb300 import _native as N
    from whale_gb300.track import _draw_seed, sample_device

    wl = make_workload(synth, args.config, args.families, 0)
    wm, ccds = wl.model, wl.ccds()
    b = W.Batch(wm, ccds, tables=True)
    b.logpdf(wm)
    nf = len(ccds)
    fams = list(range(nf))
    seeds = [_draw_seed(0, 0, f) for f in fams]
    L = N.lib()
    wm.load()
    dev = []
    for _ in range(3 + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        arrs = sample_device(b, wm, fams, seeds)
        dev.append(time.perf_counter() - t0)
    dev = dev[3:]
    nodes = sum(a.shape[0] for a in arrs)

    def host_one(f):
        need = N.i64()
        N.check(L.wg_batch_tables(b.ctx.h, b.h, f, None, 0, C.byref(need), None))
        tab = np.zeros(max(need.value, 1))
        N.check(L.wg_batch_tables(b.ctx.h, b.h, f, N.dptr(tab), need.value, C.byref(need), None))
        N.check(L.wg_backtrack_tables(wm._struct.h, ccds[f]._h, N.dptr(tab), tab.size, 1, C.c_uint64(seeds[f]), None,
                                      0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        N.check(L.wg_backtrack_tables(wm._struct.h, ccds[f]._h, N.dptr(tab), tab.size, 1, C.c_uint64(seeds[f]), buf,
                                      need.value, C.byref(need)))
        return len(buf.value)

    threads = os.cpu_count() or 1
    host = []
    with ThreadPoolExecutor(max_workers=threads) as pool:
        for _ in range(1 + max(1, args.steps // 10)):
            t0 = time.perf_counter()
            list(pool.map(host_one, fams))
            host.append(time.perf_counter() - t0)
    host = host[1:]
    # W.track end to end (one pick, trees parsed into RecTrees), both ways
    wt = {}
    for dv in (True, False):
        t0 = time.perf_counter()
        W.track(wm, ccds, [wm.rates], 1, seed=0, summary=False, device=dv)
        wt[dv] = time.perf_counter() - t0
    line = {"metric": "reconciled trees sampled per second (1 tree per family per pick, TreeTracker)",
            "value": nf / float(np.median(dev)), "unit": "trees/s", "n_gpus": 1, "steps": args.steps,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload(nf, args.config), "families": nf, "nodes_per_pick": int(nodes)},
            "device": {"ms_per_pick": 1e3 * float(np.median(dev)),
                       "what": "wg_track_device + wg_track_nodes (one GPU thread per tree, node arrays to the host)"},
            "host": {"ms_per_pick": 1e3 * float(np.median(host)), "threads": threads,
                     "what": "per family: wg_batch_tables download + wg_backtrack_tables (host sampler and text)"},
            "speedup": float(np.median(host)) / float(np.median(dev)),
            "W.track_one_pick_s": {"device": wt[True], "host": wt[False],
                                   "what": "batched logpdf! + sampling + text + RecTree parsing per family"}}
    print(json.dumps(line), flush=True)


def run_tune(args, W):
    """The autotuner on the workload: coordinate descent over the packing
    knobs, the size-class bounds, each class's CTA shape and the launch
    layout, timed by CUDA events; prints the chosen shape per class and its
    time against the defaults."""
    from whale_gb300 import autotune, synth

    wl = make_workload(synth, args.config, args.families, 0)
    wm, ccds = wl.model, wl.ccds()
    nb = {"classes": tuple(range(len(autotune.CLASS_BOUNDS))), "persistent": (0, 1), "adj_overlap": (0, 1, 2, 3),
          **{f"heavy_c{i}": (0, 512, 2048, 1 << 20) for i in range(autotune.N_CLASSES)},
          "target_ops": (320, 480, 720), "target_j": (2, 3, 4), "root_group": (8, 16, 32), "level_j": (2, 3, 4),
          "comb_warp": (0, 24, 48)}
    best, b, log = W.tune(wm, ccds, steps=max(3, args.steps), warmup=3, neighbours=nb, rounds=2)
    rep = autotune.report(best, log)
    rep.update({"metric": "autotuned ms per gradient evaluation", "config": {"workload": workload(len(ccds),
                args.config), "families": len(ccds)}, "unit": "ms", "higher_is_better": False})
    print(json.dumps(rep), flush=True)


def run_reference(args, W, rank):
    if rank != 0:
        return
    from whale_gb300 import synth

    wl = make_workload(synth, args.config, args.families, 0)
    threads = os.cpu_count() or 1
    # each step the whole workload when the run fits in about two minutes of
    # CPU work (a 20-step run on the 16-core host does), else a bounded
    # random sample of it (at 1,000 steps still ~800 families per step,
    # enough to keep every host thread busy)
    per_step = max(0.03, 120.0 / max(1, args.steps + args.warmup))
    idx = pick_cpu_sample(W, wl, per_step, threads)
    v, times = cpu_reference(W, wl, idx, args.steps, args.warmup, threads)
    # the same on one core, for the single-thread figure (a smaller sample)
    idx1 = pick_cpu_sample(W, wl, 2.0, 1)
    v1, _ = cpu_reference(W, wl, idx1, 1, 0, 1)
    line = {
        "impl": "reference", "metric": METRIC4 if args.config == 4 else METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload(args.families, args.config), "families": args.families,
                   "families_in_sample": len(idx),
                   "method": "logL + gradient by forward-mode duals of chunk 12 on host cores"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": (f"all {args.families} families per step" if len(idx) == args.families else
                                    f"{len(idx)} of {args.families} families (random, seed 7) per step")},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_one_core": {"value": v1, "unit": UNIT, "cores": 1,
                         "sample": f"{len(idx1)} of {args.families} families (random, seed 7), one step"},
        "note": "Julia is not available, so the reference itself cannot run; this is the C++ restatement "
                "of its logpdf + ForwardDiff gradient (oracle/whale_oracle.cpp), OpenMP over families; the "
                "workload is generated by the library's host parts (libwhalehost.so), the GPU library is "
                "not loaded",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)  # config 3: 1,000 successive evaluations
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, choices=[1, 4],
                    help="1: 5,000 families on 17 taxa (default); 4: 50,000 families on 40 taxa")
    ap.add_argument("--families", type=int, default=None, help="default: 5,000 (config 1), 50,000 (config 4)")
    ap.add_argument("--tune", action="store_true", help="run the autotuner on the workload and report its choice")
    ap.add_argument("--track", action="store_true",
                    help="time TreeTracker sampling (device vs host) instead of the likelihood")
    ap.add_argument("--persistent", action="store_true",
                    help="one persistent launch per pass instead of one launch per height level and size class")
    ap.add_argument("--checkpoint", action="store_true",
                    help="force per-level recomputation of the adjoint's tables (otherwise only past the budget)")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU work for the CPU leg")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    args = ap.parse_args()
    if args.families is None:
        args.families = 50000 if args.config == 4 else 5000
    if args.config == 4:
        args.no_plain = True  # one launch per family for 50,000 families; its widest families exceed shared memory
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.impl == "reference":
        # the workload is generated by the library's host parts alone: this
        # arm never loads the GPU library
        os.environ["WG_HOST_LIBRARY"] = "1"
    import __graft_entry__

    W = __graft_entry__.load_package()
    if args.impl == "reference":
        run_reference(args, W, rank)
        return
    if args.track:
        run_track(args, W)
        return
    if args.tune:
        run_tune(args, W)
        return
    import torch

    pg = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    from whale_gb300 import synth

    t0 = time.perf_counter()
    wl = make_workload(synth, args.config, args.families, rank)
    wm = wl.model
    ccds = wl.ccds()
    gen_s = time.perf_counter() - t0
    ctx = W.Context(local)
    t0 = time.perf_counter()
    batch = W.Batch(wm, ccds, grad=True, ctx=ctx, checkpoint=args.checkpoint, persistent=args.persistent)
    pack_s = time.perf_counter() - t0
    L = W._native.lib()
    W._native.check(L.wg_ctx_set_timing(ctx.h, 1))
    peak = W._native.dbl()
    W._native.check(L.wg_probe_fp64(ctx.h, W._native.C.byref(peak)))
    fp64_peak = peak.value
    rng = np.random.default_rng(1000 + rank)
    F = W._native.C.c_float
    fms, ams, rms = F(), F(), F()

    # one step through the C ABI, as a ccall caller runs it: the step's per-node
    # natural rates (host arrays) -> wg_model_set_rates (slice tables on the
    # host) -> wg_logpdf_grad (H2D from pinned memory, kernels, D2H of the
    # per-family log L and the gradient, host chain rule) into host buffers
    N_ = W._native
    K = len(wm.order)
    per_b = np.zeros(len(ccds))
    dl_b, dm_b, dq_b = np.zeros(K), np.zeros(K), np.zeros(K)
    tot_b, de_b = N_.dbl(), N_.dbl()
    hm = wm._struct.h

    # (pointers to the caller's buffers made once, as a compiled caller holds them)
    out_ptrs = (N_.dptr(per_b), N_.C.byref(tot_b), N_.dptr(dl_b), N_.dptr(dm_b), N_.dptr(dq_b),
                N_.C.byref(de_b), None, None, None)
    t_ptrs = (N_.C.byref(fms), N_.C.byref(ams), N_.C.byref(rms))

    def step(rates, bh=None):
        _, lam, mu, q, eta, pp = rates
        N_.check(L.wg_model_set_rates(hm, lam, mu, q, eta, pp))
        N_.check(L.wg_logpdf_grad(ctx.h, hm, bh or batch.h, *out_ptrs))
        N_.check(L.wg_ctx_timings(ctx.h, *t_ptrs))
        return tot_b.value, fms.value, ams.value, rms.value

    def inputs(m):
        lam, mu, q, eta, pp = m.node_rates()
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (lam, mu, q, pp)]
        return (arrs, N_.dptr(arrs[0]), N_.dptr(arrs[1]), N_.dptr(arrs[2]), float(eta), N_.dptr(arrs[3]))

    for _ in range(args.warmup):
        step(inputs(perturbed(W, wm, rng)))
    step_models = [perturbed(W, wm, rng) for _ in range(args.steps)]
    models = [inputs(m) for m in step_models]
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms, f_ms, a_ms, r_ms = [], [], [], []
    t0 = time.perf_counter()
    for m in models:
        tot, f, a, r = step(m)
        # config 4's largest families underflow FP64 (L = 0), so its total is
        # -Inf as in the reference (src/core.jl:15, :36); NaN is never valid
        if math.isnan(tot) or (not math.isfinite(tot) and args.config != 4):
            raise RuntimeError("non-finite log-likelihood in the timed region")
        f_ms.append(f)
        a_ms.append(a)
        r_ms.append(r)
        dev_ms.append(f + a + r)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if pg:
        pg.barrier()
    clk = clocks.stop()
    # parity of the timed workload: the last step's per-family log L (still in
    # the caller's buffer) against the oracle at that step's rates
    threads = os.cpu_count() or 1
    parity_per = per_b.copy()
    parity = parity_check(W, wl, step_models[-1], batch, parity_per, threads)
    dev_step = float(np.mean(dev_ms))
    wall_step = wall / args.steps
    nfw, ngr = W._native.C.c_int32(), W._native.C.c_int32()
    W._native.check(L.wg_batch_launches(batch.h, W._native.C.byref(nfw), W._native.C.byref(ngr)))
    n_launch = ngr.value
    if pg:
        t = torch.tensor([dev_step, wall_step], device=f"cuda:{local}", dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        dev_step, wall_step = float(t[0]), float(t[1]) * 1e3 / 1e3
    wall_step_ms = wall_step * 1e3
    NF = len(ccds)
    value = world * NF / (dev_step * 1e-3)
    e2e = world * NF / (wall_step_ms * 1e-3)
    NR = wm._struct.total_rows
    K = len(wm.order)
    h2d = 8 * (3 * NR + K + 3)  # slice tables, q, η and the two root-row constants
    # per-family log L plus one gradient vector per size class of the batch
    n_cls = batch.tables_layout()[0]
    d2h = 8 * NF + 8 * (3 * NR + K + 1) * n_cls
    # forward alone (for the gradient-cost ratio) and the plain one-family-per-launch path
    fwd_only = []
    for _ in range(5):
        batch.logpdf(perturbed(W, wm, rng))
        W._native.check(L.wg_ctx_timings(ctx.h, W._native.C.byref(fms), None, None))
        fwd_only.append(fms.value)
    fwd_only_ms = float(np.median(fwd_only))
    plain = None
    if not args.no_plain:
        pt = []
        for _ in range(2):
            m = perturbed(W, wm, rng)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            batch.logpdf_plain(m)
            pt.append(time.perf_counter() - t1)
        P = wm.rates.λ.size + wm.rates.μ.size + wm.rates.q.size + 1
        plain_ms = 1e3 * min(pt)
        plain = {"forward_ms": plain_ms, "fd_evaluations": 2 * P + 1,
                 "value": NF / ((2 * P + 1) * plain_ms * 1e-3), "unit": UNIT,
                 "what": "plain path (one family per launch) differentiated by central differences"}
    # The timed launch sequence overlaps each size class's adjoint with the
    # other classes' forwards, so its roofline is that of every launch of the
    # evaluation (k_fwd2 + k_adj2 + k_reduce2): their algorithmic FLOPs over
    # the evaluation's CUDA-event time.  The kernels' own rooflines come from
    # the same steps on a batch built with WG_ADJ_OVERLAP=0 (forward, then
    # adjoint, each timed on its own).
    prof = ncu_traffic() if NF == 5000 else None
    kflops = batch.flops_fwd + batch.flops_adj
    achieved = kflops / (dev_step * 1e-3) / 1e12
    peak_source = ("measured in this run: register-resident DFMA loop (wg_probe_fp64); "
                   "MEASURED_PEAKS.json has no FP64 figure")
    traffic_source = ("dram__bytes_read.sum + dram__bytes_write.sum over the kernels' launches of one evaluation, "
                      "one ncu capture of this workload (profiles/launches_cfg1_5000fam.txt"
                      + (f", commit {prof['commit']}" if prof and prof.get("commit") else "") + ")")
    roof = {"bound": "fp64", "kernel": "k_fwd2 + k_adj2 (every launch of the gradient evaluation, all levels and "
                                       "size classes)",
            "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": achieved / fp64_peak if fp64_peak else None,
            "traffic": (prof["adjoint"] + prof["forward"]) if prof else None, "traffic_source": traffic_source,
            "peak_source": peak_source, "algorithmic_flops_per_launch": kflops, "launch_ms": dev_step}
    os.environ["WG_ADJ_OVERLAP"] = "0"
    try:
        sep = W.Batch(wm, ccds, grad=True, ctx=ctx, checkpoint=args.checkpoint, persistent=args.persistent)
    finally:
        os.environ.pop("WG_ADJ_OVERLAP", None)
    for m in models[: args.warmup]:
        step(m, sep.h)
    sf, sa = [], []
    for m in models[: min(len(models), 300)]:
        _, f, a, r = step(m, sep.h)
        sf.append(f)
        sa.append(a)
    del sep
    fa = float(np.mean(sa)), float(np.mean(sf))
    adj_achieved = batch.flops_adj / (fa[0] * 1e-3) / 1e12
    kernels_alone = {
        "what": "the same steps with each size class's adjoint after every class's forward (WG_ADJ_OVERLAP=0)",
        "ms_per_step": fa[0] + fa[1], "forward_ms": fa[1], "adjoint_ms": fa[0],
        "adjoint_roofline": {"bound": "fp64", "kernel": "k_adj2 (all levels and size classes)",
                             "achieved": adj_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                             "frac": adj_achieved / fp64_peak if fp64_peak else None,
                             "traffic": prof["adjoint"] if prof else None, "traffic_source": traffic_source,
                             "algorithmic_flops_per_launch": batch.flops_adj, "launch_ms": fa[0]}}
    # the forward's own HBM figure: its algorithmic bytes over its own time
    fwd_hbm = {"kernel": "k_fwd2<true> (all levels and size classes)", "algorithmic_bytes": batch.bytes_fwd,
               "ms": fa[1], "gbs": batch.bytes_fwd / (fa[1] * 1e-3) / 1e9,
               "traffic": prof["forward"] if prof else None}
    line = {
        "metric": METRIC4 if args.config == 4 else METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload(NF, args.config),
                   "families": NF, "clades_mean": float(np.mean([c.n_clades for c in ccds])),
                   "clades_max": int(max(c.n_clades for c in ccds)),
                   "triples_mean": float(np.mean([c.n_triples for c in ccds])), "slices": NR,
                   "ctas": batch.n_groups, "device_bytes": batch.device_bytes,
                   "l2": "inputs exceed L2: sum programs + DP tables resident in HBM "
                         f"({batch.device_bytes / 1e9:.2f} GB > 129 MB)",
                   "parallelism": f"replicas x{world} (weak scaling)" if world > 1 else "single GPU",
                   "pack_seconds": pack_s, "generate_seconds": gen_s,
                   "tables": dict(zip(("size_classes", "classes_recomputing_tables", "full_bytes", "held_bytes"),
                                      (lambda t: (t[0], t[1], 8 * t[2], 8 * t[3]))(batch.tables_layout())))},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": wall_step_ms},
        "gpu_launches": n_launch * args.steps,
        "kernel_ms": {"forward": float(np.mean(f_ms)), "adjoint": float(np.mean(a_ms)),
                      "reduce": float(np.mean(r_ms)), "forward_only": fwd_only_ms},
        "grad_cost_vs_forward": dev_step / fwd_only_ms,
        "roofline": roof,
        "kernels_alone": kernels_alone,
        "forward_hbm": fwd_hbm,
        "plain_fd": plain,
        "speedup_vs_plain_fd": (value / plain["value"]) if plain else None,
        "clocks": clk,
        "parity": parity,
    }
    if args.config == 4 and not args.checkpoint:
        # the same steps on the per-level recomputation layout (what a batch
        # uses by itself once its tables exceed the device-memory budget)
        del batch
        ckb = W.Batch(wm, ccds, grad=True, ctx=ctx, checkpoint=True)
        for m in models[: args.warmup]:
            step(m, ckb.h)
        ck_ms = []
        for m in models:
            _, f, a, r = step(m, ckb.h)
            ck_ms.append(f + a + r)
        ckd = float(np.mean(ck_ms))
        t = ckb.tables_layout()
        line["checkpointed_layout"] = {
            "value": world * NF / (ckd * 1e-3), "unit": UNIT, "ms_per_step": ckd,
            "cost_vs_full_tables": ckd / dev_step, "device_bytes": ckb.device_bytes,
            "tables_held_bytes": 8 * t[3], "tables_full_bytes": 8 * t[2],
            "what": "every size class recomputes each height level's tables before the adjoint walks it"}
        ck_per = per_b.copy()
        line["checkpointed_layout"]["max_rel_logl_vs_full_tables"] = float(np.max(np.where(
            np.isneginf(ck_per) & np.isneginf(parity_per), 0.0,
            np.abs(ck_per - parity_per) / np.maximum(np.abs(parity_per), 1e-300))))
        del ckb
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        idx = pick_cpu_sample(W, wl, args.cpu_budget / 2, threads)
        v, times = cpu_reference(W, wl, idx, 1, 1, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{len(idx)} of {NF} families (random, seed 7), logL + gradient by "
                                          "forward-mode duals (chunk 12)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    if not parity["ok"]:
        print(f"parity broken: max_rel_logl {parity['max_rel_logl']:.3e} (bar {PARITY_LOGL:g}), "
              f"max_rel_grad {parity['max_rel_grad']:.3e} (bar {PARITY_GRAD:g})", file=sys.stderr, flush=True)
        sys.exit(3)


if __name__ == "__main__":
    main()
