#!/usr/bin/env python3
"""Throughput of the GB300 hot paths: chain-locus likelihood evaluations per
second, and L-mode surface grid points per second.

Default (--workload all): one JSON line whose headline is the stepwise
microsatellite workload -- 3 sampled populations (5-population tree), 100
SW loci x 30 copies per population, 64 heated chains, every chain-locus
fully evaluated per step -- with the other named workloads as sub-objects
under "configs", each with its own value, e2e, roofline, CPU baseline and
error against the plain FP64 form:
  config1_is       2 populations, 5 IS loci x (10+10) copies, 4 chains
  config2_hky      2 populations, 50 HKY loci x (20+20) x 1000 bp, 32 chains
                   (float-float pruning; the plain FP32 kernel beside it, an
                   edit-list leg and the per-call C-ABI latency)
  config4_mixed    200 HKY + 100 SW loci, U(4,60) copies x 3 populations,
                   128 chains x 8 runs
  config5_surface  G = 2^21 genealogy summaries, P = 2^16 points

  python bench.py [--steps K] [--warmup W] [--gpus N] [--workload all|sw|is|hky|mixed|surface|treeweight|popmig|updgen]
  python bench.py --impl reference ...   # the CPU restatement of the reference on every host core

value: inputs resident in HBM, device time (CUDA events on the context's
stream) of K steps, L2 flushed between steps.  e2e: the same steps through
the public C ABI from host buffers (genealogies copied host->device every
step, results copied back) on the host clock.  Multi-GPU: independent
replicas, one per rank, each on its own device.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "chain-locus likelihood evals/s"
SURF_METRIC = "L-mode grid points/s"
TW_METRIC = "genealogy weights (treeweight) per second"
UG_METRIC = "genealogy update proposals/s"
PM_METRIC = "2NM density terms (points x genealogies) per second"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def fp32_peak_tflops(sm_max_mhz):
    """Nominal FP32 FMA rate: SMs x 128 lanes x 2 FLOP x the SM clock the
    run's clock samples report as maximum (no measured figure exists)."""
    nsm = 152
    try:
        import torch

        nsm = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    mhz = sm_max_mhz or 2070.0
    return nsm * 128 * 2 * mhz * 1e6 / 1e12, "nominal: %d SMs x 128 FP32 lanes x 2 x %.0f MHz" % (nsm, mhz)


def profile_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu
    summaries (profiles/traffic.json, keyed "kernel/workload"), if captured."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get("%s/%s" % (kernel, workload))
    except Exception:
        return None


def rank_device():
    """This rank's GPU: LOCAL_RANK when the launcher leaves several devices
    visible (or none listed), else the one visible device."""
    local = int(os.environ.get("LOCAL_RANK", "0"))
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis is None:
        return local
    n = len([v for v in vis.split(",") if v.strip()])
    return local if n > 1 else 0
class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.5)  # let the sampler start before the timed region
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def aggregate(total_ms, units, steps, dist=None):
    """Replicas: every rank ran `units` per step on its own GPU; the job time
    is the slowest rank's and the value counts every rank's units."""
    world = 1
    if dist is not None:
        import torch

        world = dist.get_world_size()
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, units * steps * world / (total_ms / 1e3)


# ------------------------------------------------------------- workloads
def build_ctx(wl, api, device=0):
    ctx = api.Context(device)
    for spec in wl.loci:
        if spec[0] == "is":
            ctx.add_locus_is(spec[1])
        elif spec[0] == "hky":
            L = spec[1]
            ctx.add_locus_hky(L.seq, L.mult, L.totsites)
        else:
            ctx.add_locus_sw(spec[1], spec[2])
    ctx.set_chains(wl.nruns, wl.cpr)
    wl.upload(ctx)
    return ctx


def hky_algo_bytes(wl):
    """Algorithmic bytes of one full evaluation of every HKY chain-locus:
    per internal node and pattern 60 B (two daughter partials 32 B, their
    scales 8 B, the written partial 16 B and scale 4 B), per pattern 28 B at
    the root."""
    total = 0.0
    for spec in wl.loci:
        if spec[0] == "hky":
            n, S = spec[1].seq.shape
            total += (n - 1) * S * 60.0 + S * 28.0
    return total * wl.nchains


def sw_branch_flops(d):
    """FLOPs of one SW branch term: 30 for |d| < 2, else 30 + 6 (|d| +
    floor(sqrt(40 |d|))) -- the length of the reference's Miller recurrence."""
    d = np.abs(np.asarray(d))
    return np.where(d < 2, 30.0, 30.0 + 6.0 * (d + np.floor(np.sqrt(40.0 * d))))


def sw_algo_flops(wl, max_chains=None):
    """FLOPs of one evaluation of every SW chain-locus (a sample of chains,
    scaled, when max_chains is given)."""
    ch = np.arange(wl.nchains)
    if max_chains is not None and wl.nchains > max_chains:
        ch = np.linspace(0, wl.nchains - 1, max_chains).astype(int)
    tot = 0.0
    for li, spec in enumerate(wl.loci):
        if spec[0] != "sw":
            continue
        for c in ch:
            g, A = wl.tree(int(c), li), np.asarray(wl.allele(int(c), li))
            keep = g.down >= 0
            tot += float(sw_branch_flops(A[keep] - A[g.down[keep]]).sum())
    return tot * wl.nchains / len(ch)


def is_algo_bytes(wl):
    """Per evaluation: (2n-1) x 20 B of topology and time, S x ceil(n/32) x 4 B
    of site bit sets, 8 B out."""
    total = 0.0
    for spec in wl.loci:
        if spec[0] == "is":
            n, S = spec[1].shape
            total += (2 * n - 1) * 20.0 + S * math.ceil(n / 32) * 4.0 + 8.0
    return total * wl.nchains


def oracle_packs(wl, limit):
    """An even sample of the workload's chain-loci, packed per model kind for
    the oracle's batched C entry points."""
    from oracle import pyoracle as O

    ci, li = wl.pairs()
    # an even sample of `limit` pairs; a workload with fewer pairs is cycled
    # through until the batch holds `limit` (thread start-up per call stays
    # small against the work)
    idx = np.linspace(0, len(ci) - 1, limit).astype(int) if limit < len(ci) else np.resize(np.arange(len(ci)), limit)
    by = {}
    for k in idx:
        c, l = int(ci[k]), int(li[k])
        spec = wl.loci[l]
        data = spec[1] if spec[0] in ("is", "hky") else wl.allele(c, l)
        by.setdefault(spec[0], []).append((spec[0], wl.tree(c, l), float(wl.u[c, l]), float(wl.par[c, l]), data))
    return [O.PackedItems(v) for v in by.values()]


def cpu_rate(packs, seconds, threads):
    """Chain-locus evaluations per second of the oracle's batched C path on
    `threads` host threads, repeated for about `seconds`."""
    n, t = 0, 0.0
    while t < seconds or n == 0:
        for p in packs:
            t0 = time.perf_counter()
            p.run(threads)
            t += time.perf_counter() - t0
            n += p.nitems
    return n / t, n, t


CPU_SAMPLE = 8192  # chain-loci per batched oracle call, in this line and in the reference arm


def cpu_baseline(wl, seconds, limit=CPU_SAMPLE):
    cores = os.cpu_count() or 1
    packs = oracle_packs(wl, limit)
    v, n, t = cpu_rate(packs, seconds, cores)
    return {"value": round(v, 1), "unit": "evals/s", "cores": cores, "kind": "port",
            "sample": "%d chain-locus evaluations in %.1f s over an even %d-pair sample of the workload's %d "
                      "pairs, the oracle's batched C path on %d threads"
                      % (n, t, sum(p.nitems for p in packs), wl.nchains * wl.nloci, cores)}


def dirty_edits(wl, rng, ndirty=4):
    """Four internal (non-root) nodes of every chain-locus moved down in time,
    one after another, each inside the bounds its daughters and parent set
    at that moment, as a genealogy update leaves them: the packed arrays with
    the new times, the edit lists [pairs][4] (the moved nodes: their
    daughters' branches changed) and how many nodes each evaluation
    recomputes (the moved nodes and their ancestors)."""
    pci, pli, up0, up1, down, tm = wl.packed()
    tm = tm.copy()
    ci, li = wl.pairs()
    edits = np.full((len(ci), 4), -1, np.int32)
    recomputed = 0
    off = 0
    for k in range(len(ci)):
        spec = wl.loci[int(li[k])]
        n = spec[1].seq.shape[0] if spec[0] == "hky" else (spec[1] if spec[0] == "sw" else spec[1].shape[0])
        nl = 2 * n - 1
        u0, u1, dn, t = up0[off:off + nl], up1[off:off + nl], down[off:off + nl], tm[off:off + nl]
        cand = [j for j in range(n, nl) if dn[j] >= 0]
        pick = rng.choice(cand, size=min(ndirty, len(cand)), replace=False)
        fresh = set()
        for j in pick:
            lo = max(t[u0[j]], t[u1[j]])
            t[j] = 0.5 * (lo + t[j])   # below its old time, above both daughters
            x = int(j)
            while x >= 0 and x not in fresh:
                fresh.add(x)
                x = int(dn[x])
        edits[k, :len(pick)] = pick
        recomputed += len(fresh)
        off += nl
    return (pci, pli, up0, up1, down, tm), edits, recomputed / len(ci)


def kdelta(k0, k1):
    n = k1[0] - k0[0]
    return n, (k1[1] - k0[1]) / max(n, 1)


def measure_lik(args, api, wl, steps, dist=None, device=0, hky_legs=False):
    """One likelihood workload: every chain-locus fully evaluated per step
    (the batched form of changet_RY1's all-locus re-likelihood)."""
    world = dist.get_world_size() if dist else 1
    rank = dist.get_rank() if dist else 0
    ctx = build_ctx(wl, api, device)
    ci, li = wl.pairs()
    u, par = wl.u.ravel(), wl.par.ravel()
    units = len(ci)
    prec = api.PREC_FAST
    batch = ctx.batch_create(ci, li, u, par, precision=prec)
    for _ in range(args.warmup):
        batch.run(use_graph=True)
    tuned = batch.autotune(reps=5)
    batch.run(use_graph=True)
    ctx.synchronize()
    res_fast, st_fast = batch.results()
    kinds = {s[0] for s in wl.loci}

    # ---------------- timed region: resident inputs, L2 flushed between steps
    kstat = {k: None for k in (api.K_IS, api.K_HKY_FAST, api.K_SW_FAST)}
    ctx.set_profiling(True)
    n0 = ctx.launch_count()
    for k in kstat:
        kstat[k] = ctx.kernel_stats(k)
    times = []
    if dist:
        dist.barrier()
    with Clocks(device) as clk:
        for _ in range(steps):
            ctx.flush_l2()
            ctx.timer_begin()
            batch.run(use_graph=False)
            times.append(ctx.timer_end())
    n_launch = ctx.launch_count() - n0
    per = {k: kdelta(kstat[k], ctx.kernel_stats(k)) for k in kstat}
    ctx.set_profiling(False)
    total_ms, value = aggregate(float(sum(times)), units, steps, dist)
    clocks = clk.summary()

    # ---------------- roofline of the dominant kernel
    hbm, _, src = measured_peaks()
    fp32, fp32_src = fp32_peak_tflops(clocks["sm_max_mhz"] if clocks else None)
    roof, composite = None, None
    if "hky" in kinds:
        nl_, ms = per[api.K_HKY_FAST]
        b = hky_algo_bytes(wl)
        ach = b / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        roof = {"kernel": "k_hky_fast (float-float)", "bound": "hbm", "achieved": round(ach, 1), "peak": hbm,
                "unit": "GB/s", "frac": round(ach / hbm, 4), "peak_source": src + " (of %s)" % src,
                "traffic": profile_traffic("k_hky_fast", wl.name), "algorithmic_bytes_per_launch": b,
                "avg_launch_ms": round(ms, 5), "launches": nl_}
    if "sw" in kinds:
        nl_, ms = per[api.K_SW_FAST]
        fl = sw_algo_flops(wl, max_chains=16)
        ach = fl / (ms / 1e3) / 1e12 if ms > 0 else 0.0
        sroof = {"kernel": "k_sw_fast", "bound": "fp32", "achieved": round(ach, 3), "peak": round(fp32, 1),
                 "unit": "TFLOP/s", "frac": round(ach / fp32, 4), "peak_source": fp32_src,
                 "traffic": profile_traffic("k_sw_fast", wl.name), "algorithmic_flops_per_launch": fl,
                 "avg_launch_ms": round(ms, 5), "launches": nl_,
                 "note": "algorithmic FLOPs of the reference's Bessel terms; the kernel issues them in "
                         "float-float, about ten FP32 instructions each"}
        if roof is None:
            roof = sroof
        else:
            # batched uneven workload: the per-kind bounds added up against the step time
            hb = hky_algo_bytes(wl) / (hbm * 1e9) + fl / (fp32 * 1e12)
            composite = {"time_bound_ms": round(1e3 * hb, 4), "step_ms": round(total_ms / steps, 4),
                         "frac": round(1e3 * hb / (total_ms / steps), 4),
                         "note": "HKY algorithmic bytes at the measured HBM rate plus SW algorithmic FLOPs at "
                                 "the nominal FP32 rate, over the measured step time"}
            roof["sw"] = sroof
    if roof is None:
        nl_, ms = per[api.K_IS]
        b = is_algo_bytes(wl)
        ach = b / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        roof = {"kernel": "k_is", "bound": "hbm", "achieved": round(ach, 2), "peak": hbm, "unit": "GB/s",
                "frac": round(ach / hbm, 6), "peak_source": src, "traffic": profile_traffic("k_is", wl.name),
                "algorithmic_bytes_per_launch": b, "avg_launch_ms": round(ms, 5), "launches": nl_,
                "note": "latency-bound: %d chain-loci per launch" % units}

    # ---------------- plain FP64 per-chain form on the same GPU
    def form(precision, reps):
        b = ctx.batch_create(ci, li, u, par, precision=precision)
        for _ in range(2):
            b.run(use_graph=False)
        tt = []
        for _ in range(reps):
            ctx.flush_l2()
            ctx.timer_begin()
            b.run(use_graph=False)
            tt.append(ctx.timer_end())
        r, _ = b.results()
        b.destroy()
        return r, units / (statistics.median(tt) / 1e3)

    res64, v64 = form(api.PREC_FP64, max(3, min(steps, 10)))
    ok = (st_fast == 0)
    err = np.abs(res_fast[ok] - res64[ok])
    out = {
        "value": round(value, 1), "unit": "evals/s", "ms_per_step": round(total_ms / steps, 5), "steps": steps,
        "config": {"workload": wl.describe, "global_batch": units * world, "chain_loci_per_step": units,
                   "l2": "flushed between timed steps",
                   "precision": "float-float pruning / Bessel terms, FP64 sums" if kinds & {"hky", "sw"}
                   else "FP64"},
        "roofline": roof,
        "fp64_form": {"value": round(v64, 1), "unit": "evals/s", "speedup": round(value / world / v64, 2)},
        "error_vs_fp64": {"max_abs": float(err.max()) if len(err) else None,
                          "median_abs": float(np.median(err)) if len(err) else None,
                          "max_rel": float((err / np.abs(res64[ok])).max()) if len(err) else None},
        "gpu_launches": int(n_launch), "clocks": clocks,
        "autotune": {"hky_variant": tuned[0], "sw_variant": tuned[1]},
    }
    if composite:
        out["roofline_composite"] = composite
    if "hky" in kinds:
        # the plain FP32 pruning kernel on the same batch: its speed and error
        res32, v32 = form(api.PREC_FP32, max(3, min(steps, 20)))
        e32 = np.abs(res32[ok] - res64[ok])
        out["fp32_form"] = {"value": round(v32, 1), "unit": "evals/s",
                            "error_vs_fp64": {"max_abs": float(e32.max()), "median_abs": float(np.median(e32))},
                            "note": "FP32 partials: a pattern's rounding repeats in each of its sites"}
        batch.run(use_graph=False)  # the float-float partials are the committed ones below
        ctx.synchronize()

    # ---------------- e2e through the C ABI from host buffers
    # every step re-times every genealogy (changet_RY1's pattern: topology
    # kept, node times rescaled) and re-evaluates every chain-locus
    pci, pli, up0, up1, down, tm = wl.packed()
    scaled = np.where(tm > 0, tm * (1.0 + 1e-6), tm)
    nodes = len(up0)
    # FP64 time per node in, a result and a status per chain-locus out (the
    # lengths are summed on the device; the request list repeats, so the
    # staged one is kept)
    h2d = nodes * 8
    d2h = units * (8 + 4)
    assert np.array_equal(pci, ci) and np.array_equal(pli, li)
    e2e_t = []
    for s in range(args.warmup + min(steps, 100)):
        tms = scaled if s % 2 else tm
        t0 = time.perf_counter()
        ctx.eval_times(ci, li, tms, u, par, precision=prec)
        t1 = time.perf_counter()
        if s >= args.warmup:
            e2e_t.append(t1 - t0)
    # the same step as two calls (ima_gpu_set_times, ima_gpu_eval), and where
    # its time goes: the upload, and an evaluation with nothing to upload
    two_t, set_t, fl_t, ev_t = [], [], [], []
    for s in range(args.warmup + min(steps, 50)):
        tms = scaled if s % 2 else tm
        t0 = time.perf_counter()
        ctx.set_times(ci, li, tms)
        t1 = time.perf_counter()
        ctx.eval(ci, li, u, par, precision=prec)
        t2 = time.perf_counter()
        ctx.set_times(ci, li, tm if s % 2 else scaled)
        t3 = time.perf_counter()
        ctx.synchronize()
        t4 = time.perf_counter()
        ctx.eval(ci, li, u, par, precision=prec)
        t5 = time.perf_counter()
        if s >= args.warmup:
            two_t.append(t2 - t0)
            set_t.append(t1 - t0)
            fl_t.append(t4 - t3)
            ev_t.append(t5 - t4)
    # device time of the step's kernels (events around each launch, in a
    # loop of its own: recording them costs host time)
    ctx.set_profiling(True)
    kk = [k for k in (api.K_TIMES, api.K_IS, api.K_HKY_FAST, api.K_SW_FAST)]
    k0 = {k: ctx.kernel_stats(k) for k in kk}
    nprof = 20
    for s in range(nprof):
        ctx.eval_times(ci, li, scaled if s % 2 else tm, u, par, precision=prec)
    kms = {k: (ctx.kernel_stats(k)[1] - k0[k][1]) / nprof for k in kk}
    ctx.set_profiling(False)
    e2e = units * world / statistics.median(e2e_t)
    out["e2e"] = {"value": round(e2e, 1), "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
                  "d2h_bytes_per_step": int(d2h),
                  "ms_per_step": round(1e3 * statistics.median(e2e_t), 4),
                  "api": "ima_gpu_eval_times",
                  "ms_upload_kernels": round(kms[api.K_TIMES], 4),
                  "ms_evaluation_kernels": round(sum(kms[k] for k in kk[1:]), 4),
                  "note": "every step re-times every genealogy (topology kept, as changet_RY1 moves) and "
                          "evaluates every chain-locus in one call: the device reads the step's FP64 times "
                          "from the caller's buffer, makes their float-float form and the tree lengths, "
                          "evaluates, and the results come back",
                  "two_calls": {"value": round(units * world / statistics.median(two_t), 1),
                                "ms_per_step": round(1e3 * statistics.median(two_t), 4),
                                "ms_set_times": round(1e3 * statistics.median(set_t), 4),
                                "ms_upload_wait": round(1e3 * statistics.median(fl_t), 4),
                                "ms_eval_resident": round(1e3 * statistics.median(ev_t), 4),
                                "note": "ima_gpu_set_times (one copy from the caller's buffer) then "
                                        "ima_gpu_eval"}}
    ctx.set_genealogies(pci, pli, up0, up1, down, tm)

    if hky_legs:
        out["edit_lists"] = edit_list_leg(ctx, api, wl, ci, li, u, par, steps)
        out["per_call"] = per_call_leg(ctx, api, wl)

    # ---------------- MC3 swap sweeps of every run on the resident sums
    ctx.commit(ci, li, np.ones(units, np.uint8))
    ctx.set_probg(np.zeros(wl.nchains))
    ctx.setheat(0.9, 0.8, 1)
    tries = max(1, wl.cpr // 10)
    for _ in range(3):
        ctx.swapchains(tries, True, seed=7)
    ctx.synchronize()
    ctx.timer_begin()
    nsw = 200
    for _ in range(nsw):
        ctx.swapchains(tries, True, seed=7)
    sw_ms = ctx.timer_end() / nsw
    out["swaps"] = {"runs": wl.nruns, "chains_per_run": wl.cpr, "swaptries": tries,
                    "ms_per_sweep": round(sw_ms, 5),
                    "attempts_per_s": round(wl.nruns * tries / (sw_ms / 1e3), 1)}
    if wl.nruns > 1:
        out["sweep"] = sweep_leg(ctx, api, ci, li, u, par, prec, tuned, tries, steps)
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    batch.destroy()
    ctx.close()
    return out


def sweep_leg(ctx, api, ci, li, u, par, prec, tuned, tries, steps):
    """One MC3 sweep of every run: every chain-locus evaluated, committed,
    then each run's swap attempts -- as one graph launch
    (ima_gpu_batch_sweep) and as separate launches, device time per sweep."""
    b = ctx.batch_create(ci, li, u, par, precision=prec)
    b.set_variants(*tuned)
    k = max(3, min(steps, 30))

    def timed(graph):
        for _ in range(3):
            b.sweep(tries, seed=5, use_graph=graph)
        ctx.synchronize()
        n0 = ctx.launch_count()
        ctx.timer_begin()
        for _ in range(k):
            b.sweep(tries, seed=5, use_graph=graph)
        ms = ctx.timer_end() / k
        return ms, (ctx.launch_count() - n0) / k

    ms_g, kern = timed(True)
    ms_l, _ = timed(False)
    b.destroy()
    return {"ms_per_sweep_graph": round(ms_g, 4), "ms_per_sweep_launches": round(ms_l, 4),
            "kernels_per_sweep": kern, "graph_launches_per_sweep": 1,
            "chain_locus_evals_per_s": round(len(ci) / (ms_g / 1e3), 1),
            "note": "every (run, chain, locus) evaluated, accepted and committed, then swapchains of every run "
                    "(%d attempts, Philox stream) -- all kernels of a sweep in one CUDA graph" % tries}


def edit_list_leg(ctx, api, wl, ci, li, u, par, steps):
    """The genealogy-update case: four internal nodes of every chain-locus
    moved, each evaluation given those four as its edit list (e1..e4), so
    only they and their ancestors are recomputed (device time, L2 flushed)."""
    rng = np.random.default_rng(99)
    packed, edits, nrec = dirty_edits(wl, rng)
    # the partials of the unmoved genealogies, committed: the clean nodes'
    # partials the edit-list evaluations start from
    ctx.set_genealogies(*wl.packed())
    full = ctx.batch_create(ci, li, u, par, precision=api.PREC_FAST)
    full.run(use_graph=False)
    ctx.commit(ci, li, np.ones(len(ci), np.uint8))
    ctx.set_times(packed[0], packed[1], packed[5])
    b = ctx.batch_create(ci, li, u, par, edits=edits, precision=api.PREC_FAST)
    for _ in range(3):
        b.run(use_graph=True)
    tt = []
    for _ in range(max(3, min(steps, 200))):
        ctx.flush_l2()
        ctx.timer_begin()
        b.run(use_graph=False)
        tt.append(ctx.timer_end())
    r_ff, _ = b.results()
    b.destroy()
    # the same genealogies evaluated in full: the float-float form gives the
    # same bits, the FP64 form the error
    full.run(use_graph=False)
    r_full, _ = full.results()
    full.destroy()
    b64 = ctx.batch_create(ci, li, u, par, precision=api.PREC_FP64)
    b64.run(use_graph=False)
    r64, _ = b64.results()
    b64.destroy()
    ms = statistics.median(tt)
    return {"value": round(len(ci) / (ms / 1e3), 1), "unit": "evals/s", "ms_per_step": round(ms, 5),
            "dirty_nodes_per_eval": 4, "recomputed_nodes_per_eval": round(nrec, 2),
            "same_bits_as_full_evaluation": bool(np.array_equal(r_ff, r_full)),
            "error_vs_fp64_max_abs": float(np.abs(r_ff - r64).max())}


def per_call_leg(ctx, api, wl, calls=2000):
    """The per-call drop-in (ima_gpu_likelihoodHKY, one chain-locus per call,
    result copied back and synchronised) against one host core running the
    oracle's C likelihood on the same chain-loci."""
    from oracle import pyoracle as O

    nl = wl.nloci
    lat = []
    for k in range(calls + 50):
        l = k % nl
        t0 = time.perf_counter()
        ctx.likelihoodHKY(0, l, float(wl.u[0, l]), float(wl.par[0, l]), -1, -1, -1, -1)
        if k >= 50:
            lat.append(time.perf_counter() - t0)
    lat_up = []
    for k in range(200):
        l = k % nl
        g = wl.tree(0, l)
        t0 = time.perf_counter()
        ctx.set_genealogy(0, l, g)
        ctx.likelihoodHKY(0, l, float(wl.u[0, l]), float(wl.par[0, l]), -1, -1, -1, -1)
        lat_up.append(time.perf_counter() - t0)
    # the kernel's own time per call (CUDA events around each launch, in a
    # separate loop: recording them costs host time)
    ctx.set_profiling(True)
    k0 = ctx.kernel_stats(api.K_HKY_FAST)
    for k in range(200):
        l = k % nl
        ctx.likelihoodHKY(0, l, float(wl.u[0, l]), float(wl.par[0, l]), -1, -1, -1, -1)
    nk, kms = kdelta(k0, ctx.kernel_stats(api.K_HKY_FAST))
    ctx.set_profiling(False)
    items = [("hky", wl.tree(0, l), float(wl.u[0, l]), float(wl.par[0, l]), wl.loci[l][1]) for l in range(nl)]
    pack = O.PackedItems(items)
    v, n, t = cpu_rate([pack], 1.0, 1)
    return {"us_per_call": round(1e6 * statistics.median(lat), 2),
            "kernel_us_per_call": round(1e3 * kms, 2),
            "us_per_call_with_genealogy_upload": round(1e6 * statistics.median(lat_up), 2),
            "cpu_us_per_eval_1core": round(1e6 / v, 2),
            "note": "one chain-locus (20+20 copies, 1000 bp) per call; the genealogy stays resident unless "
                    "uploaded"}


def run_likelihood_line(args, name):
    """--workload is|hky|sw|mixed alone."""
    from ima2p_gb300 import api, workloads

    dist = init_dist()
    wl = workloads.make(name)
    steps = args.steps if name != "mixed" else min(args.steps, 50)
    out = measure_lik(args, api, wl, steps, dist, rank_device(), hky_legs=(name == "hky"))
    emit(args, out, METRIC, dist)


def init_dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None
    import torch.distributed as dist_mod
    dist_mod.init_process_group("gloo")
    return dist_mod


def emit(args, sub, metric, dist, extra=None):
    """Print the contract's JSON line (rank 0) around a measurement dict."""
    world = dist.get_world_size() if dist else 1
    out = {"metric": metric, "value": sub["value"], "unit": sub["unit"], "n_gpus": world,
           "steps": sub.get("steps", args.steps), "warmup": args.warmup, "ms_per_step": sub["ms_per_step"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": sub.get("dtype", "ff32 (float-float on FP32) + fp64 sums"),
           "data": "synthetic (seeded IM coalescent genealogies and simulated data, shapes of the named config)"}
    out["config"] = dict(sub["config"], parallelism="replicas%d" % world)
    for k, v in sub.items():
        if k not in out and k not in ("config", "steps"):
            out[k] = v
    if extra:
        out.update(extra)
    if (dist.get_rank() if dist else 0) == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()
# ------------------------------------------------------------------ surface
def surface_inputs(args):
    from ima2p_gb300 import synth

    rng = np.random.default_rng(1005)
    G, P = 1 << args.surface_log2g, 1 << args.surface_log2p
    rows, lognorm, off = synth.surface_stats(rng, G, 5, 8, 2)
    pts = synth.surface_points(rng, P)
    return G, P, rows, lognorm, pts


def surface_cpu(rows, lognorm, pts, seconds, threads):
    """The oracle's exact jointp (C) on `threads` host threads over the first
    points, as many as about `seconds` take; points per second."""
    from oracle import pyoracle as O

    n = max(threads, 1)
    t = 0.0
    done = 0
    while True:
        k = min(n, len(pts) - done) if done < len(pts) else n
        sub = pts[done % len(pts): done % len(pts) + k]
        t0 = time.perf_counter()
        O.jointp_batch(rows, 5, 8, 3, sub, 0, lognorm, threads)
        t += time.perf_counter() - t0
        done += len(sub)
        if t >= seconds:
            return done / t, done, t
        # grow the next batch toward the time left
        n = max(threads, int(done / t * max(0.5, seconds - t)))


def measure_surface(args, api, steps, extended=True, device=0):
    """Config 5: G = 2^21 genealogy summaries (K = 48 row width), P = 2^16
    points; the tensor-core screen with exact float-float refinement."""
    G, P, rows, lognorm, pts = surface_inputs(args)
    ctx = api.Context(device)
    ctx.add_locus_sw(2, 1)
    ctx.set_chains(1, 1)
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    method = api.SURF_TC if args.surface_method == "tc" else api.SURF_FAST
    kind = api.K_SURF_TC if method == api.SURF_TC else api.K_SURF_FAST
    for _ in range(args.warmup):
        q, ess = ctx.surface_eval(pts, 0, method)
    ctx.set_profiling(True)
    k0 = ctx.kernel_stats(kind)
    n0 = ctx.launch_count()
    wall = []
    with Clocks(device) as clk:
        for _ in range(steps):
            ctx.flush_l2()
            t0 = time.perf_counter()
            q, ess = ctx.surface_eval(pts, 0, method)
            wall.append(time.perf_counter() - t0)
    k1 = ctx.kernel_stats(kind)
    n_timed = ctx.launch_count() - n0
    ctx.set_profiling(False)
    dev_ms = (k1[1] - k0[1]) / max(1, k1[0] - k0[0])
    value = P / (dev_ms / 1e3)
    e2e = P / statistics.median(wall)
    retaken = ctx.surface_retaken() if method == api.SURF_TC else 0
    # the same points again: the screens give the same bits every call
    q_again, _ = ctx.surface_eval(pts, 0, method)
    # plain FP64 CUDA-core form on a subset of points, extrapolated per point
    sub = pts[:512]
    ctx.surface_eval(sub, 0, api.SURF_FP64)
    t0 = time.perf_counter()
    q64, e64 = ctx.surface_eval(sub, 0, api.SURF_FP64)
    v64 = len(sub) / (time.perf_counter() - t0)
    rel = np.abs(q[:512] - q64) / np.abs(q64)
    flops = 2.0 * G * 26  # the contraction's algorithmic FLOPs per point
    hbm, bf16, src = measured_peaks()
    out = {
        "value": round(value, 1), "unit": "points/s", "ms_per_step": round(dev_ms, 4), "steps": steps,
        "dtype": "bf16 split (3 products, FP32 accumulate) screen + float-float exact terms + FP64 sums",
        "config": {"workload": "config5-surface: G=2^%d genealogy summaries, K=48 row width "
                               "(5 theta, 8 m), P=2^%d points, full model"
                               % (args.surface_log2g, args.surface_log2p), "global_batch": P,
                   "l2": "flushed between timed steps"},
        "e2e": {"value": round(e2e, 1), "unit": "points/s", "h2d_bytes_per_step": int(P * 13 * 8),
                "d2h_bytes_per_step": int(P * 16)},
        "screen": "tcgen05 split-bf16 GEMM (3 products) into TMEM + exact float-float refinement"
                  if method == api.SURF_TC else "FP32 CUDA-core FMA + exact float-float refinement",
        "roofline": {"kernel": "surface (prep + screen + merge)", "bound": "tensor",
                     "achieved": round(flops * P / (dev_ms / 1e3) / 1e12, 2), "peak": bf16,
                     "unit": "TFLOP/s", "frac": round(flops * P / (dev_ms / 1e3) / 1e12 / bf16, 5),
                     "peak_source": src, "traffic": None,
                     "note": "achieved counts the algorithmic 2*G*26 FLOP per point; the split-bf16 "
                             "screen issues 3 x 2*G*32 on the tensor pipe"},
        "fp64_form": {"value": round(v64, 1), "unit": "points/s", "speedup": round(value / v64, 2),
                      "sample": "512 points"},
        "error_vs_fp64": {"max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
                          "ess_max_rel": float(np.max(np.abs(ess[:512] - e64) / e64))},
        "repeat_bitwise": bool(np.array_equal(q_again, q)),
        "points_retaken": int(retaken),
        "gpu_launches": int(n_timed), "clocks": clk.summary(),
    }
    cores = os.cpu_count() or 1
    v_cpu, n_cpu, t_cpu = surface_cpu(rows, lognorm, pts, args.cpu_seconds, cores)
    out["cpu_baseline"] = {"value": round(v_cpu, 3), "unit": "points/s", "cores": cores, "kind": "port",
                           "sample": "%d points in %.1f s, the oracle's exact jointp over all %d genealogies "
                                     "on %d threads" % (n_cpu, t_cpu, G, cores)}
    if extended:
        # 1-D marginal densities (fillvec): 13 parameters x 1000 grid points,
        # each a sum over all G genealogies, FP64 as the reference sums it
        from oracle import pyoracle as O
        pmin, pmax = np.zeros(13), np.array([20.0] * 5 + [2.0] * 8)
        ctx.fillvec(pmin, pmax, 1000)
        ctx.set_profiling(True)
        m0 = ctx.kernel_stats(api.K_MARGIN)
        t0 = time.perf_counter()
        xs_m, ys_m = ctx.fillvec(pmin, pmax, 1000)
        wall_m = time.perf_counter() - t0
        m1 = ctx.kernel_stats(api.K_MARGIN)
        ctx.set_profiling(False)
        dev_m = (m1[1] - m0[1]) / max(1, m1[0] - m0[0])
        t0 = time.perf_counter()
        nm_cpu = 0
        while time.perf_counter() - t0 < max(0.5, args.cpu_seconds / 4) or nm_cpu == 0:
            O.margincalc(rows, 5, 8, nm_cpu % 13, xs_m[nm_cpu % 13, (nm_cpu * 37) % 1000])
            nm_cpu += 1
        cpu_m = nm_cpu / (time.perf_counter() - t0)
        out["marginals"] = {"grid_points": 13000, "ms_device": round(dev_m, 3), "ms_e2e": round(1e3 * wall_m, 3),
                            "points_per_s": round(13000 / (dev_m / 1e3), 1),
                            "terms_per_s": round(13000 * G / (dev_m / 1e3), 1),
                            "cpu_points_per_s_1core": round(cpu_m, 3)}
        if not args.no_peak_search:
            # the L-mode peak search (modelloop): differential evolution with
            # 100 x 13 trial points per generation, one batched surface
            # evaluation per generation
            upper = [20.0] * 5 + [2.0] * 8
            t0 = time.perf_counter()
            best, ess_pk, gens, runs, _ = ctx.modelloop(upper, 0, seed=1234, multiplier=100, method=method)
            dt = time.perf_counter() - t0
            evals = (gens + runs) * 1300
            out["peak_search"] = {"generations": gens, "restarts": runs, "seconds": round(dt, 3),
                                  "ms_per_generation": round(1e3 * dt / (gens + runs), 4),
                                  "points_per_s": round(evals / dt, 1), "population": 1300,
                                  "peak_neg_log_density": float(best[-1]), "ess": ess_pk,
                                  "cpu_seconds_per_generation_all_cores": round(1300 / v_cpu, 1)}
    ctx.close()
    return out


def run_surface(args):
    from ima2p_gb300 import api

    out = measure_surface(args, api, args.steps, True, rank_device())
    emit(args, out, SURF_METRIC, None)


def tw_workload(nloci=300, nchains=128, nbase=60, seed=1011):
    """Config-4-shaped genealogy-weight workload: 3 populations
    ((0,1):3,2):4, per-population samples U(4,60), IM genealogies with their
    population labels and migrations (theta 2-6, m 0.3); nbase distinct loci
    cycled over nloci, the same genealogies in every chain (one split-time
    row).  Returns (popmodel, packed inputs, gen_locus, gen_tv, hval,
    samppop, tvals, labelled base genealogies, base index per genealogy)."""
    from ima2p_gb300 import api, popmodel, synth
    rng = np.random.default_rng(seed)
    pm = popmodel.build("((0,1):3,2):4", 3)
    tv = np.array([[0.6, 1.4]])
    base, samp = [], []
    for b in range(nbase):
        s = [int(v) for v in rng.integers(4, 61, 3)]
        theta = list(rng.uniform(2.0, 6.0, 5))
        base.append(synth.sim_im_labeled(rng, s, theta, 0.3, [(0.6, 0, 1, 3), (1.4, 3, 2, 4)]))
        samp.append(s)
    bp = [api.pack_labelled([g]) for g in base]
    seq = np.tile(np.arange(nloci) % nbase, nchains)
    nn = np.array([len(bp[b][1]) for b in range(nbase)])
    nm = np.array([int(bp[b][4][-1]) for b in range(nbase)])
    node_off = np.zeros(len(seq) + 1, np.int32)
    node_off[1:] = np.cumsum(nn[seq])
    up0 = np.concatenate([bp[b][1] for b in seq])
    time_ = np.concatenate([bp[b][2] for b in seq])
    pop = np.concatenate([bp[b][3] for b in seq])
    mbase = np.concatenate([[0], np.cumsum(nm[seq])])
    mig_off = np.concatenate([bp[b][4][:-1] + mbase[i] for i, b in enumerate(seq)] + [[mbase[-1]]]).astype(np.int32)
    mig_t = np.concatenate([bp[b][5] for b in seq])
    mig_p = np.concatenate([bp[b][6] for b in seq]).astype(np.int32)
    packed = (node_off, up0, time_, pop, mig_off, mig_t, mig_p)
    gen_locus = np.tile(np.arange(nloci), nchains).astype(np.int32)
    gen_tv = np.zeros(len(seq), np.int32)
    hval = np.ones(nloci)
    samppop = np.array([samp[li % nbase] for li in range(nloci)], np.int32)
    return pm, packed, gen_locus, gen_tv, hval, samppop, tv, base, seq


def run_treeweight(args):
    """treeweight for every chain-locus of a config-4-sized chain set (128
    chains x 300 loci) and the per-chain p(G) integrals: one step = the
    weights of all genealogies and all chains' integrals, as a split-time
    update (changet) needs them."""
    from ima2p_gb300 import api
    from oracle import pyoracle as O
    nloci, nch = 300, 128
    pm, packed, gl, gt, hval, samp, tv, base, seq = tw_workload(nloci, nch)
    ngen = len(gl)
    ctx = api.Context(0)
    nth, nmg = len(pm.th_cells), len(pm.mg_cells)
    ctx.set_popmodel(pm, 15.0, 0.0, 2.0, 0.0, 1.0)
    goff = (np.arange(nch + 1) * nloci).astype(np.int32)
    for _ in range(args.warmup):
        w = ctx.treeweight(packed, gl, gt, hval, samp, tv)
        probg, q, m, _ = ctx.tree_prob(goff)
    ctx.set_profiling(True)
    k0, p0 = ctx.kernel_stats(api.K_TREEWEIGHT), ctx.kernel_stats(api.K_TREE_PROB)
    n0 = ctx.launch_count()
    wall = []
    with Clocks(0) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            t0 = time.perf_counter()
            w = ctx.treeweight(packed, gl, gt, hval, samp, tv)
            probg, q, m, _ = ctx.tree_prob(goff)
            wall.append(time.perf_counter() - t0)
    k1, p1 = ctx.kernel_stats(api.K_TREEWEIGHT), ctx.kernel_stats(api.K_TREE_PROB)
    n_timed = ctx.launch_count() - n0
    ctx.set_profiling(False)
    nk = max(1, k1[0] - k0[0])
    tw_ms = (k1[1] - k0[1]) / nk
    tp_ms = (p1[1] - p0[1]) / max(1, p1[0] - p0[0])
    dev_ms = tw_ms + tp_ms
    value = ngen / (dev_ms / 1e3)
    e2e = ngen / statistics.median(wall)
    node_off, up0, time_, pop, mig_off, mig_t, mig_p = packed
    N, Nm = len(up0), len(mig_t)
    T, M = pm.T, pm.M
    h2d = (ngen + 1) * 4 + N * 20 + 4 + Nm * 12 + ngen * 8 + samp.size * 4 + tv.size * 8 + nloci * 16 + (nch + 1) * 4
    d2h = ngen * (T * 20 + M * 12 + 20) + nch * 8 * (1 + nth + nmg)
    # algorithmic bytes of one treeweight launch: node records, migrations,
    # weights written
    algo = N * 20 + Nm * 12 + ngen * (T * 20 + M * 12 + 20)
    hbm, _, src = measured_peaks()
    gbs = algo / (tw_ms / 1e3) / 1e9
    events = int((ngen - len(seq)) + sum(int((len(base[b].pop) - 1) // 2) for b in seq)) + int(Nm) + 2 * ngen
    out = {
        "metric": TW_METRIC, "value": round(value, 1), "unit": "genealogies/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic population-labelled IM genealogies",
        "config": {"workload": "config4-treeweight: %d chains x %d loci, 3 populations ((0,1):3,2):4, "
                               "samples U(4,60) per population, %d genealogies, %d nodes, %d migrations"
                               % (nch, nloci, ngen, N, Nm),
                   "global_batch": ngen, "l2": "flushed between timed steps"},
        "e2e": {"value": round(e2e, 1), "unit": "genealogies/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "kernels_ms": {"treeweight": round(tw_ms, 4), "tree_prob": round(tp_ms, 4)},
        "events_per_s": round(events / (tw_ms / 1e3), 1),
        "roofline": {"kernel": "k_treeweight", "bound": "hbm", "achieved": round(gbs, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(gbs / hbm, 5), "peak_source": src, "traffic": None,
                     "note": "a serial event sweep per genealogy: latency and FP64-issue bound, far from HBM"},
        "gpu_launches": int(n_timed), "clocks": clk.summary(),
    }
    # CPU: the oracle's treeweight (C) over whole chains of the same inputs, one core
    sub = nloci * 8  # eight chains per call
    spk = (node_off[:sub + 1], up0[:node_off[sub]], time_[:node_off[sub]], pop[:node_off[sub]],
           mig_off[:node_off[sub] + 1], mig_t[:mig_off[node_off[sub]]], mig_p[:mig_off[node_off[sub]]])
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < args.cpu_seconds or n == 0:
        bad, ow = O.treeweight_batch(pm, spk, gl[:sub], gt[:sub], hval, samp, tv)
        n += sub
    dt = time.perf_counter() - t0
    assert bad == 0 and np.array_equal(ow["fc"], w["fc"][:sub]) and np.array_equal(ow["mc"], w["mc"][:sub])
    out["cpu_baseline"] = {"value": round(n / dt, 1), "unit": "genealogies/s", "cores": 1, "kind": "port",
                           "sample": "%d genealogies (8 chains x %d loci per call) through the oracle's "
                                     "treeweight in C" % (n, nloci)}
    out["splittime_sweep"] = splittime_sweep(pm, packed, samp, tv, base, seq, nloci, nch, args)
    print(json.dumps(out), flush=True)
    ctx.close()


def splittime_sweep(pm, packed, samp, tv, base, seq, nloci, nch, args):
    """The device-resident split-time update (changet_RY1) on the same
    chain set, loci with infinite-sites data simulated on their genealogies:
    one update of every chain per sweep (ima2p_gb300.splittime.
    ResidentChainSet), timed on the host clock around whole sweeps."""
    import copy
    from ima2p_gb300 import api, splittime, synth
    from oracle import pyoracle as O
    rng = np.random.default_rng(1012)
    nbase = len(base)
    seqs = [synth.is_data(rng, base[b].g, 1.0, min_sites=2) for b in range(nbase)]
    ctx = api.Context(0)
    for li in range(nloci):
        ctx.add_locus_is(seqs[li % nbase])
    ctx.set_chains(1, nch)
    nth, nmg = len(pm.th_cells), len(pm.mg_cells)
    ctx.set_popmodel(pm, [15.0] * nth, [0.0] * nth, [2.0] * nmg, [0.0] * nmg, [1.0] * nmg)
    gens = [[copy.deepcopy(base[li % nbase]) for li in range(nloci)] for _ in range(nch)]
    t0 = time.perf_counter()
    cs = splittime.ResidentChainSet(ctx, gens, np.repeat(tv, nch, axis=0), np.linspace(1.0, 0.5, nch),
                                    np.ones(nloci), samp, np.ones(nloci))
    setup_s = time.perf_counter() - t0
    mt = api.MT19937(99)
    prng = np.random.default_rng(3)
    tprior = [(0.0, 3.0), (0.0, 6.0)]
    for _ in range(args.warmup):
        cs.sweep_device_mt(prng.integers(0, 2, nch), mt, tprior)
        cs.sweep_device(prng.integers(0, 2, nch), mt, tprior, 3)
        cs.sweep(prng.integers(0, 2, nch), mt, tprior, 3)
    ctx.synchronize()
    nsw = 10
    acc = 0
    t0 = time.perf_counter()
    for _ in range(nsw):
        acc += int(cs.sweep_device_mt(prng.integers(0, 2, nch), mt, tprior).sum())
    ctx.synchronize()
    wall = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(nsw):
        cs.sweep_device(prng.integers(0, 2, nch), mt, tprior, 3)
    ctx.synchronize()
    wall_pydraws = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(nsw):
        cs.sweep(prng.integers(0, 2, nch), mt, tprior, 3)
    ctx.synchronize()
    wall_host = time.perf_counter() - t0
    # one core: the same update of one chain on the oracle's C functions
    # (rubber band in numpy, treeweight, p(G), likelihoodIS)
    node_off, up0, time_, pop, mig_off, mig_t, mig_p = packed
    one = (node_off[:nloci + 1], up0[:node_off[nloci]], time_[:node_off[nloci]].copy(), pop[:node_off[nloci]],
           mig_off[:node_off[nloci] + 1], mig_t[:mig_off[node_off[nloci]]].copy(), mig_p[:mig_off[node_off[nloci]]])
    gl = np.arange(nloci, dtype=np.int32)
    slk = [O.is_sumlogk(seqs[li % nbase], base[li % nbase].g)[1] for li in range(nloci)]
    t0 = time.perf_counter()
    ncpu = 0
    while time.perf_counter() - t0 < max(1.0, args.cpu_seconds / 2) or ncpu == 0:
        t = one[2]
        lo = (t > 0) & (t <= tv[0, 0])
        t[lo] = t[lo] * (tv[0, 0] * 1.0001) / tv[0, 0]
        bad, w = O.treeweight_batch(pm, one, gl, np.zeros(nloci, np.int32), np.ones(nloci), samp, tv)
        tot = O.sum_weights([{k: w[k][i] for k in ("cc", "hcc", "fc", "mc", "fm")} for i in range(nloci)], pm)
        O.tree_prob(pm, tot, [15.0] * nth, [0.0] * nth, [2.0] * nmg, [0.0] * nmg, [1.0] * nmg)
        for li in range(nloci):
            O.is_likelihood(seqs[li % nbase], base[li % nbase].g, w["lens"][li, 0], 1.0, slk[li])
        ncpu += 1
    cpu = ncpu / (time.perf_counter() - t0)
    ctx.close()
    return {"chain_updates_per_s": round(nsw * nch / wall, 1), "ms_per_sweep": round(1e3 * wall / nsw, 3),
            "ms_per_sweep_python_draws": round(1e3 * wall_pydraws / nsw, 3),
            "ms_per_sweep_host_decisions": round(1e3 * wall_host / nsw, 3),
            "chains": nch, "loci": nloci, "accept_rate": round(acc / (nsw * nch), 3),
            "setup_s": round(setup_s, 2),
            "cpu_chain_updates_per_s_1core": round(cpu, 2),
            "note": "resident genealogies, labels and times; per sweep one ima_gpu_changet_ry1_sweep_mt: MT19937 "
                    "draws (getnewt, acceptance) and the Hastings logs in the library; rubber band, weights, "
                    "p(G), infinite-sites likelihoods, MH decisions and commits on the GPU (python_draws: the "
                    "draws in Python; host_decisions: the decisions taken in Python too); CPU: one chain's "
                    "update on the oracle's C functions"}


def updgen_context(api, w, precision_hky=True):
    """A context holding the genealogy-update workload: HKY loci, every chain
    from the locus's coalescent draw, population labels, locus populations,
    base frequencies, geometric heats."""
    from ima2p_gb300 import popmodel
    ctx = api.Context(0)
    for l, loc in enumerate(w.loci):
        if w.kind == "sw":
            ctx.add_locus_sw(len(w.base[l].pop) // 2 + 1, 1)
        else:
            ctx.add_locus_hky(loc.seq, loc.mult, loc.totsites)
    ctx.set_chains(1, w.nch)
    pm = popmodel.build(w.tree, w.npops, nomig=True)
    th_max, th_min, _, _, _ = popmodel.priors(pm, 30.0, 0.0)
    ctx.set_popmodel(pm, th_max, th_min)
    nl = len(w.loci)
    ci = np.repeat(np.arange(w.nch, dtype=np.int32), nl)
    li = np.tile(np.arange(nl, dtype=np.int32), w.nch)
    flat = [w.base[l] for _ in range(w.nch) for l in range(nl)]
    ctx.set_genealogies(ci, li, np.concatenate([g.g.up0 for g in flat]), np.concatenate([g.g.up1 for g in flat]),
                        np.concatenate([g.g.down for g in flat]), np.concatenate([g.g.time for g in flat]),
                        length=np.full(len(flat), -1.0))
    ctx.set_labels(ci, li, flat)
    ctx.set_locus_pops(np.ones(nl), w.samppop)
    for c in range(w.nch):
        for l in range(nl):
            if w.kind == "sw":
                ctx.set_alleles(c, l, w.alleles[l])
            else:
                ctx.set_pi(c, l, w.loci[l].pi)
    ctx.set_betas(ug_betas(w.nch))
    return ctx, pm, th_max, th_min


def ug_betas(nch):
    """Linear heating, 1 / (1 + 0.05 k) for chain k of each run of up to
    128 chains."""
    return 1.0 / (1.0 + 0.05 * (np.arange(nch) % 128))


def updgen_cpu(args, w, pm, th_max, th_min):
    """The oracle's restatement of updategenealogy (C: treeweight, p(G),
    FP64 HKY from the edited edges) over every host core: whole sweeps of at
    least as many chains as cores, the call's set-up timed apart and
    subtracted."""
    from oracle import pyoracle as O
    nl = len(w.loci)
    cores = os.cpu_count() or 1
    if w.kind == "sw":
        ul = O.UgLoci([("sw", len(w.base[l].pop) // 2 + 1, int(w.arange[l][0]), int(w.arange[l][1]))
                       for l in range(nl)], np.ones(nl), w.samppop)
    else:
        ul = O.UgLoci([("hky", loc) for loc in w.loci], np.ones(nl), w.samppop)
    nc = min(w.nch, max(cores, 8))
    gens = [[w.base[l] for l in range(nl)] for _ in range(nc)]
    pis = np.array([np.zeros(4) if w.kind == "sw" else w.loci[l].pi for _ in range(nc) for l in range(nl)])
    al = {(c, l): w.alleles[l] for c in range(nc) for l in range(nl)} if w.kind == "sw" else None

    def cpu_run(ns):
        rr = [O.UgRng(1000 + c) for c in range(nc)]
        t = time.perf_counter()
        st = O.ug_run(pm, th_max, th_min, ul, gens, np.tile(w.tvals, (nc, 1)), ug_betas(nc),
                      np.tile(w.u, nc), np.tile(w.kappa, nc), pis, ns, rr, nthreads=cores, record=False,
                      alleles=al)[0]
        assert st == 0
        return time.perf_counter() - t

    t_setup = cpu_run(0)
    ncpu = 1
    while True:
        t_cpu = cpu_run(ncpu) - t_setup
        if t_cpu > max(1.0, args.cpu_seconds / 2) or ncpu >= 1024:
            break
        ncpu *= 2
    return {"value": round(ncpu * nc * nl / max(t_cpu, 1e-9), 1), "unit": "proposals/s", "cores": cores,
            "kind": "port",
            "sample": "%d sweeps of %d chains x %d loci through the oracle's restatement of updategenealogy in C "
                      "on %d threads, its set-up (%.0f ms) subtracted" % (ncpu, nc, nl, cores, 1e3 * t_setup)}


def measure_updgen(args, api, w, sweeps):
    """The genealogy update (ima_gpu_updategenealogy_sweep) on the whole
    chain set: one call of `sweeps` sweeps after a warm-up call, timed on the
    host clock around the call (its set-up -- one full evaluation and the
    chains' weights -- included), with the device time of its kernels by
    kind; the oracle's restatement on every host core for the CPU rate."""
    from oracle import pyoracle as O
    nl, nch = len(w.loci), w.nch
    ctx, pm, th_max, th_min = updgen_context(api, w)
    chains = np.arange(nch, dtype=np.int32)
    tv = np.tile(w.tvals, (nch, 1))
    u, kap = np.tile(w.u, nch), np.tile(w.kappa, nch)
    rngs = [api.UgRng(1000 + c) for c in range(nch)]
    ar = w.arange
    ctx.updategenealogy_sweep(chains, tv, args.warmup, rngs, u, kap, precision=api.PREC_FAST, allele_range=ar)
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.updategenealogy_sweep(chains, tv, 0, rngs, u, kap, precision=api.PREC_FAST, allele_range=ar)
    setup_s = time.perf_counter() - t0
    n0 = ctx.launch_count()
    with Clocks(0) as clk:
        t0 = time.perf_counter()
        acc, top, probg = ctx.updategenealogy_sweep(chains, tv, sweeps, rngs, u, kap, precision=api.PREC_FAST,
                                                    allele_range=ar)
        wall = time.perf_counter() - t0
    n_timed = ctx.launch_count() - n0
    # where a sweep's device time goes: the same call again with an event pair
    # around every launch (which slows the call; not the timed one)
    ctx.set_profiling(True)
    kinds = {"proposal_and_decision": api.K_UG, "treeweight": api.K_TREEWEIGHT, "hky": api.K_HKY_FAST}
    k0 = {k: ctx.kernel_stats(v) for k, v in kinds.items()}
    ctx.updategenealogy_sweep(chains, tv, sweeps, rngs, u, kap, precision=api.PREC_FAST, allele_range=ar)
    k1 = {k: ctx.kernel_stats(v) for k, v in kinds.items()}
    ctx.set_profiling(False)
    t0 = time.perf_counter()
    ctx.updategenealogy_sweep(chains, tv, sweeps, rngs, u, kap, precision=api.PREC_FP64, allele_range=ar)
    wall64 = time.perf_counter() - t0
    ctx.close()
    props = sweeps * nch * nl
    dev_ms = {k: round((k1[k][1] - k0[k][1]) / sweeps, 4) for k in kinds}
    cpu = updgen_cpu(args, w, pm, th_max, th_min)
    return {
        "metric": UG_METRIC, "value": round(props / wall, 1), "unit": "proposals/s",
        "ms_per_sweep": round(1e3 * wall / sweeps, 3), "sweeps": sweeps,
        "config": {"workload": w.describe},
        "e2e": {"value": round(props / wall, 1), "unit": "proposals/s", "h2d_bytes_per_step": int(nch * 2520 * 2 / sweeps),
                "d2h_bytes_per_step": int(nch * (nl * 8 + 8) / sweeps),
                "note": "one ima_gpu_updategenealogy_sweep call of all sweeps, its set-up included (%.1f ms: a "
                        "full evaluation and the chains' weights summed afresh); the chains' generators go in "
                        "and come back" % (1e3 * setup_s)},
        "device_ms_per_sweep": dev_ms,
        "fp64_form": {"value": round(props / wall64, 1), "unit": "proposals/s"},
        "accept_rate": round(float(acc.sum()) / props, 3),
        "topology_changes_accepted": int(top.sum()),
        "gpu_launches": int(n_timed), "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }


def updgen_workload(args):
    """The genealogy-update workload both arms run: the model's (HKY: 32
    chains, SW: 64) with --updgen-chains chains when given."""
    from ima2p_gb300 import workloads
    make = workloads.make_updgen_sw if args.updgen_model == "sw" else workloads.make_updgen
    return make() if args.updgen_chains is None else make(nch=args.updgen_chains)


def run_updgen(args):
    from ima2p_gb300 import api
    sub = measure_updgen(args, api, updgen_workload(args), max(1, min(args.steps, 20)))
    line = {"metric": sub.pop("metric"), "value": sub.pop("value"), "unit": sub.pop("unit"), "n_gpus": 1,
            "steps": sub["sweeps"], "warmup": args.warmup, "ms_per_step": sub["ms_per_sweep"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64 (SW terms and weights)" if w.kind == "sw" else "ff32 HKY + fp64 weights",
            "data": "synthetic population-labelled genealogies (no migration) and HKY data"}
    line.update(sub)
    print(json.dumps(line), flush=True)


def run_popmig(args):
    """The 2NM curves of print_populationmigrationrate_histograms for a
    3-population model (5 population sizes, 8 migration rates; its 8 default
    2NM terms) over G = 300,000 saved genealogies (MAXGENEALOGIESTOSAVE):
    one step = every term's range scan and its curve of GRIDSIZE 1000
    points, every point a sum over all G genealogies of calc_popmig's
    incomplete-gamma term.  The metric counts the curve terms (points x
    genealogies); the scan is overhead in both implementations."""
    from ima2p_gb300 import api, popmodel, synth
    from oracle import pyoracle as O

    G, grid = args.popmig_g, 1000
    rng = np.random.default_rng(1013)
    rows = synth.peaked_stats(rng, G, 5, 8, 2)
    pm = popmodel.build("((0,1):3,2):4", 3)
    terms = popmodel.popmig_terms(pm)
    tlist = [(t, m) for t, m, _ in terms]
    qmax, mmax = np.full(5, 20.0), np.full(8, 2.0)
    ctx = api.Context(0)
    ctx.surface_load(rows, 5, 8, 3)
    for _ in range(args.warmup):
        xs, ys, mx = ctx.popmig_curves(tlist, qmax, mmax, gridsize=grid)
    ctx.set_profiling(True)
    k0 = ctx.kernel_stats(api.K_POPMIG)
    n0 = ctx.launch_count()
    wall = []
    with Clocks(0) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            t0 = time.perf_counter()
            xs, ys, mx = ctx.popmig_curves(tlist, qmax, mmax, gridsize=grid)
            wall.append(time.perf_counter() - t0)
    k1 = ctx.kernel_stats(api.K_POPMIG)
    n_timed = ctx.launch_count() - n0
    ctx.set_profiling(False)
    nk = max(1, k1[0] - k0[0])
    # scan points per step: each term scans down from the top in batches of
    # 32, 128, 512, ... points until a density above 1e-9
    nscan = 0
    for (t, m), v in zip(tlist, mx):
        pmmax = qmax[t] * mmax[m] / 2.0
        need = grid - int(round(v * grid / pmmax - 0.5)) if v < pmmax else grid
        b, left = 32, grid
        while need > 0 and left > 0:
            nscan += min(b, left)
            need -= b
            left -= b
            b *= 4
    launch_ms = (k1[1] - k0[1]) / nk
    dev_ms = launch_ms * nk / args.steps
    pts = len(tlist) * grid  # curve points; the top-down scan for each term's range is overhead
    units = pts * G
    value = units / (dev_ms / 1e3)
    e2e = units / statistics.median(wall)
    hbm, _, src = measured_peaks()
    algo = G * rows.shape[1] * 4 + len(tlist) * grid * 8 * 3  # rows once, points and partials per launch
    gbs = algo / (launch_ms / 1e3) / 1e9
    out = {
        "metric": PM_METRIC, "value": round(value, 1), "unit": "terms/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic gsampinf rows with interior peaks (cc ~ Poisson(15), fc/cc ~ U(1,5), mc ~ Poisson(4), "
                "mc/fm ~ U(0.3,2), log integrals ~ N(0,1))",
        "config": {"workload": "popmig-curves: G=%d genealogies, 3 populations (5 theta, 8 m), %d 2NM terms, "
                               "curves of %d points each after the top-down range scan, posterior form"
                               % (G, len(tlist), grid),
                   "global_batch": pts, "l2": "flushed between timed steps (rows 57.6 MB; L2-resident within a step)"},
        "e2e": {"value": round(e2e, 1), "unit": "terms/s", "h2d_bytes_per_step": int(pts * 40 + nscan * 40),
                "d2h_bytes_per_step": int(pts * 16 + nscan * 8)},
        "scan_points_per_step": nscan,
        "curve_points_per_s": round(pts / (dev_ms / 1e3), 1),
        "roofline": {"kernel": "k_popmig", "bound": "hbm", "achieved": round(gbs, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(gbs / hbm, 6), "peak_source": src, "traffic": None,
                     "note": "FP64-issue bound: one or two incomplete gamma series / continued fractions per "
                             "(point, genealogy); HBM is not the limit"},
        "gpu_launches": int(n_timed), "clocks": clk.summary(),
    }
    # CPU: the oracle's calc_popmig (C) over all G genealogies, one core
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < args.cpu_seconds or n == 0:
        t, m = tlist[n % len(tlist)]
        O.popmig(rows, 5, 8, t, m, xs[n % len(tlist), (n * 37) % grid], qmax[t], mmax[m])
        n += 1
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": round(n * G / dt, 1), "unit": "terms/s", "cores": 1, "kind": "port",
                           "sample": "%d curve points over all %d genealogies through the oracle's "
                                     "calc_popmig in C" % (n, G)}
    # findmarginpeaks on the same genealogies: 13 parameters x 3 genealogy
    # ranges of bracket + golden-section searches, the migration tests, the
    # 95% limits, and the 8 2NM terms' scans, searches and tests
    tmin, mmin = np.zeros(5), np.zeros(8)
    t0 = time.perf_counter()
    pk = ctx.findmarginpeaks(tmin, qmax, mmin, mmax, terms=tlist)
    pk_s = time.perf_counter() - t0
    # the oracle's findmarginpeaks in C on a genealogy sample, scaled per genealogy
    gs = args.peaks_cpu_g
    t0 = time.perf_counter()
    O.findmarginpeaks(rows[:gs], 5, 8, tmin, qmax, mmin, mmax, terms=tlist)
    cpu_s = (time.perf_counter() - t0) * G / gs
    # the saved genealogies as a .ti file (the reference's "%.6f" tab-separated
    # text), loaded by the library's parser and by the reference's value loop
    import tempfile
    tdir = tempfile.mkdtemp()
    tpath = os.path.join(tdir, "popmig.ti")
    with open(tpath, "w") as f:
        f.write("IMa2p-style header\nVALUESSTART\n")
        np.savetxt(f, rows, fmt="%.6f", delimiter="\t")
    mb = os.path.getsize(tpath) / 1e6
    t0 = time.perf_counter()
    lrows, _ = api.ti_read([tpath], rows.shape[1])
    ti_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    orows = O.ti_load(tpath, rows.shape[1], G)
    ti_cpu = time.perf_counter() - t0
    bpath = os.path.join(tdir, "popmig.tib")
    api.ti_write_binary(bpath, lrows)
    t0 = time.perf_counter()
    brows = api.ti_read_binary(bpath)
    tib_s = time.perf_counter() - t0
    assert np.array_equal(lrows, orows) and np.array_equal(brows, lrows)
    for fp in (tpath, bpath):
        os.unlink(fp)
    os.rmdir(tdir)
    out["ti_load"] = {"genealogies": int(len(lrows)), "mb": round(mb, 1), "seconds": round(ti_s, 3),
                      "mb_per_s": round(mb / ti_s, 1), "binary_seconds": round(tib_s, 4),
                      "cpu_seconds_1core": round(ti_cpu, 3),
                      "cpu": "the reference's loop (fgets per genealogy, sscanf per value) in the oracle, one core",
                      "rows_equal": True}
    out["marginal_peaks"] = {"seconds": round(pk_s, 3), "rounds": pk["rounds"],
                             "cpu_seconds_1core_scaled": round(cpu_s, 1),
                             "cpu_sample": "the oracle's findmarginpeaks on the first %d genealogies, "
                                           "scaled by %d/%d" % (gs, G, gs),
                             "note": "all searches advance together; each round one batched launch per density "
                                     "kind and genealogy range"}
    print(json.dumps(out), flush=True)
    ctx.close()



# ------------------------------------------------------- default: all configs
def run_all(args):
    """Config 3 (SW) as the headline line; configs 1, 2, 4 and 5 as sub-objects."""
    from ima2p_gb300 import api, workloads

    dist = init_dist()
    dev = rank_device()
    head = measure_lik(args, api, workloads.make("sw"), args.steps, dist, dev)
    configs = {}
    sub_steps = min(args.steps, 200)
    configs["config1_is"] = measure_lik(args, api, workloads.make("is"), sub_steps, dist, dev)
    configs["config2_hky"] = measure_lik(args, api, workloads.make("hky"), sub_steps, dist, dev, hky_legs=True)
    configs["config4_mixed"] = measure_lik(args, api, workloads.make("mixed"), min(args.steps, 30), dist, dev)
    configs["config5_surface"] = measure_surface(args, api, min(args.steps, 20), not args.no_peak_search, dev)
    # 20 sweeps: a timed call of 40-200 ms, long against the clock sampler's
    # 200 ms queries (one of them in a 100 ms call moved its rate 3x)
    configs["genealogy_update"] = measure_updgen(args, api, workloads.make_updgen(), 20)
    configs["genealogy_update_1024_chains"] = measure_updgen(args, api, workloads.make_updgen(nch=1024), 20)
    configs["genealogy_update_sw"] = measure_updgen(args, api, workloads.make_updgen_sw(), 20)
    emit(args, head, METRIC, dist, {"configs": configs})


# ------------------------------------------------------- the reference arm
def run_reference(args):
    """The reference's CPU path on every host core: the oracle (a C
    restatement of the reference functions, pinned to the compiled reference
    by the golden fixtures) through its batched C entry points on one thread
    per core.  Headline: the stepwise-microsatellite workload; sub-objects:
    the other named workloads (the surface on a bounded sample of points,
    extrapolated per point)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from ima2p_gb300 import workloads

    cores = os.cpu_count() or 1
    name = "sw" if args.workload == "all" else args.workload
    if name == "updgen":
        from ima2p_gb300 import popmodel
        w = updgen_workload(args)
        pm = popmodel.build(w.tree, w.npops, nomig=True)
        th_max, th_min, _, _, _ = popmodel.priors(pm, 30.0, 0.0)
        cpu = updgen_cpu(args, w, pm, th_max, th_min)
        print(json.dumps({"impl": "reference", "metric": UG_METRIC, "value": cpu["value"], "unit": cpu["unit"],
                          "n_gpus": 0, "steps": 1, "warmup": args.warmup, "ms_per_step": None,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
                          "data": "synthetic", "config": {"workload": w.describe}, "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": cpu["unit"], "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    if name in ("treeweight", "popmig"):
        print(json.dumps({"impl": "reference", "unavailable": "%s: the CPU rate is the line's cpu_baseline"
                          % name}))
        return

    def lik_arm(wl, k_steps, step_seconds):
        packs = oracle_packs(wl, CPU_SAMPLE)
        times, done = [], 0
        for s in range(args.warmup + k_steps):
            v, n, t = cpu_rate(packs, step_seconds, cores)
            if s >= args.warmup:
                times.append(t)
                done += n
        v = done / sum(times)
        return {"value": round(v, 1), "unit": "evals/s", "ms_per_step": round(1e3 * statistics.median(times), 3),
                "config": {"workload": wl.describe},
                "cpu_baseline": {"value": round(v, 1), "unit": "evals/s", "cores": cores, "kind": "port",
                                 "sample": "an even sample of %d chain-loci of the workload's %d, the oracle's "
                                           "batched C path on %d threads, >= %.2f s per step"
                                           % (sum(p.nitems for p in packs), wl.nchains * wl.nloci, cores,
                                              step_seconds)},
                "e2e": {"value": round(v, 1), "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    def surface_arm():
        G, P, rows, lognorm, pts = surface_inputs(args)
        v, n, t = surface_cpu(rows, lognorm, pts, max(args.cpu_seconds, 20.0), cores)
        return {"value": round(v, 3), "unit": "points/s", "ms_per_step": round(1e3 * P / v, 1),
                "config": {"workload": "config5-surface: G=2^%d, P=2^%d" % (args.surface_log2g, args.surface_log2p)},
                "cpu_baseline": {"value": round(v, 3), "unit": "points/s", "cores": cores, "kind": "port",
                                 "sample": "%d points in %.1f s (exact jointp over all %d genealogies, %d "
                                           "threads), extrapolated per point to the %d-point grid"
                                           % (n, t, G, cores, P)},
                "e2e": {"value": round(v, 3), "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    k_steps = max(1, min(args.steps, 50))
    step_s = max(0.05, min(0.5, 60.0 / (k_steps + args.warmup)))
    if name == "surface":
        head, metric = surface_arm(), SURF_METRIC
    else:
        head, metric = lik_arm(workloads.make(name), k_steps, step_s), METRIC
    line = {"impl": "reference", "metric": metric, "value": head["value"], "unit": head["unit"], "n_gpus": 0,
            "steps": k_steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
            "config": head["config"], "cpu_baseline": head["cpu_baseline"], "e2e": head["e2e"]}
    if args.workload == "all":
        line["configs"] = {
            "config1_is": lik_arm(workloads.make("is"), 3, 0.5),
            "config2_hky": lik_arm(workloads.make("hky"), 3, 0.5),
            "config4_mixed": lik_arm(workloads.make("mixed"), 3, 0.5),
            "config5_surface": surface_arm(),
        }
        from ima2p_gb300 import popmodel
        for key, w in (("genealogy_update", workloads.make_updgen()), ("genealogy_update_sw", workloads.make_updgen_sw())):
            pm = popmodel.build(w.tree, w.npops, nomig=True)
            th_max, th_min, _, _, _ = popmodel.priors(pm, 30.0, 0.0)
            cpu = updgen_cpu(args, w, pm, th_max, th_min)
            line["configs"][key] = {"value": cpu["value"], "unit": cpu["unit"], "config": {"workload": w.describe},
                                    "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="all", choices=["all", "sw", "is", "hky", "mixed", "surface",
                                                        "treeweight", "popmig", "updgen"])
    ap.add_argument("--cpu-seconds", type=float, default=3.0)
    ap.add_argument("--surface-log2g", type=int, default=21, help="log2 genealogies (config 5: 21)")
    ap.add_argument("--surface-log2p", type=int, default=16, help="log2 points (config 5: 16)")
    ap.add_argument("--surface-method", default="tc", choices=["tc", "fp32"])
    ap.add_argument("--no-peak-search", action="store_true", help="surface: skip the marginals and peak search")
    ap.add_argument("--popmig-g", type=int, default=300000, help="popmig: saved genealogies")
    ap.add_argument("--peaks-cpu-g", type=int, default=6000, help="popmig: genealogies in the CPU peaks sample")
    ap.add_argument("--updgen-chains", type=int, default=None,
                    help="updgen: chains (default: the model's workload, 32 for hky, 64 for sw)")
    ap.add_argument("--updgen-model", default="hky", choices=["hky", "sw"],
                    help="updgen: config-2 HKY loci or config-3 SW loci")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "all":
        run_all(args)
    elif args.workload == "surface":
        run_surface(args)
    elif args.workload == "treeweight":
        run_treeweight(args)
    elif args.workload == "popmig":
        run_popmig(args)
    elif args.workload == "updgen":
        run_updgen(args)
    else:
        run_likelihood_line(args, args.workload)


if __name__ == "__main__":
    main()
