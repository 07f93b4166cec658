#!/usr/bin/env python3
"""Benchmark of the batched pairwise-alignment hot path on GB300.

Default workload: the uneven Smith-Waterman batch -- 200,000 DNA pairs,
query log-uniform 50-1,000 bp, target = query at 5 % divergence between
uniform 0-500 bp flanks, scoring {2,-3,3,1}, score + end + start + CIGAR for
every pair.  A step is one pass of the aligner over the whole batch.

* ``value``: GCUPS (sum of text_len * pattern_len over the batch / step time)
  with the batch already resident in HBM, through the device-resident entry
  (ga_sw_device), timed with CUDA events on the launch stream.
* ``e2e``: the same metric through the public C ABI call (ga_align_sw_batch)
  with host buffers: staging, host-to-device copy, kernels, device-to-host copy
  and CIGAR/validation materialisation are inside every step.
* ``roofline``: the dominant kernel's cells per launch over its average
  event-timed launch duration, against the integer-pipe peak measured by a
  microbenchmark kernel on this GPU (6 integer operations per cell).
* ``cpu_baseline``: the CPU oracle (a restatement of the reference's CPU path)
  on a bounded sample, on this host's cores.
* ``extra.wfa``: WFA pairs/s on the 10,000-pair 150 bp / 2 % batch (smax 64,
  CIGAR) the same two ways.

``--impl reference`` times the reference's CPU path (the oracle port) on the
host cores on bounded samples of the same workload and prints the same line
with ``impl: reference``.  With N GPUs (torchrun) every rank runs an
independent replica: the path has no exchange step.
"""
from __future__ import annotations

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

METRIC = "WFA pairs/s & SW GCUPS on 1 GB300, learned-bucketed vs plain, bit-exact"
SCORING = (2, -3, 3, 1)
OPS_PER_CELL = 6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=200_000)
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    return ap.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampler running across the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(gpu_index), "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [ln.split(",") for ln in self.f.read().strip().splitlines() if ln.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def sw_cells(ps):
    return int((ps.a_len.astype(np.int64) * ps.b_len.astype(np.int64)).sum())


def cpu_baseline_sw(ps, seconds, threads):
    """The oracle (a restatement of the reference's CPU path) on a bounded
    sample: pairs taken from a fixed random permutation until ~`seconds`."""
    import oracle
    order = np.random.default_rng(123).permutation(ps.n)
    done_cells, t_used, k, chunk = 0, 0.0, 0, 256
    while t_used < seconds and k < ps.n:
        idx = order[k:k + chunk]
        sub = ps.subset(idx)
        ts, pp = sub.lists()
        t0 = time.perf_counter()
        oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, threads=threads)
        t_used += time.perf_counter() - t0
        done_cells += sw_cells(sub)
        k += chunk
        chunk = min(chunk * 2, 8192)
    return done_cells / t_used / 1e9, k, done_cells


def cpu_baseline_wfa(ps, seconds, threads):
    import oracle
    pats, txts = ps.lists()
    done, t_used = 0, 0.0
    while t_used < seconds and done < 4 * ps.n:
        t0 = time.perf_counter()
        oracle.wfa_batch(pats, txts, smax=64, with_cigar=True, threads=threads)
        t_used += time.perf_counter() - t0
        done += ps.n
    return done / t_used, done


def run_reference(args, rank, world):
    from genoaligner_gb300 import workloads
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ps = workloads.sw_uneven_200k(n=args.pairs)
    per_step = max(2.0, 60.0 / max(1, args.steps + args.warmup))
    vals = []
    samples = []
    for s in range(args.warmup + args.steps):
        g, k, cells = cpu_baseline_sw(ps, per_step, threads)
        if s >= args.warmup:
            vals.append(g)
            samples.append((k, cells))
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sw_cells(ps) / (v * 1e9) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator, seed 2)",
        "config": {"workload": "sw_uneven_200k: 200,000 pairs, query log-uniform 50-1,000 bp, target = query at "
                               "5% (sub/ins/del 60/20/20) between U{0..500} flanks, scoring {2,-3,3,1}, "
                               "score+end+start+CIGAR", "pairs": ps.n, "cells": sw_cells(ps)},
        "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": "port",
                         "sample": f"per step: pairs from a fixed random permutation until ~{per_step:.0f} s of "
                                   f"CPU time (last step {samples[-1][0]} pairs, {samples[-1][1] / 1e9:.2f} Gcells)"},
        "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from genoaligner_gb300 import api, workloads
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    ps = workloads.sw_uneven_200k(n=args.pairs)
    cells = sw_cells(ps)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    n = ps.n
    out_score = torch.empty(n, dtype=torch.int32, device=dev)
    out_pos = torch.empty(4 * n, dtype=torch.int32, device=dev)
    out_len = torch.empty(n, dtype=torch.int32, device=dev)
    out_cig = torch.empty(max(batch.out_bytes, 1), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        api.sw_device(batch, SCORING, True, out_score, out_pos, out_len, out_cig, stream=stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    launches0 = api.kernel_launches()
    api.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    api.profile(False)
    barrier(world)
    launches = api.kernel_launches() - launches0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world)
    prof = api.profile_read()
    value = world * cells / (ms * 1e-3) / 1e9

    # dominant kernel and its roofline
    top = max(prof.items(), key=lambda kv: kv[1][0]) if prof else ("none", (0.0, 1))
    top_name, (top_ms, top_n) = top
    widths = {"sw8_trace": 8, "sw16_trace": 16, "sw32_trace": 32}
    C = widths.get(top_name, 32)
    sel = np.array([api_width(int(x)) == C for x in ps.b_len])
    top_cells = int((ps.a_len.astype(np.int64)[sel] * ps.b_len.astype(np.int64)[sel]).sum())
    achieved_gcups = top_cells / (top_ms / top_n * 1e-3) / 1e9 if top_ms > 0 else 0.0
    peak_ops = api.int_peak(0)
    peak_gcups = peak_ops / OPS_PER_CELL / 1e9
    roofline = {"bound": "int32", "achieved": achieved_gcups, "peak": peak_gcups, "unit": "GCUPS",
                "frac": achieved_gcups / peak_gcups if peak_gcups else None, "traffic": None,
                "kernel": top_name, "ops_per_cell": OPS_PER_CELL,
                "peak_source": f"measured int32 microbenchmark: {peak_ops / 1e12:.2f} T lane-ops/s (add+max)",
                "kernel_ms_per_launch": top_ms / top_n, "kernel_share": top_ms / sum(v[0] for v in prof.values())}

    # correctness gate of the measured run: CIGAR strings of a sample vs the oracle
    import oracle
    idx = np.random.default_rng(7).choice(n, 64, replace=False)
    sc = out_score.cpu().numpy()
    sub = ps.subset(idx)
    ts, pp = sub.lists()
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True)
    parity_ok = bool(np.array_equal(sc[idx], want.score))

    # e2e through the public C ABI with host buffers
    reqs = api.make_sw_requests(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING, True)
    res = np.zeros(n, api.SWRES_DT)
    cig = np.empty(int(api.load().ga_align_sw_cigar_bytes(reqs.ctypes.data, n)), np.uint8)
    for _ in range(max(1, args.warmup - 1)):
        api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING,
                                  _reqs=reqs, _res=res, _cig=cig)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING,
                                      _reqs=reqs, _res=res, _cig=cig)
    e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
    e2e_ms = max_over_ranks(e2e_ms, world)
    h2d, d2h = api.last_transfer_bytes()
    parity_ok = parity_ok and r.status == api.Status.ok and bool(
        np.array_equal(r.res["score"][idx], want.score)) and all(
        r.cigar(int(i)) == want.cigars[q] for q, i in enumerate(idx))

    extra = {}
    if not args.no_extra:
        extra["wfa"] = bench_wfa(api, workloads, torch, dev, stream, args)

    cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        g, k, done = cpu_baseline_sw(ps, args.cpu_seconds, threads)
        cpu = {"value": g, "unit": "GCUPS", "cores": threads, "kind": "port",
               "sample": f"{k} pairs ({done / 1e9:.2f} Gcells) of the same batch, fixed random permutation"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator, seed 2)",
            "config": {"workload": "sw_uneven_200k: 200,000 pairs, query log-uniform 50-1,000 bp, target = query "
                                   "at 5% (sub/ins/del 60/20/20) between U{0..500} flanks, scoring {2,-3,3,1}, "
                                   "score+end+start+CIGAR", "pairs": n, "cells": cells,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "inputs (%.0f MB) and direction tables exceed the 129 MB L2" % (batch.input_bytes / 1e6)},
            "e2e": {"value": world * cells / (e2e_ms * 1e-3) / 1e9, "unit": "GCUPS", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
            "parity_sample_ok": parity_ok,
            "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()},
            "extra": extra,
        }
        print(json.dumps(line), flush=True)


def api_width(n):
    if n <= 256:
        return 8
    if n <= 512:
        return 16
    return 32


def bench_wfa(api, workloads, torch, dev, stream, args):
    ps = workloads.wfa_150bp_2pct()
    n = ps.n
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    sc = torch.empty(n, dtype=torch.int32, device=dev)
    ln = torch.empty(n, dtype=torch.int32, device=dev)
    cg = torch.empty(batch.out_bytes, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(3):
        api.wfa_device(batch, 64, True, sc, ln, cg, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(args.steps, 5)):
        flush.zero_()                                   # evict the batch from L2
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        api.wfa_device(batch, 64, True, sc, ln, cg, stream=stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    dev_ms = statistics.median(times)
    reqs = api.make_requests(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, 64, True)
    res = np.zeros(n, api.RES_DT)
    cig = np.empty(int(api.load().ga_align_cigar_bytes(reqs.ctypes.data, n)), np.uint8)
    for _ in range(3):
        api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, _reqs=reqs, _res=res,
                               _cig=cig)
    t = []
    for _ in range(max(args.steps, 5)):
        t0 = time.perf_counter()
        api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, _reqs=reqs, _res=res,
                               _cig=cig)
        t.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(t) * 1e3
    cpu_pps, done = cpu_baseline_wfa(ps, 4.0, os.cpu_count() or 1)
    return {"workload": "wfa_150bp_2pct: 10,000 pairs, 150 bp, 2% (sub/ins/del equal), smax 64, CIGAR",
            "pairs_per_s": n / (dev_ms * 1e-3), "ms_per_step": dev_ms,
            "e2e_pairs_per_s": n / (e2e_ms * 1e-3), "e2e_ms_per_step": e2e_ms,
            "cpu_baseline_pairs_per_s": cpu_pps, "cpu_cores": os.cpu_count(), "cpu_kind": "port",
            "l2": "256 MB buffer written between steps"}


if __name__ == "__main__":
    main()
