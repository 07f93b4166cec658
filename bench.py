#!/usr/bin/env python3
"""Benchmark of the batched pairwise-alignment hot path on GB300.

Headline workload: the uneven Smith-Waterman batch -- 200,000 DNA pairs,
query log-uniform 50-1,000 bp, target = query at 5 % divergence between
uniform 0-500 bp flanks, scoring {2,-3,3,1}, score + end + start + CIGAR for
every pair, all pairs in one persistent launch.  A step is one pass of the
aligner over the whole batch.

* ``value``: GCUPS (sum of text_len * pattern_len over the batch / step time)
  with the batch resident in HBM, through the device-resident entry
  (ga_sw_device), timed with CUDA events on the launch stream.
* ``e2e``: the same metric through the public C ABI call (ga_align_sw_batch)
  with host buffers: staging, host-to-device copy, kernels, device-to-host
  copy and CIGAR/validation materialisation are inside every step.
* ``roofline``: the dominant kernel's cells per launch over its average
  event-timed launch duration, against the DPX rate this GPU retires
  (__viaddmax_s32, measured by peak.cu) divided by 6 instructions per cell;
  ``traffic`` is its DRAM bytes per launch from the committed ncu summary.
* ``cpu_baseline``: the CPU oracle (a restatement of the reference's CPU path)
  on a bounded sample, on this host's cores.
* ``extra``: the WFA workloads (150 bp / 2 %; the 1,000,000-pair mixed batch,
  plain fixed smax 64 against the learned-bucketed form; the long 1-10 kb
  batch at smax 2048) and the long Smith-Waterman batch (4,096 pairs).

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
# DRAM bytes per cell of the two-pairs-per-warp trace kernel, from
# profiles/sw16ck_trace_sw_uneven.md (ncu, 20,000-pair sample of the same
# batch: read + write bytes / cells; traffic grows with the cells processed)
SW16CK_DRAM_BYTES_PER_CELL = 0.2348
SW_WORKLOAD = ("sw_uneven_200k: 200,000 pairs, query log-uniform 50-1,000 bp, target = query at 5% "
               "(sub/ins/del 60/20/20) between U{0..500} flanks, scoring {2,-3,3,1}, score+end+start+CIGAR")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=200_000)
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=60.0,
                    help="--impl reference: host seconds over all warm-up and timed steps")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the device's current kernel setting instead of autotuning on the batch")
    ap.add_argument("--only", choices=["wfa_150bp", "wfa_mixed_1m", "wfa_long", "sw_long", "sw_score_only"],
                    help="run one of the extra workloads alone (no CPU baseline) and print its JSON")
    ap.add_argument("--set-tune", default=None,
                    help="kernel setting fields k=v[,k=v...] set before any run (and no autotuning), e.g. sw_pack16=0")
    ap.add_argument("--wfa-model", default=None,
                    help="WFA cost-model .npz to load instead of the committed one")
    ap.add_argument("--only-pairs", type=int, default=None,
                    help="with --only: the workload's first N pairs instead of all (small profiling cases)")
    return ap.parse_args()


def dist_setup():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
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
    """nvidia-smi sampler started before the warm-up; stop() keeps the samples
    whose timestamps fall inside the timed region (mark_begin / mark_end)."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, period_ms=50):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.t0 = self.t1 = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(gpu_index), "-lms", str(period_ms)], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def wait_first(self, limit_s=5.0):
        """Block until the sampler wrote its first line (at most limit_s)."""
        end = time.time() + limit_s
        while self.p is not None and time.time() < end:
            if os.path.getsize(self.f.name) > 0:
                return
            time.sleep(0.02)

    def mark_begin(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    @staticmethod
    def _when(ts):
        import datetime
        try:
            return datetime.datetime.strptime(ts.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

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
        os.unlink(self.f.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

        def summarise(sel):
            sm, mx, reasons = [], [], set()
            for r in sel:
                try:
                    sm.append(float(r[2]))
                    mx.append(float(r[3]))
                    for k, nm in enumerate(names):
                        if r[6 + k].strip().lower() == "active":
                            reasons.add(nm)
                except (ValueError, IndexError):
                    continue
            return sm, mx, reasons

        window = "timed region"
        sel = []
        if self.t0 is not None and self.t1 is not None:
            for r in rows:
                w = self._when(r[0]) if r else None
                if w is not None and self.t0 - 0.06 <= w <= self.t1 + 0.06:
                    sel.append(r)
        sm, mx, reasons = summarise(sel)
        if not sm:                      # no sample stamped inside: every sample of the run
            window = "warm-up and timed region"
            sm, mx, reasons = summarise(rows)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "window": window, "reasons": sorted(reasons)}


def sw_cells(ps):
    return int((ps.a_len.astype(np.int64) * ps.b_len.astype(np.int64)).sum())


# ------------------------------------------------------------------ checks --
# Comparisons of GPU outputs with the oracle's (the reference's CPU path
# restated): every field, every pair.
def wfa_equal_packed(got, want):
    """A host-entry WFA result (api.PackedResult) against oracle.WfaBatch."""
    r = got.res
    if got.status.name != want.status:
        return False
    for f in ("rescore_ok", "wellformed_ok", "resolved"):
        if not np.array_equal(r[f].astype(bool), getattr(want, f)):
            return False
    if not np.array_equal(r["score"], want.score):
        return False
    buf = got.cigar_buf
    return all(buf[o:o + n].tobytes() == c
               for o, n, c in zip(r["cigar_offset"].tolist(), r["cigar_len"].tolist(), want.cigars))


def sw_equal_packed(got, want):
    """A host-entry SW result against oracle.SwBatch."""
    r = got.res
    if got.status.name != want.status:
        return False
    for f in ("score", "start_i", "start_j", "end_i", "end_j"):
        if not np.array_equal(r[f], getattr(want, f)):
            return False
    for f in ("resolved", "rescore_ok", "wellformed_ok", "too_large"):
        if not np.array_equal(r[f].astype(bool), getattr(want, f)):
            return False
    buf = got.cigar_buf
    return all(buf[o:o + n].tobytes() == c
               for o, n, c in zip(r["cigar_offset"].tolist(), r["cigar_len"].tolist(), want.cigars))


def slot_ends(batch):
    """End of every pair's CIGAR slot in a device batch's output buffer."""
    return (batch.out_off.cpu().numpy() + batch.a_len.cpu().numpy().astype(np.int64) +
            batch.b_len.cpu().numpy().astype(np.int64))


def wfa_equal_device(out, want):
    """Device-entry WFA outputs (score, CIGAR length, CIGAR slots, slot ends)."""
    sc, ln, cg, ends = out
    if not np.array_equal(sc, want.score):
        return False
    lens = np.fromiter((len(c) for c in want.cigars), np.int64, count=len(want.cigars))
    if not np.array_equal(ln.astype(np.int64), lens):
        return False
    return all(cg[e - n:e].tobytes() == c for e, n, c in zip(ends.tolist(), lens.tolist(), want.cigars))


def sw_equal_device(out, want):
    """Device-entry SW outputs (score, positions, CIGAR length, slots, slot ends)."""
    sc, pos, ln, cg, ends = out
    pos = pos.reshape(-1, 4)
    if not np.array_equal(sc, want.score):
        return False
    for k, f in enumerate(("start_i", "start_j", "end_i", "end_j")):
        if not np.array_equal(pos[:, k], getattr(want, f)):
            return False
    lens = np.fromiter((len(c) for c in want.cigars), np.int64, count=len(want.cigars))
    if not np.array_equal(ln.astype(np.int64), lens):
        return False
    return all(cg[e - n:e].tobytes() == c for e, n, c in zip(ends.tolist(), lens.tolist(), want.cigars))


# ------------------------------------------------------------ CPU baseline --
def one_core_sample(run, n, seconds, first=64, cap=1 << 20):
    """Units per second of `run(idx)` (which returns (units, C seconds)) on
    one thread, over pairs of a fixed random permutation taken in growing
    chunks (passing over the batch again when it is used up) until ~`seconds`
    of C time; returns (rate, pairs run, C seconds)."""
    order = np.random.default_rng(777).permutation(n)
    units, used, done, k, chunk = 0, 0.0, 0, 0, first
    for _ in range(100_000):
        if used >= seconds:
            break
        idx = order[k:k + chunk]
        u, t = run(idx)
        units += u
        used += t
        done += len(idx)
        k += len(idx)
        if k >= n:
            k = 0
        chunk = min(chunk * 2, cap)
    return units / used if used > 0 else None, done, used


def cpu_baseline_sw(ps, seconds, threads):
    """The oracle on a bounded sample of the SW batch (pairs from a fixed
    random permutation until ~`seconds` of C time): GCUPS, pairs, cells,
    C seconds."""
    import oracle
    order = np.random.default_rng(123).permutation(ps.n)
    done_cells, t_used, k, chunk = 0, 0.0, 0, 256
    while t_used < seconds and k < ps.n:
        idx = order[k:k + chunk]
        sub = ps.subset(idx)
        ts, pp = sub.lists()
        got = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, threads=threads)
        t_used += got.seconds
        done_cells += sw_cells(sub)
        k += chunk
        chunk = min(chunk * 2, 8192)
    return done_cells / t_used / 1e9, k, done_cells, t_used


def run_reference(args, rank, world):
    from genoaligner_gb300 import workloads
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ps = workloads.sw_uneven_200k(n=args.pairs)
    per_step = max(0.5, args.ref_seconds / max(1, args.steps + args.warmup))
    vals, samples = [], []
    for s in range(args.warmup + args.steps):
        g, k, cells, used = cpu_baseline_sw(ps, per_step, threads)
        if s >= args.warmup:
            vals.append(g)
            samples.append((k, cells, used))
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sw_cells(ps) / (v * 1e9) * 1e3,
        "ms_per_step_is": "the whole batch's cells at the measured rate (each step times a sample)",
        "sample_seconds_per_step": [round(x[2], 3) for x in samples],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator, seed 2)",
        "config": {"workload": SW_WORKLOAD, "pairs": ps.n, "cells": sw_cells(ps)},
        "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": "port",
                         "build": "oracle/ga_oracle.c, gcc -O3 (no -march: the same code on x86 and Arm)",
                         "sample": f"per step: pairs from a fixed random permutation until ~{per_step:.1f} s of "
                                   f"C time (last step {samples[-1][0]} pairs, {samples[-1][1] / 1e9:.2f} Gcells, "
                                   f"{samples[-1][2]:.2f} s)"},
        "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def extra_steps(args):
    """Timed calls of each extra workload line: 5 to 10."""
    return max(5, min(args.steps, 10))


def timed(fn, stream, steps, flush=None):
    """Median CUDA-event time of `steps` calls of fn on `stream` (ms)."""
    import torch
    ts = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def bench_wfa_150(api, workloads, torch, dev, stream, args, keep):
    ps = workloads.wfa_150bp_2pct()
    n = ps.n
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    sc = torch.empty(n, dtype=torch.int32, device=dev)
    ln = torch.empty(n, dtype=torch.int32, device=dev)
    cg = torch.empty(batch.out_bytes, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    fn = lambda: api.wfa_device(batch, 64, True, sc, ln, cg, stream=stream.cuda_stream)
    for _ in range(3):
        fn()
    dev_ms = timed(fn, stream, extra_steps(args), flush)
    reqs = api.make_requests(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, 64, True)
    res = np.zeros(n, api.RES_DT)
    cig = np.empty(int(api.load().ga_align_cigar_bytes(reqs.ctypes.data, n)), np.uint8)
    call = lambda: api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, _reqs=reqs,
                                          _res=res, _cig=cig)
    for _ in range(3):
        call()
    t = []
    for _ in range(extra_steps(args)):
        t0 = time.perf_counter()
        r = call()
        t.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(t) * 1e3
    keep["wfa_150bp"] = {"ps": ps, "device": (sc.cpu().numpy(), ln.cpu().numpy(), cg.cpu().numpy(), slot_ends(batch)),
                         "e2e": r}
    return {"workload": "wfa_150bp_2pct: 10,000 pairs, 150 bp, 2% (sub/ins/del equal), smax 64, CIGAR",
            "pairs_per_s": n / (dev_ms * 1e-3), "ms_per_step": dev_ms,
            "e2e_pairs_per_s": n / (e2e_ms * 1e-3), "e2e_ms_per_step": e2e_ms,
            "l2": "256 MB buffer written between steps"}


ROUTE_BUCKETS = 32          # genoaligner_gb300/csrc/route.cuh
LANE_MAXLEN = 256


def route_report(items, score, smax, lane_smax, classes, lane_ok):
    """How the router's queue items compare with the ones the exact distance
    selects under the same rule (first smax = ceil(1.25 d + 2), lane queue iff
    that is <= lane_smax for an eligible pair, warp-queue bucket = its bit
    length; a pair unresolved at smax belongs in the warp queue at the top
    bucket, or is proven unresolved by the bound).  Per class: pairs in each
    queue, queue mispredictions (queue differs from the exact one), lane-queue
    pairs whose predicted first smax is below their distance (a lane runs its
    pair on past it: an under-prediction, not a rerun), warp-queue pairs
    whose bucket differs from the exact one."""
    d = score.astype(np.int64)
    unres = d < 0
    s_star = np.where(unres, smax, np.minimum(smax, np.ceil(1.25 * d + 2))).astype(np.int64)
    lane_star = (~unres) & lane_ok & (s_star <= lane_smax)
    bound = items < 0
    key = items & 0xFF
    first = items >> 8
    lane = (~bound) & (key >= ROUTE_BUCKETS)
    warp = (~bound) & (key < ROUTE_BUCKETS)
    bitlen = lambda x: np.floor(np.log2(np.maximum(x, 1))).astype(np.int64) + 1
    bucket_star = np.minimum(bitlen(s_star), ROUTE_BUCKETS - 1)
    out = {}
    for name, sel in classes.items():
        nl, nw = int((lane & sel).sum()), int((warp & sel).sum())
        qmis = int(((lane != lane_star) & ~bound & sel).sum())
        esc = int((lane & sel & (unres | (first < d))).sum())
        boff = int((warp & sel & ~unres & (key != bucket_star)).sum())
        out[name] = {"pairs": int(sel.sum()), "lane_queue": nl, "warp_queue": nw,
                     "unresolved_by_bound": int((bound & sel).sum()),
                     "queue_mispredicted_rate": qmis / max(1, int(sel.sum())),
                     "lane_underpredicted_rate": esc / max(1, nl),
                     "warp_bucket_mispredicted_rate": boff / max(1, nw)}
    return out


def wfa_arms(api, torch, dev, stream, batch, n, smax, steps, flush, tune_first, out):
    """The plain fixed-smax form, the learned-bucketed form and the same queues
    keyed by the lower bound alone, through ga_wfa_device_ex; device time per
    call, route items of the routed arms, bit-identity to the plain form."""
    res = {}
    for arm, learned in (("plain", 0), ("learned", 1), ("bound_only", 2)):
        sc = torch.empty(n, dtype=torch.int32, device=dev)
        ln = torch.empty(n, dtype=torch.int32, device=dev)
        cg = torch.zeros(batch.out_bytes, dtype=torch.uint8, device=dev)     # (compared whole below)
        fn = lambda: api.wfa_device(batch, smax, True, sc, ln, cg, stream=stream.cuda_stream, learned=learned)
        if arm == "learned" and tune_first:
            chosen, trials = api.autotune_wfa(batch, smax, True, sc, ln, cg, reps=2)
            out["tune"] = {"chosen": chosen, "trials": [dict(t, ms=round(ms, 3)) for t, ms in trials]}
        for _ in range(3):
            fn()
        ms = timed(fn, stream, steps, flush)
        out[arm] = {"pairs_per_s": n / (ms * 1e-3), "ms_per_step": ms}
        # one more call with per-kernel events (outside the timed calls)
        torch.cuda.synchronize()
        api.profile(True)
        fn()
        torch.cuda.synchronize()
        api.profile(False)
        out[arm]["kernel_ms_one_call"] = {k: round(v[0], 4) for k, v in api.profile_read().items()}
        res[arm] = (sc.cpu().numpy(), ln.cpu().numpy(), cg.cpu().numpy())
        if learned:
            fn()
            torch.cuda.synchronize()
            small, big, rest = api.wfa_route_stats()
            out[arm].update({"lane_queue_pairs": small, "warp_queue_pairs": big, "escalated": rest[0],
                             "escalation_rate": rest[0] / max(1, small), "whole_block_pairs": rest[1],
                             "unresolved_by_bound_or_search": int((res[arm][0] < 0).sum())})
            out[arm]["_items"] = api.wfa_route_items(n)
            out[arm]["bit_identical_to_plain"] = bool(all(np.array_equal(x, y) for x, y in zip(res["plain"], res[arm])))
    for arm in ("learned", "bound_only"):
        out[arm + "_over_plain"] = out["plain"]["ms_per_step"] / out[arm]["ms_per_step"]
    return res["plain"]


def wfa_e2e(api, ps, smax, learned, steps):
    """The same batch through the public host entry (ga_align_batch_ex: staging,
    copies, kernels, result checks on the device, results and CIGAR strings on
    the host): median wall ms, bytes each way, the last result."""
    reqs = api.make_requests(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax, True)
    res = np.zeros(ps.n, api.RES_DT)
    cig = np.empty(int(api.load().ga_align_cigar_bytes(reqs.ctypes.data, ps.n)), np.uint8)
    call = lambda: api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=smax,
                                          max_smax=max(smax, 511), learned=learned, _reqs=reqs, _res=res, _cig=cig)
    for _ in range(2):
        call()
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        r = call()
        t.append(time.perf_counter() - t0)
    h2d, d2h = api.last_transfer_bytes()
    return statistics.median(t) * 1e3, h2d, d2h, r


def bench_wfa_mixed(api, workloads, cost_model, torch, dev, stream, args, keep, n_pairs=None):
    """1,000,000 mixed-divergence pairs: plain fixed smax 64, the
    learned-bucketed form and the lower-bound-only queues, bit-exact check,
    misprediction rates per divergence class, end to end (learned form)."""
    ps = workloads.wfa_mixed(n=n_pairs or 1_000_000)
    n = ps.n
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    out = {"workload": "wfa_mixed_1m: 1,000,000 pairs, 150-250 bp, error 70% U[0,2%] / 25% U[2,10%] / "
                       "5% U[10,30%], smax 64, CIGAR", "model_loaded": cost_model.load_default(args.wfa_model)}
    if not out["model_loaded"]:
        return out
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    plain = wfa_arms(api, torch, dev, stream, batch, n, 64, extra_steps(args), flush, not args.no_tune, out)
    rate = ps.meta["rate"]
    classes = {"all": np.ones(n, bool), "low (<2%)": rate < 0.02, "mid (2-10%)": (rate >= 0.02) & (rate < 0.10),
               "high (>=10%)": rate >= 0.10}
    lane_ok = (ps.a_len <= LANE_MAXLEN) & (ps.b_len <= LANE_MAXLEN)      # every pair here is pure A/C/G/T
    lane_smax = api.tune_get()["wfa_lane_smax"]
    for arm in ("learned", "bound_only"):
        out[arm]["misprediction"] = route_report(out[arm].pop("_items"), plain[0], 64, lane_smax, classes, lane_ok)
    e2e_ms, h2d, d2h, r = wfa_e2e(api, ps, 64, True, extra_steps(args))
    out["e2e_learned"] = {"pairs_per_s": n / (e2e_ms * 1e-3), "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                          "d2h_bytes_per_step": d2h, "entry": "ga_align_batch_ex (learned = 1)"}
    keep["wfa_mixed_1m"] = {"ps": ps, "device": plain + (slot_ends(batch),), "e2e": r}
    return out


def bench_wfa_long(api, workloads, cost_model, torch, dev, stream, args, keep, n_pairs=None):
    """The long WFA batch at smax 2048: the plain form (one pair per warp, in
    batch order), the learned-bucketed form (queues by estimated distance,
    largest first; pairs estimated at s >= 256 on whole blocks) and the same
    queues keyed by the lower bound alone."""
    ps = workloads.wfa_long_1k_10k(n=n_pairs or 2_000)
    n = ps.n
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    out = {"workload": "wfa_long_1k_10k: 2,000 pairs, 1-10 kb, error 1-15%, geometric indels, smax 2048, CIGAR",
           "model_loaded": cost_model.load_default(args.wfa_model)}
    if not out["model_loaded"]:
        return out
    plain = wfa_arms(api, torch, dev, stream, batch, n, 2048, 3, None, False, out)
    lane_ok = np.zeros(n, bool)                    # 1-10 kb: never the lane queue
    for arm in ("learned", "bound_only"):
        items = out[arm].pop("_items")
        rep = route_report(items, plain[0], 2048, 0, {"all": np.ones(n, bool)}, lane_ok)
        d = plain[0].astype(np.int64)
        est_block = (items >= 0) & ((items & 0xFF) < ROUTE_BUCKETS) & ((items & 0xFF) >= 9)
        exact_block = (d < 0) | (np.ceil(1.25 * d + 2) >= 256)
        rep["all"]["whole_block_mispredicted_rate"] = float((est_block != exact_block).mean())
        out[arm]["misprediction"] = rep
    out.update({"pairs_per_s": out["plain"]["pairs_per_s"], "ms_per_step": out["plain"]["ms_per_step"],
                "unresolved": int((plain[0] < 0).sum())})
    out["learned_over_plain"] = out["plain"]["ms_per_step"] / out["learned"]["ms_per_step"]
    e2e_ms, h2d, d2h, r = wfa_e2e(api, ps, 2048, True, 3)
    out["e2e_learned"] = {"pairs_per_s": n / (e2e_ms * 1e-3), "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                          "d2h_bytes_per_step": d2h, "entry": "ga_align_batch_ex (max_smax 2048, learned = 1)"}
    keep["wfa_long"] = {"ps": ps, "device": plain + (slot_ends(batch),), "e2e": r}
    return out


def sw_long_subset(full):
    """The stratified subset of the long SW batch the CPU leg checks: its 64
    largest pairs and 64 more drawn at random."""
    cells = full.a_len.astype(np.int64) * full.b_len.astype(np.int64)
    order = np.argsort(-cells, kind="stable")
    rng = np.random.default_rng(55)
    return np.concatenate([order[:64], rng.choice(order[64:], size=64, replace=False)])


def bench_sw_long(api, workloads, torch, dev, stream, n_pairs, keep, tune=True):
    """The long SW batch (2-30 kb queries, 0-5 kb flanks), or its first n_pairs."""
    ps = workloads.sw_long_4k(n=n_pairs)
    cells = sw_cells(ps)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    n = ps.n
    sc = torch.empty(n, dtype=torch.int32, device=dev)
    pos = torch.empty(4 * n, dtype=torch.int32, device=dev)
    ln = torch.empty(n, dtype=torch.int32, device=dev)
    cg = torch.empty(batch.out_bytes, dtype=torch.uint8, device=dev)
    fn = lambda: api.sw_device(batch, SCORING, True, sc, pos, ln, cg, stream=stream.cuda_stream,
                               trace_cell_limit=-1)
    # the autotuner's setting for this batch (variants picked per pair: 16-bit
    # pairs two per warp, 32-bit pairs one per warp or, above the threshold, one
    # per block), then the plain single-variant form: every pair one per warp
    # in 32 bits
    saved = api.tune_get()
    if tune:
        chosen, trials = api.autotune_sw(batch, SCORING, sc, pos, ln, cg, reps=1)
    else:
        chosen, trials = saved, []
    fn()
    ms = timed(fn, stream, 1)
    out = sc.cpu().numpy().copy(), ln.cpu().numpy().copy()
    if n_pairs == 4096:
        idx = sw_long_subset(ps)
        ends = slot_ends(batch)[idx]
        keep["sw_long"] = {"ps": ps.subset(idx), "device": (out[0][idx], pos.cpu().numpy().reshape(-1, 4)[idx],
                                                             out[1][idx], cg.cpu().numpy(), ends)}
    # the SW variant model's routing: pure pairs beyond the proven 16-bit
    # bound try the 16-bit kernel when the model predicts their score fits
    # (the two-pairs-per-warp kernel on, the tuned fields otherwise kept)
    learned = None
    from genoaligner_gb300 import sw_model
    if sw_model.load_default():
        api.tune_set(**dict(chosen, sw_pack16=1))
        fl = lambda: api.sw_device(batch, SCORING, True, sc, pos, ln, cg, stream=stream.cuda_stream,
                                   trace_cell_limit=-1, learned=True)
        fl()
        ms_l = timed(fl, stream, 1)
        learned = {"form": "the autotuner's setting with sw_pack16 1 and the 16-bit choice by the SW variant model",
                   "gcups": cells / (ms_l * 1e-3) / 1e9, "ms_per_step": ms_l,
                   "bit_identical_to_tuned": bool(np.array_equal(out[0], sc.cpu().numpy()) and
                                                  np.array_equal(out[1], ln.cpu().numpy()))}
        api.tune_set(**chosen)
    api.tune_set(**dict(saved, sw_pack16=0, sw_coop_log2=40))
    fn()
    ms_plain = timed(fn, stream, 1)
    same = bool(np.array_equal(out[0], sc.cpu().numpy()) and np.array_equal(out[1], ln.cpu().numpy()))
    api.tune_set(**saved)
    return {"workload": f"sw_long_4k ({n} of 4,096 pairs): query 2-30 kb at 10%, 0-5 kb flanks, "
                        "scoring {2,-3,3,1}, score+CIGAR, no trace-cell limit",
            "gcups": cells / (ms * 1e-3) / 1e9, "ms_per_step": ms, "cells": cells,
            "tune": {"chosen": chosen, "trials": [dict(t, ms=round(m, 1)) for t, m in trials]},
            "learned_variant": learned,
            "plain_single_variant": {"form": "every pair one per warp, int32 (sw_pack16 0, no whole-block pairs)",
                                     "gcups": cells / (ms_plain * 1e-3) / 1e9, "ms_per_step": ms_plain},
            "bit_identical_to_plain": same}


def bench_sw_score_only(api, torch, dev, stream, args, ps, batch, trace_scores):
    """The headline batch without traceback: score and end cell per pair
    (the reference's score-only path), on the device and end to end."""
    n = ps.n
    cells = sw_cells(ps)
    sc = torch.empty(n, dtype=torch.int32, device=dev)
    pos = torch.empty(4 * n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    fn = lambda: api.sw_device(batch, SCORING, False, sc, pos, None, None, stream=stream.cuda_stream)
    for _ in range(3):
        fn()
    ms = timed(fn, stream, extra_steps(args), flush)
    same = bool(np.array_equal(sc.cpu().numpy(), trace_scores))
    reqs = api.make_sw_requests(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING, False)
    res = np.zeros(n, api.SWRES_DT)
    call = lambda: api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING,
                                             with_cigar=False, _reqs=reqs, _res=res)
    for _ in range(2):
        call()
    t = []
    for _ in range(extra_steps(args)):
        t0 = time.perf_counter()
        r = call()
        t.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(t) * 1e3
    same = same and r.status == api.Status.ok and bool(np.array_equal(r.res["score"], trace_scores))
    return {"workload": SW_WORKLOAD.replace("score+end+start+CIGAR", "score + end cell (score-only)"),
            "pairs": n, "cells": cells, "gcups": cells / (ms * 1e-3) / 1e9, "ms_per_step": ms,
            "e2e_gcups": cells / (e2e_ms * 1e-3) / 1e9, "e2e_ms_per_step": e2e_ms,
            "l2": "256 MB buffer written between steps",
            "scores_equal_traceback_run": same}


def cpu_and_parity(keep, ps_sw, sw_e2e, sw_dev_scores, threads):
    """The CPU oracle on every workload, which is both the CPU baseline and the
    full-size parity check of this run's GPU outputs.  All host threads over
    the whole batch (the long SW batch: its stratified 128-pair subset, on as
    many threads as host memory allows), timed on the C calls alone; one
    thread on a bounded sample of each; edit_distance_cpu on a sample of the
    mixed batch.  Returns (cpu figures, parity booleans)."""
    import oracle
    cpu, parity = {}, {}

    def wfa_leg(key, smax, unit_seconds):
        k = keep.get(key)
        if not k:
            return
        ps = k["ps"]
        pats, txts = ps.lists()
        want = oracle.wfa_batch(pats, txts, smax=smax, with_cigar=True, threads=threads, max_smax=max(smax, 511))
        parity[key] = {"device_plain": wfa_equal_device(k["device"], want),
                       "e2e": wfa_equal_packed(k["e2e"], want), "pairs": ps.n}
        # all threads: further passes over the batch until ~unit_seconds of C
        # time (or 20 s of wall time)
        passes, secs, w0 = 1, want.seconds, time.perf_counter()
        while secs < unit_seconds and time.perf_counter() - w0 < 20.0:
            secs += oracle.wfa_batch(pats, txts, smax=smax, with_cigar=True, threads=threads,
                                     max_smax=max(smax, 511)).seconds
            passes += 1

        def run(idx):
            sub = ps.subset(idx)
            a, b = sub.lists()
            g = oracle.wfa_batch(a, b, smax=smax, with_cigar=True, threads=1, max_smax=max(smax, 511))
            return sub.n, g.seconds
        one, k1, t1 = one_core_sample(run, ps.n, unit_seconds, first=8 if smax > 511 else 256)
        cpu[key] = {"unit": "pairs/s", "all_cores": passes * ps.n / secs, "all_cores_threads": threads,
                    "all_cores_sample": f"the whole batch ({ps.n} pairs) x {passes}, {secs:.2f} s",
                    "one_core": one, "one_core_sample": f"{k1} pairs, {t1:.2f} s"}

    wfa_leg("wfa_150bp", 64, 1.0)
    wfa_leg("wfa_long", 2048, 3.0)
    wfa_leg("wfa_mixed_1m", 64, 2.0)

    # edit_distance_cpu (src/reference/edit_distance_cpu.hpp) for scale, on
    # 20,000 pairs of the mixed batch
    if "wfa_mixed_1m" in keep:
        sub = keep["wfa_mixed_1m"]["ps"].subset(np.arange(20000))
        a, b = sub.lists()
        d1, t1 = oracle.edit_distance(a, b, threads=1, timing=True)
        dn, tn = oracle.edit_distance(a, b, threads=threads, timing=True)
        cpu["edit_distance_cpu"] = {"unit": "pairs/s", "one_core": sub.n / t1, "all_cores": sub.n / tn,
                                    "all_cores_threads": threads, "sample": "the mixed batch's first 20,000 pairs",
                                    "agrees_with_wfa_scores_within_smax": bool(np.array_equal(
                                        np.where(dn <= 64, dn, -1), keep["wfa_mixed_1m"]["device"][0][:20000]))}

    # the uneven SW batch, whole
    ts, pp = ps_sw.lists()
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, threads=threads)
    cells = sw_cells(ps_sw)
    parity["sw_uneven_200k"] = {"e2e": sw_equal_packed(sw_e2e, want),
                                "device_scores": bool(np.array_equal(sw_dev_scores, want.score)), "pairs": ps_sw.n}

    def run_sw(idx):
        sub = ps_sw.subset(idx)
        a, b = sub.lists()
        g = oracle.sw_batch(a, b, scoring=SCORING, with_cigar=True, threads=1)
        return sw_cells(sub), g.seconds
    one, k1, t1 = one_core_sample(run_sw, ps_sw.n, 3.0, first=64, cap=4096)
    cpu["sw_uneven_200k"] = {"unit": "GCUPS", "all_cores": cells / want.seconds / 1e9, "all_cores_threads": threads,
                             "all_cores_sample": f"the whole batch ({ps_sw.n} pairs, {cells / 1e9:.2f} Gcells), "
                                                 f"{want.seconds:.2f} s",
                             "one_core": one / 1e9 if one else None, "one_core_sample": f"{k1} pairs, {t1:.2f} s"}
    sw_all = (cells / want.seconds / 1e9, want.seconds)
    del want

    # the long SW batch: its stratified subset
    k = keep.get("sw_long")
    if k:
        ps = k["ps"]
        cl = ps.a_len.astype(np.int64) * ps.b_len.astype(np.int64)
        try:
            avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
        except (ValueError, OSError):
            avail = 16 << 30
        th = int(max(1, min(threads, avail // 2 // int(cl.max() * 1.1))))
        ts, pp = ps.lists()
        want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, threads=th, trace_cell_limit=-1)
        parity["sw_long_4k_subset"] = {"device": sw_equal_device(k["device"], want), "pairs": ps.n,
                                       "subset": "the 64 largest pairs (0.5-1.2 Gcells) and 64 drawn at random"}
        # one thread: the subset's smallest pairs, about 0.4 Gcells (1-2 s)
        order = np.argsort(cl)
        k1 = int(np.searchsorted(np.cumsum(cl[order]), 4e8)) + 1
        sub = ps.subset(order[:k1])
        a, b = sub.lists()
        g = oracle.sw_batch(a, b, scoring=SCORING, with_cigar=True, threads=1, trace_cell_limit=-1)
        cpu["sw_long_4k"] = {"unit": "GCUPS", "all_cores": int(cl.sum()) / want.seconds / 1e9, "all_cores_threads": th,
                             "all_cores_sample": f"the stratified subset ({ps.n} pairs, {cl.sum() / 1e9:.1f} Gcells), "
                                                 f"{want.seconds:.2f} s",
                             "one_core": sw_cells(sub) / g.seconds / 1e9,
                             "one_core_sample": f"the subset's {k1} smallest pairs ({sw_cells(sub) / 1e9:.2f} Gcells), "
                                                f"{g.seconds:.2f} s"}
        del want
    return cpu, parity, sw_all


def score_only_alone(api, workloads, torch, dev, stream, args):
    """The score-only line on the first --pairs pairs of the headline batch
    (one traceback call first gives the scores it is compared with)."""
    ps = workloads.sw_uneven_200k(n=args.pairs)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device=dev)
    n = ps.n
    sc = torch.empty(n, dtype=torch.int32, device=dev)
    pos = torch.empty(4 * n, dtype=torch.int32, device=dev)
    ln = torch.empty(n, dtype=torch.int32, device=dev)
    cg = torch.empty(max(batch.out_bytes, 1), dtype=torch.uint8, device=dev)
    api.sw_device(batch, SCORING, True, sc, pos, ln, cg, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    return bench_sw_score_only(api, torch, dev, stream, args, ps, batch, sc.cpu().numpy())


def main():
    args = parse()
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from genoaligner_gb300 import api, cost_model, workloads
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.set_tune:
        fields = dict(kv.split("=") for kv in args.set_tune.split(","))
        api.tune_set(**dict(api.tune_get(), **{k: int(v) for k, v in fields.items()}))
        args.no_tune = True

    if args.only:
        stream = torch.cuda.current_stream(dev)
        keep = {}
        m = args.only_pairs
        run = {"wfa_150bp": lambda: bench_wfa_150(api, workloads, torch, dev, stream, args, keep),
               "wfa_mixed_1m": lambda: bench_wfa_mixed(api, workloads, cost_model, torch, dev, stream, args, keep, m),
               "wfa_long": lambda: bench_wfa_long(api, workloads, cost_model, torch, dev, stream, args, keep, m),
               "sw_long": lambda: bench_sw_long(api, workloads, torch, dev, stream, m or 4096, keep,
                                                not args.no_tune),
               "sw_score_only": lambda: score_only_alone(api, workloads, torch, dev, stream, args)}[args.only]
        if rank == 0:
            print(json.dumps({args.only: run()}), flush=True)
        return

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

    # the autotuner picks this device's kernel setting on the batch itself
    # (untimed, like the warm-up; every setting gives the same results)
    if args.no_tune:
        tune = {"chosen": api.tune_get(), "trials": [], "by": "built-in default"}
    else:
        chosen, trials = api.autotune_sw(batch, SCORING, out_score, out_pos, out_len, out_cig, reps=2)
        tune = {"chosen": chosen, "trials": [dict(t, ms=round(ms, 3)) for t, ms in trials],
                "by": "ga_autotune_sw on this batch (wall time per call, coordinate search)"}

    clocks = Clocks(local)
    clocks.wait_first()
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    launches0 = api.kernel_launches()
    api.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.mark_begin()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.mark_end()
    api.profile(False)
    barrier(world)
    launches = api.kernel_launches() - launches0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world)
    prof = api.profile_read()
    value = world * cells / (ms * 1e-3) / 1e9

    # dominant kernel and its roofline: the trace kernels together process
    # every cell of the batch once per step (one launch each per step)
    total_ms = sum(v[0] for v in prof.values())
    top_name, (top_ms, top_n) = max(prof.items(), key=lambda kv: kv[1][0])
    sw_names = [k for k in prof if k.startswith("sw")]
    sw_ms = sum(prof[k][0] for k in sw_names)
    achieved = cells * args.steps / (sw_ms * 1e-3) / 1e9 if sw_ms > 0 else 0.0
    dpx = api.int_peak(1)
    peak = dpx / OPS_PER_CELL / 1e9
    roofline = {"bound": "dpx", "achieved": achieved, "peak": peak, "unit": "GCUPS",
                "frac": achieved / peak if peak else None,
                "traffic": SW16CK_DRAM_BYTES_PER_CELL * cells if top_name == "sw16x2_trace" else None,
                "kernel": top_name, "kernels_counted": sw_names, "ops_per_cell": OPS_PER_CELL,
                "peak_source": f"measured by peak.cu on this GPU: __viaddmax_s32 at {dpx / 1e12:.2f} T "
                               "lane-instructions/s, / 6 per cell (not in MEASURED_PEAKS.json, which holds "
                               "HBM and bf16 peaks)",
                "kernel_ms_per_launch": top_ms / max(1, top_n), "kernel_share": top_ms / total_ms if total_ms else None,
                "frac_of_int16x2_ceiling": achieved / (2 * peak) if peak else None,
                "int16x2_ceiling": "the 16-bit kernel's own ceiling: __viaddmax_s16x2 retires at the __viaddmax_s32 "
                                   "rate with two cells per lane-instruction, so 2 x the int32 roofline",
                "traffic_source": "profiles/sw16ck_trace_sw_uneven.md (bytes/cell x cells per launch)"}

    sc = out_score.cpu().numpy()            # checked against the oracle below

    # e2e through the public C ABI with host buffers
    reqs = api.make_sw_requests(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING, True)
    res = np.zeros(n, api.SWRES_DT)
    cig = np.empty(int(api.load().ga_align_sw_cigar_bytes(reqs.ctypes.data, n)), np.uint8)
    call = lambda: api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, SCORING,
                                             _reqs=reqs, _res=res, _cig=cig)
    for _ in range(2):
        call()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = call()
    e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
    e2e_ms = max_over_ranks(e2e_ms, world)
    h2d, d2h = api.last_transfer_bytes()

    extra, keep = {}, {}
    if not args.no_extra:
        extra["sw_score_only"] = bench_sw_score_only(api, torch, dev, stream, args, ps, batch, sc)
        extra["wfa_150bp"] = bench_wfa_150(api, workloads, torch, dev, stream, args, keep)
        extra["wfa_mixed_1m"] = bench_wfa_mixed(api, workloads, cost_model, torch, dev, stream, args, keep)
        extra["wfa_long"] = bench_wfa_long(api, workloads, cost_model, torch, dev, stream, args, keep)
        extra["sw_long"] = bench_sw_long(api, workloads, torch, dev, stream, 4096, keep, not args.no_tune)

    # the CPU leg (rank 0, after every GPU measurement): the oracle over each
    # workload is the CPU baseline and the full-size parity check at once
    cpu = cpu_all = parity = None
    if rank == 0:
        threads = os.cpu_count() or 1
        cpu_all, parity, (g, secs) = cpu_and_parity(keep, ps, r, sc, threads)
        cpu = {"value": g, "unit": "GCUPS", "cores": threads, "kind": "port",
               "build": "oracle/ga_oracle.c, gcc -O3 (no -march: the same code on x86 and Arm)",
               "sample": f"the whole batch ({n} pairs, {cells / 1e9:.2f} Gcells) in one pass on all host threads, "
                         f"{secs:.1f} s of C time"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int16x2/int32", "data": "synthetic (seeded generator, seed 2)",
            "config": {"workload": SW_WORKLOAD, "pairs": n, "cells": cells, "tune": tune,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "inputs (%.0f MB) and checkpoint/edge stores exceed the 129 MB L2" %
                             (batch.input_bytes / 1e6)},
            "e2e": {"value": world * cells / (e2e_ms * 1e-3) / 1e9, "unit": "GCUPS", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "cpu_baselines": cpu_all,
            "clocks": clk,
            "parity_full": parity,
            "parity_ok": bool(parity) and all(v for d in parity.values() for k, v in d.items()
                                              if isinstance(v, bool)),
            "parity": "every workload's GPU outputs against the oracle, every field of every pair (the long SW "
                      "batch on its stratified subset)",
            "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()},
            "extra": extra,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
