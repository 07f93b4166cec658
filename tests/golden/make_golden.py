#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs here only (it needs the reference checkout at REF_ROOT, default
/root/reference).  It builds oracle/_ref/libgaref.so -- the reference's own
wfa_trace_kernel / wfa_score_kernel_flat / sw_trace_kernel / sw_score_kernel
bodies and src/api/api.cpp compiled for the host with the reference's CPU shim
(oracle/ref_wrap.cpp) -- and records their outputs on:

* WFA: the reference's control set (tests/parity/data/control_seed12345.tsv,
  1000 pairs) at smax 64 on the trace and score-only paths; the hand cases of
  tests/parity/traceback_cpu.cpp and the reproducers of
  tests/parity/wfa_diag.cpp; exhaustive short pairs; seeded random batches
  with non-ACGT bytes, empty sides, several smax values and batch-min-smax.
* SW: the documented example and known answers of tests/api/test_api.cpp; the
  hand cases of tests/sw/test_sw_reference.cpp; seeded random batches under
  the schemes the reference gates ({1,-1,2,1}, {2,-3,3,1}, {2,-3,5,2}); mixed
  with_cigar batches; score-only batches (the warp kernel's end-cell rule,
  run under the shim's real-thread warp emulation), including gap_extend >
  gap_open.

Output: tests/golden/wfa_golden.json.gz and tests/golden/sw_golden.json.gz,
one record per batch: inputs, batch parameters and every result field.
"""
from __future__ import annotations

import ctypes
import gzip
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_ROOT = os.environ.get("REF_ROOT", "/root/reference")


def build_ref():
    r = subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_ROOT={REF_ROOT}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        sys.exit("cannot build oracle/_ref:\n" + r.stdout + r.stderr)
    L = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libgaref.so"))
    c = ctypes
    L.ref_wfa_pair.argtypes = [c.c_char_p, c.c_int, c.c_char_p, c.c_int, c.c_int, c.c_int, c.c_int,
                               c.c_char_p, c.POINTER(c.c_int), c.POINTER(c.c_int), c.POINTER(c.c_int)]
    L.ref_wfa_pair.restype = c.c_int
    L.ref_edit_distance.argtypes = [c.c_char_p, c.c_int, c.c_char_p, c.c_int]
    L.ref_sw_batch.argtypes = [c.c_int, c.c_void_p, c.c_void_p, c.c_void_p, c.c_void_p,
                               c.c_int, c.c_int, c.c_int, c.c_int, c.c_void_p, c.c_void_p,
                               c.c_void_p, c.c_void_p, c.c_void_p, c.POINTER(c.c_char_p)]
    L.ref_sw_batch.restype = c.c_int
    return L


def wfa_batch(L, pats, txts, smaxs, wants):
    """align_batch semantics over the reference kernels: batch smax = min,
    trace path iff any with_cigar, CIGAR capacity = max(m+n+2)."""
    smax = min(smaxs)
    trace = any(wants)
    cap = max(1, max(len(p) + len(t) + 2 for p, t in zip(pats, txts)))
    res = []
    for p, t in zip(pats, txts):
        buf = ctypes.create_string_buffer(len(p) + len(t) + 8)
        cl, rs, wf = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        s = L.ref_wfa_pair(p, len(p), t, len(t), smax, int(trace), cap, buf,
                           ctypes.byref(cl), ctypes.byref(rs), ctypes.byref(wf))
        res.append({"score": s, "resolved": int(s >= 0), "cigar": buf.raw[:cl.value].decode("latin-1"),
                    "rescore_ok": rs.value, "wellformed_ok": wf.value})
    return {"kind": "wfa", "pairs": [[p.decode("latin-1"), t.decode("latin-1")] for p, t in zip(pats, txts)],
            "smax": list(smaxs), "with_cigar": [int(w) for w in wants], "results": res,
            "resolved_count": sum(r["resolved"] for r in res),
            "unresolved_count": sum(1 - r["resolved"] for r in res)}


def sw_batch(L, txts, pats, scheme, wants):
    n = len(txts)
    tb = [ctypes.c_char_p(t) for t in txts]
    pb = [ctypes.c_char_p(p) for p in pats]
    tarr = (ctypes.c_char_p * n)(*tb)
    parr = (ctypes.c_char_p * n)(*pb)
    tl = np.array([len(t) for t in txts], np.int32)
    pl = np.array([len(p) for p in pats], np.int32)
    w = np.array([1 if x else 0 for x in wants], np.uint8)
    fields = np.zeros(n * 9, np.int32)
    per = tl.astype(np.int64) + pl + 8
    off = np.zeros(n, np.int64)
    off[1:] = np.cumsum(per)[:-1]
    cig = ctypes.create_string_buffer(int(per.sum()) + 8)
    clen = np.zeros(n, np.int32)
    err = ctypes.c_char_p()
    st = L.ref_sw_batch(n, ctypes.cast(tarr, ctypes.c_void_p), tl.ctypes.data,
                        ctypes.cast(parr, ctypes.c_void_p), pl.ctypes.data, *scheme,
                        w.ctypes.data, fields.ctypes.data, ctypes.cast(cig, ctypes.c_void_p),
                        off.ctypes.data, clen.ctypes.data, ctypes.byref(err))
    names = ["score", "resolved", "start_i", "start_j", "end_i", "end_j", "rescore_ok",
             "wellformed_ok", "too_large"]
    res = []
    raw = cig.raw
    for i in range(n):
        r = {k: int(fields[i * 9 + j]) for j, k in enumerate(names)}
        r["cigar"] = raw[off[i]:off[i] + clen[i]].decode("latin-1")
        res.append(r)
    status = ["ok", "invalid_argument", "device_error"][st]
    return {"kind": "sw", "pairs": [[t.decode("latin-1"), p.decode("latin-1")] for t, p in zip(txts, pats)],
            "scoring": list(scheme), "with_cigar": [int(x) for x in wants], "status": status,
            "error": err.value.decode() if err.value else None, "results": res,
            "resolved_count": sum(r["resolved"] for r in res),
            "unresolved_count": sum(1 - r["resolved"] for r in res)}


def rand_seq(rng, n, alpha=b"ACGT"):
    a = np.frombuffer(alpha, np.uint8)
    return a[rng.integers(0, len(alpha), size=n)].tobytes()


def mutate(rng, s, rate, alpha=b"ACGT"):
    out = bytearray()
    for ch in s:
        if rng.random() < rate:
            t = rng.integers(0, 3)
            if t == 0:
                out.append(alpha[rng.integers(0, len(alpha))])
            elif t == 1:
                out.append(ch)
                out.append(alpha[rng.integers(0, len(alpha))])
        else:
            out.append(ch)
    return bytes(out)


def main():
    L = build_ref()
    wfa = []
    # 1. the reference's own control set
    tsv = os.path.join(REF_ROOT, "tests/parity/data/control_seed12345.tsv")
    pats, txts = [], []
    with open(tsv) as f:
        for line in f:
            if line.startswith("#") or line.startswith("pattern\t"):
                continue
            cols = line.rstrip("\n").split("\t")
            pats.append(cols[0].encode())
            txts.append(cols[1].encode())
    n = len(pats)
    wfa.append(dict(wfa_batch(L, pats, txts, [64] * n, [True] * n), name="control_seed12345_trace_smax64"))
    wfa.append(dict(wfa_batch(L, pats, txts, [64] * n, [False] * n), name="control_seed12345_score_smax64"))
    # 2. hand cases and reproducers (traceback_cpu.cpp:344-359, wfa_diag.cpp:90-96,
    #    test_api.cpp:104-137, 187-210, 291-330)
    hand = [(b"ACGT", b"ACGT"), (b"ACGT", b"ACGA"), (b"ACGTA", b"ACGT"), (b"ACGT", b"ACGTA"),
            (b"GG", b"TTT"), (b"C", b"GT"), (b"CT", b"CCC"), (b"CG", b"GAC"), (b"A", b"AA"),
            (b"", b""), (b"ACGT", b""), (b"", b"ACGT"), (b"AAAA", b"AAAAA"),
            (b"ACGTACGT", b"TTTTTTTT"), (b"ACGTACGT", b"ACGTTCGT"), (b"AAAA", b"AAAA"),
            (b"AC", b"AC")]
    hp = [h[0] for h in hand]
    ht = [h[1] for h in hand]
    for smax in (0, 1, 2, 8, 32, 64, 128):
        wfa.append(dict(wfa_batch(L, hp, ht, [smax] * len(hp), [True] * len(hp)), name=f"hand_trace_smax{smax}"))
        wfa.append(dict(wfa_batch(L, hp, ht, [smax] * len(hp), [False] * len(hp)), name=f"hand_score_smax{smax}"))
    lens = [8, 40, 120, 300, 55]
    hp2, ht2 = [], []
    for Lh in lens:
        t = bytes(b"ACGT"[i % 4] for i in range(Lh))
        p = bytearray(t)
        p[Lh // 2] = ord("C") if p[Lh // 2] == ord("A") else ord("A")
        hp2.append(bytes(p))
        ht2.append(t)
    wfa.append(dict(wfa_batch(L, hp2, ht2, [64] * 5, [True] * 5), name="heterogeneous_lengths"))
    # 3. exhaustive short pairs over {A,C} (both lengths <= 4)
    import itertools
    words = [b""] + [bytes(w) for k in range(1, 5) for w in itertools.product(b"AC", repeat=k)]
    ep = [a for a in words for b in words]
    et = [b for a in words for b in words]
    wfa.append(dict(wfa_batch(L, ep, et, [8] * len(ep), [True] * len(ep)), name="exhaustive_AC_len4_smax8"))
    wfa.append(dict(wfa_batch(L, ep, et, [2] * len(ep), [True] * len(ep)), name="exhaustive_AC_len4_smax2"))
    # 4. seeded random batches
    rng = np.random.default_rng(20261203)
    for name, alpha, nb, maxlen, rate, smax in [
        ("random_acgt_short", b"ACGT", 400, 60, 0.15, 16),
        ("random_acgt_mid", b"ACGT", 300, 400, 0.05, 64),
        ("random_acgtn_lower", b"ACGTNacgt", 300, 200, 0.05, 32),
        ("random_unrelated", b"ACGT", 200, 50, 1.0, 48),
        ("random_smax511", b"ACGT", 60, 1200, 0.2, 511),
    ]:
        ps, ts = [], []
        for _ in range(nb):
            ln = int(rng.integers(0, maxlen + 1))
            p = rand_seq(rng, ln, alpha)
            t = rand_seq(rng, int(rng.integers(0, maxlen + 1)), alpha) if rate >= 1.0 else mutate(rng, p, rate, alpha)
            ps.append(p)
            ts.append(t)
        wfa.append(dict(wfa_batch(L, ps, ts, [smax] * nb, [True] * nb), name=name + "_trace"))
        wfa.append(dict(wfa_batch(L, ps, ts, [smax] * nb, [False] * nb), name=name + "_score"))
    # batch-min-smax and mixed with_cigar (test_batch_semantics.cpp:98-132)
    ps = [rand_seq(rng, 100) for _ in range(40)]
    ts = [mutate(rng, p, 0.08) for p in ps]
    sm = [200 if i % 7 else 8 for i in range(40)]
    wc = [i % 3 == 0 for i in range(40)]
    wfa.append(dict(wfa_batch(L, ps, ts, sm, wc), name="min_smax_mixed_cigar"))

    sw = []
    # SW documented example and known answers (test_api.cpp:104-117, 403-477)
    sc = (2, -3, 5, 2)
    t6 = b"AACCGGTT" + b"C" * 6 + b"TTGGCCAA"
    kat_t = [b"TTTACGTGTT", b"ACGTACGT", t6, b"AAAAAAAA", b"ACGT", b"", b""]
    kat_p = [b"ACGTGT", b"ACGTACGT", b"AACCGGTTTTGGCCAA", b"CCCCCCCC", b"", b"ACGT", b""]
    sw.append(dict(sw_batch(L, kat_t, kat_p, sc, [True] * len(kat_t)), name="api_kats_trace"))
    sw.append(dict(sw_batch(L, kat_t, kat_p, sc, [False] * len(kat_t)), name="api_kats_score"))
    sw.append(dict(sw_batch(L, [b"ACGT"], [b"ACGT"], (2, -3, 1, 2), [False]), name="ge_gt_go_score_only"))
    # test_sw_reference.cpp hand cases under {1,-1,2,1}
    core = b"ACGTACGTACGT"
    ref_t = [b"T" * 10 + core + b"G" * 10, b"ACGT", b"A", b"A" * 20, b"AAAAAAAA", b"ACGTACGT",
             b"AAAAAA", b"A", b"ACGTACGT" + b"T" * 20, b"T" * 20 + b"ACGTACGT", b"ACGTTTACGT",
             b"ACACACAC", b"", b"ACGT", b""]
    ref_p = [b"C" * 10 + core + b"A" * 10, b"ACGT", b"A", b"A" * 20, b"CCCCCCCC", b"TGCATGCA",
             b"CCCCCC", b"C", b"ACGTACGT" + b"G" * 20, b"G" * 20 + b"ACGTACGT", b"ACGTACGT",
             b"ACAC", b"ACGT", b"", b""]
    sw.append(dict(sw_batch(L, ref_t, ref_p, (1, -1, 2, 1), [True] * len(ref_t)), name="sw_reference_hand_trace"))
    sw.append(dict(sw_batch(L, ref_t, ref_p, (1, -1, 2, 1), [False] * len(ref_t)), name="sw_reference_hand_score"))
    # seeded random batches
    rng = np.random.default_rng(20261204)
    for scheme in [(1, -1, 2, 1), (2, -3, 3, 1), (2, -3, 5, 2), (3, -2, 4, 4)]:
        ts = [rand_seq(rng, int(rng.integers(0, 140))) for _ in range(120)]
        ps = [rand_seq(rng, int(rng.integers(0, 140))) for _ in range(120)]
        sw.append(dict(sw_batch(L, ts, ps, scheme, [True] * 120), name=f"random_unrelated_{scheme}"))
        core = [rand_seq(rng, int(rng.integers(1, 300))) for _ in range(60)]
        ts = [rand_seq(rng, int(rng.integers(0, 100))) + mutate(rng, c, 0.1) + rand_seq(rng, int(rng.integers(0, 100)))
              for c in core]
        sw.append(dict(sw_batch(L, ts, core, scheme, [True] * 60), name=f"random_embedded_{scheme}"))
        wc = [bool(i % 2) for i in range(60)]
        sw.append(dict(sw_batch(L, ts, core, scheme, wc), name=f"random_embedded_mixed_{scheme}"))
    # N / lowercase bytes, repeats (ties), and score-only end-cell rule
    ts = [rand_seq(rng, int(rng.integers(1, 90)), b"ACGTNa") for _ in range(60)]
    ps = [rand_seq(rng, int(rng.integers(1, 90)), b"ACGTNa") for _ in range(60)]
    sw.append(dict(sw_batch(L, ts, ps, (2, -3, 3, 1), [True] * 60), name="random_nbytes_trace"))
    rep_t = [b"AC" * int(k) for k in rng.integers(1, 40, size=24)] + [b"A" * int(k) for k in rng.integers(1, 70, size=24)]
    rep_p = [b"AC" * int(k) for k in rng.integers(1, 40, size=24)] + [b"A" * int(k) for k in rng.integers(1, 70, size=24)]
    sw.append(dict(sw_batch(L, rep_t, rep_p, (1, -1, 2, 1), [True] * 48), name="repeats_trace"))
    sw.append(dict(sw_batch(L, rep_t, rep_p, (1, -1, 2, 1), [False] * 48), name="repeats_score"))
    for scheme in [(2, -3, 3, 1), (1, -1, 2, 1), (2, -3, 1, 2)]:
        ts = [rand_seq(rng, int(rng.integers(0, 80))) for _ in range(24)]
        ps = [rand_seq(rng, int(rng.integers(0, 80))) for _ in range(24)]
        core = [rand_seq(rng, int(rng.integers(1, 70))) for _ in range(24)]
        ts += [rand_seq(rng, int(rng.integers(0, 30))) + mutate(rng, c, 0.1) for c in core]
        ps += core
        sw.append(dict(sw_batch(L, ts, ps, scheme, [False] * 48), name=f"score_only_{scheme}"))

    for fname, recs in (("wfa_golden.json.gz", wfa), ("sw_golden.json.gz", sw)):
        with gzip.open(os.path.join(HERE, fname), "wt", compresslevel=9) as f:
            for r in recs:
                f.write(json.dumps(r, separators=(",", ":")) + "\n")
        print(fname, len(recs), "batches", sum(len(r["pairs"]) for r in recs), "pairs")


if __name__ == "__main__":
    main()
