"""gene_qc: pairwise QC of protein-coding gene FASTA files on the GPU.

The same task, arguments and TSV as the reference's tools/gene_qc.cpp: every
record of a gene file is aligned (Smith-Waterman with CIGAR) to one bait
chosen from a reference file, and each CIGAR is walked for coverage,
frameshifts and in-frame stop codons.  Here the path stays on the device:

  1. both FASTA files are read into pinned, device-ready arenas (ga_fasta_*);
     the record arena goes to the GPU in one copy, the bait once after it;
  2. one ga_sw_device call aligns every record to the bait (the records are
     the text axis, the bait the pattern axis, as in the reference tool);
  3. ga_sw_qc_device walks every CIGAR where the kernels left it and
     ga_sw_validate_device checks it, so only scores, spans and four QC
     integers per record come back to the host.

Bait choice (host, tools/gene_qc.cpp:118-136): for each bait record the frame
with the fewest stop codons; fewest overall wins, ties to a frame starting
with ATG, then to the longer record.  Flags (:223-232): NO_ALIGN when the pair
is unresolved or scores <= --min-score, else LOW_COV (coverage of the record
below --min-cov), FS=<net> when the net indel length is not a multiple of 3,
STOP=<n> for in-frame stops other than the span's own terminator, OK when
none applies.

    python -m genoaligner_gb300.gene_qc seqs.fasta --ref ref.fasta [--code 1|2]
        [--emit out.tsv] [--scoring m,x,go,ge] [--min-cov f] [--min-score n]
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from . import api

SW_MAX_TRACE_CELLS = 1 << 26
HEADER = "acc\tlen\tscore\tsi\tsj\tei\tej\tcov_text\tfs_runs\tfs_net\tstops\tstop_end\tflag\n"


def is_stop(a: int, b: int, c: int, code: int) -> bool:
    """Stop codon of genetic code 1 (standard) or 2 (vertebrate mitochondrial)."""
    if a == 84 and b == 65 and c in (65, 71):                  # TAA TAG
        return True
    if code == 1 and a == 84 and b == 71 and c == 65:          # TGA
        return True
    if code == 2 and a == 65 and b == 71 and c in (65, 71):    # AGA AGG
        return True
    return False


def stops_in_frame(s: bytes, frame: int, code: int) -> int:
    return sum(1 for i in range(frame, len(s) - 2, 3) if is_stop(s[i], s[i + 1], s[i + 2], code))


def pick_bait(seqs, code: int):
    """(index, frame, stops) of the bait: fewest stops over records and frames,
    ties to an ATG-led frame, then to the longer record."""
    best, best_stops, frame, best_atg = 0, 1 << 30, 0, False
    for r, s in enumerate(seqs):
        for f in range(3):
            st = stops_in_frame(s, f, code)
            atg = f + 2 < len(s) and s[f:f + 3] == b"ATG"
            better = (st < best_stops or (st == best_stops and atg and not best_atg) or
                      (st == best_stops and atg == best_atg and len(s) > len(seqs[best])))
            if better:
                best_stops, best, frame, best_atg = st, r, f, atg
    return best, frame, best_stops


def scheme_error(sc):
    """The SW scheme checks of align_sw_batch (None when the scheme is valid)."""
    m, x, go, ge = sc
    if m <= 0:
        return "SW scoring: match must be > 0 (the score is 0 for every input otherwise)"
    if x >= m:
        return "SW scoring: mismatch must be < match"
    if go <= 0 or ge <= 0:
        return "SW scoring: gap costs must be > 0"
    if ge > go:
        return ("SW scoring: gap_extend > gap_open with with_cigar cannot re-score to its own score (api.hpp; "
                "RESULTADO_H9_SW2_TRACE.md). Score-only requests may use it")
    return None


def run(seqs_path: str, ref_path: str, code: int = 1, scoring=(1, -1, 2, 1), min_cov: float = 0.5,
        min_score: int = 0, device: str = "cuda:0"):
    """Align and check every record; returns (rows, info) with rows the TSV
    lines (without the header) and info the bait choice and summary counts."""
    import torch
    recs = api.fasta_read(seqs_path)
    refs = api.fasta_read(ref_path)
    bait_seqs = [refs.sequence(i) for i in range(refs.n)]
    bi, frame, bait_stops = pick_bait(bait_seqs, code)
    bait = bait_seqs[bi]
    n = recs.n
    # one device arena: the record arena as read, then the bait
    base = recs.arena.nbytes
    seq = torch.zeros(base + (len(bait) + 31) // 32 * 32 + 64, dtype=torch.uint8, device=device)
    recs.upload(seq)
    seq[base:base + len(bait)] = torch.frombuffer(bytearray(bait), dtype=torch.uint8).to(device)
    a_len = recs.lengths.copy()
    batch = api.DeviceBatchT.from_device_arena(seq, recs.offsets.copy(), a_len, np.full(n, base, np.int64),
                                               np.full(n, len(bait), np.int32))
    sc = torch.empty(n, dtype=torch.int32, device=device)
    pos = torch.empty(4 * n, dtype=torch.int32, device=device)
    ln = torch.empty(n, dtype=torch.int32, device=device)
    cg = torch.empty(max(batch.out_bytes, 1), dtype=torch.uint8, device=device)
    qc = torch.empty(4 * n, dtype=torch.int32, device=device)
    vf = torch.empty(n, dtype=torch.uint8, device=device)
    api.sw_device(batch, scoring, True, sc, pos, ln, cg, trace_cell_limit=SW_MAX_TRACE_CELLS)
    api.sw_validate_device(batch, scoring, sc, pos, ln, cg, vf)
    api.sw_qc_device(batch, sc, pos, ln, cg, frame, code, qc)
    torch.cuda.synchronize()
    score, p4, q4, flags = sc.cpu().numpy(), pos.cpu().numpy().reshape(-1, 4), qc.cpu().numpy().reshape(-1, 4), \
        vf.cpu().numpy()
    rows = []
    cnt = {"OK": 0, "NO_ALIGN": 0, "LOW_COV": 0, "FS": 0, "STOP": 0, "invalid": 0}
    for k in range(n):
        s = int(score[k])
        tlen = int(a_len[k])
        resolved = s >= 0
        if not resolved:                    # above the trace limit: the defaults of an unresolved result
            s, si, sj, ei, ej = -1, -1, -1, -1, -1
        elif s == 0:
            si, sj, ei, ej = -1, -1, int(p4[k, 2]), int(p4[k, 3])
        else:
            si, sj, ei, ej = (int(v) for v in p4[k])
        fs, fs_net, stops, stop_end = (int(v) for v in q4[k])
        cov = (ei - si + 1) / tlen if resolved and s > 0 else 0.0
        if not resolved or s <= min_score:
            flag = "NO_ALIGN"
        else:
            flag = "LOW_COV" if cov < min_cov else ""
            if fs_net != 0:
                flag += ("+" if flag else "") + f"FS={fs_net}"
            if stops > 0:
                flag += ("+" if flag else "") + f"STOP={stops}"
            if not flag:
                flag = "OK"
        rows.append(f"{recs.ids[k]}\t{tlen}\t{s}\t{si}\t{sj}\t{ei}\t{ej}\t{cov:.3f}\t{fs}\t{fs_net}\t{stops}\t"
                    f"{stop_end}\t{flag}\n")
        if flag == "OK":
            cnt["OK"] += 1
        else:
            for key, pat in (("NO_ALIGN", "NO_ALIGN"), ("LOW_COV", "LOW_COV"), ("FS", "FS="), ("STOP", "STOP=")):
                if pat in flag:
                    cnt[key] += 1
        if resolved and s > 0 and flags[k] != 3:
            cnt["invalid"] += 1
    info = {"records": n, "bait": refs.ids[bi], "bait_len": len(bait), "frame": frame, "bait_stops": bait_stops,
            "code": code, **cnt}
    recs.close()
    refs.close()
    return rows, info


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="gene_qc", description="pairwise QC of a gene FASTA against its bait, on the GPU")
    ap.add_argument("seqs")
    ap.add_argument("--ref", required=True)
    ap.add_argument("--code", type=int, default=1, choices=[1, 2])
    ap.add_argument("--emit")
    ap.add_argument("--scoring", default="1,-1,2,1")
    ap.add_argument("--min-cov", type=float, default=0.5)
    ap.add_argument("--min-score", type=int, default=0)
    ap.add_argument("--batch-size", type=int, default=400, help="accepted for compatibility; one batch is used")
    a = ap.parse_args(argv)
    scoring = tuple(int(v) for v in a.scoring.split(","))
    err = scheme_error(scoring)
    if err:
        print(f"batch: {err}", file=sys.stderr)
        return 1
    try:
        rows, info = run(a.seqs, a.ref, a.code, scoring, a.min_cov, a.min_score)
    except ValueError as e:
        print(f"fasta error: {e}", file=sys.stderr)
        return 1
    print(f"gene_qc: {info['records']} records vs ref {info['bait']} ({info['bait_len']} bp, frame {info['frame']}, "
          f"bait_stops {info['bait_stops']}, code {info['code']}) on {api.backend_name()}")
    if info["bait_stops"] > 0:
        print(f"WARN: bait itself carries {info['bait_stops']} stops in its best frame -- stop counts for this gene "
              "are weak evidence", file=sys.stderr)
    out = open(a.emit, "w") if a.emit else sys.stdout
    out.write(HEADER)
    out.writelines(rows)
    if a.emit:
        out.close()
    print(f"summary: {info['records']} seqs | OK={info['OK']} NO_ALIGN={info['NO_ALIGN']} LOW_COV={info['LOW_COV']} "
          f"FS={info['FS']} STOP={info['STOP']} | invalid={info['invalid']}", file=sys.stderr)
    return 1 if info["invalid"] else 0


if __name__ == "__main__":
    sys.exit(main())
