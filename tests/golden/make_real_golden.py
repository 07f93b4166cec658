#!/usr/bin/env python3
"""Generate tests/golden/real_golden.json.gz: WFA batches on real sequences.

Runs here only (it needs the reference checkout at REF_ROOT, default
/root/reference).  The inputs are the two mitochondrial genomes the
reference's real-sequence test reads (tests/data/mtdna_human.fa, NC_012920.1,
16,569 bp with one N; tests/data/mtdna_chimp.fa, NC_001643.1, 16,554 bp),
cut into the batches that test aligns (tests/real/test_real_sequences.cpp):

1. 400 bp fragments of the human genome against themselves and against a
   copy with two substitutions, smax 64 with CIGAR;
2. the control region across the origin (1,169 bp, tandem repeats) against
   itself, a rotation by 3 and a copy with every 23rd base substituted,
   smax 64 with CIGAR;
3. co-linear human / chimp windows: 600 bp at smax 64 with CIGAR and at
   smax 200 score-only (all unresolved: d ~300), 100 bp at smax 64 with CIGAR
   (resolved);
4. the whole genomes, human / human and human / chimp, smax 511 score-only;
5. a 200 bp window around the human N against itself and its reverse,
   smax 200 score-only.

Every batch is run through the reference's own WFA kernels compiled for the
host (oracle/_ref, built by tests/golden/make_golden.py's recipe) and its
edit_distance_cpu; the fixture holds, one batch per line, its pairs,
parameters, every result field and the edit distances.
"""
from __future__ import annotations

import gzip
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402


def read_fasta_one(path: str) -> bytes:
    with open(path, "rb") as f:
        lines = f.read().splitlines()
    return b"".join(l.strip() for l in lines if l and not l.startswith(b">"))


def main():
    L = mg.build_ref()
    hum = read_fasta_one(os.path.join(mg.REF_ROOT, "tests/data/mtdna_human.fa"))
    chi = read_fasta_one(os.path.join(mg.REF_ROOT, "tests/data/mtdna_chimp.fa"))

    def sl(g, a, n):
        s = hum if g == "human" else chi
        return s[a:a + n]

    batches = []

    def add(name, pairs, smax, with_cigar):
        pats = [p for p, _ in pairs]
        txts = [t for _, t in pairs]
        rec = mg.wfa_batch(L, pats, txts, [smax] * len(pairs), [with_cigar] * len(pairs))
        rec["name"] = name
        rec["edit_distance"] = [int(L.ref_edit_distance(p, len(p), t, len(t))) for p, t in zip(pats, txts)]
        batches.append(rec)

    def flip(s: bytes, i: int, a: str, b: str) -> bytes:
        """base i becomes b where it is a, else a"""
        x = bytearray(s)
        x[i] = ord(b) if x[i] == ord(a) else ord(a)
        return bytes(x)

    # 1. fragments of one molecule: identical, two substitutions
    pairs = []
    for s in (1000, 3000, 4500, 6000, 9000, 12000, 15000):
        frag = sl("human", s, 400)
        if len(frag) < 400:
            continue
        pairs.append((frag, frag))
        pairs.append((frag, flip(flip(frag, 10, "A", "C"), 200, "G", "T")))
    add("fragments: identical + 2 substitutions", pairs, 64, True)

    # 2. the control region across the origin
    dloop = sl("human", 16000, 569) + sl("human", 0, 600)
    mut = bytearray(dloop)
    for i in range(0, len(mut) - 7, 23):
        mut[i] = ord("C") if mut[i] == ord("A") else ord("A")
    add("control region: self, rotation by 3, every 23rd base substituted",
        [(dloop, dloop), (dloop, dloop[3:] + dloop[:3]), (dloop, bytes(mut))], 64, True)

    # 3. human / chimp co-linear windows
    wins = (500, 2000, 4000, 8000, 11000, 14000)
    p600 = [(sl("human", w, 600), sl("chimp", w, 600)) for w in wins]
    p600 = [(p, t) for p, t in p600 if len(p) == 600 and len(t) == 600]
    add("human/chimp 600 bp windows, smax 64", p600, 64, True)
    add("human/chimp 600 bp windows, smax 200, score-only", p600, 200, False)
    p100 = [(sl("human", w, 100), sl("chimp", w, 100)) for w in wins]
    add("human/chimp 100 bp windows, smax 64", p100, 64, True)

    # 4. whole genomes
    add("whole genomes, smax 511, score-only", [(hum, hum), (hum, chi)], 511, False)

    # 5. the N
    npos = hum.find(b"N")
    assert npos >= 0, "the human genome should hold one N"
    p = hum[max(0, npos - 100):max(0, npos - 100) + 200]
    add("200 bp around the N, itself and reversed, smax 200, score-only", [(p, p), (p, p[::-1])], 200, False)

    out = os.path.join(HERE, "real_golden.json.gz")
    with gzip.open(out, "wt") as f:                   # one batch per line, as the other fixtures
        for b in batches:
            b["source"] = (f"reference tests/data/mtdna_human.fa ({len(hum)} bp, N at {npos}), "
                           f"tests/data/mtdna_chimp.fa ({len(chi)} bp)")
            f.write(json.dumps(b) + "\n")
    print(out, sum(len(b["pairs"]) for b in batches), "pairs in", len(batches), "batches")


if __name__ == "__main__":
    main()
