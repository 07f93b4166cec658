"""Seeded synthetic DNA pair workloads.

Five workloads, by what they are:

* ``wfa_150bp_2pct``     10,000 pairs, pattern 150 bp iid ACGT, text = pattern
                          at 2 % per-base error (sub/ins/del equal, 1-base indels);
                          smax 64, with CIGAR.
* ``sw_uneven_200k``     200,000 pairs, query log-uniform 50-1,000 bp, target =
                          uniform 0-500 bp flank + query at 5 % (sub/ins/del
                          60/20/20) + uniform 0-500 bp flank; text = target (rows),
                          pattern = query (columns); scoring {2,-3,3,1}.
* ``wfa_long_1k_10k``    2,000 pairs, length log-uniform 1-10 kb, per-pair error
                          log-uniform 1-15 %, sub/ins/del equal, indel length
                          geometric (p = 0.5, mean 2); smax 2048.
* ``wfa_mixed_1m``       1,000,000 pairs, length uniform 150-250 bp, per-pair error
                          from the mixture 70 % U[0,2 %], 25 % U[2,10 %], 5 % U[10,30 %],
                          sub/ins/del equal, 1-base indels.
* ``sw_long_4k``         4,096 pairs, query log-uniform 2-30 kb, target = uniform
                          0-5 kb flank + query at 10 % (50/25/25) + uniform 0-5 kb flank.

Mutation model: each base of the source independently carries an event with
probability e; the event type is drawn from the stated mix; a substitution
draws one of the three other bases uniformly; an insertion adds random bases
after the base; a deletion removes the base (and, for geometric lengths, the
following bases of the run).

Sequences are returned packed: one uint8 ASCII buffer per side plus int64
offsets and int32 lengths, the layout the C ABI and the device kernels take.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


@dataclass
class PairSet:
    """Packed pairs.  For WFA: a = pattern, b = text.  For SW: a = text (rows),
    b = pattern (columns)."""
    name: str
    a_buf: np.ndarray
    a_off: np.ndarray
    a_len: np.ndarray
    b_buf: np.ndarray
    b_off: np.ndarray
    b_len: np.ndarray
    meta: dict

    @property
    def n(self) -> int:
        return int(self.a_len.shape[0])

    def a(self, i: int) -> bytes:
        o = int(self.a_off[i])
        return self.a_buf[o:o + int(self.a_len[i])].tobytes()

    def b(self, i: int) -> bytes:
        o = int(self.b_off[i])
        return self.b_buf[o:o + int(self.b_len[i])].tobytes()

    def subset(self, idx) -> "PairSet":
        idx = np.asarray(idx)
        a = [self.a(int(i)) for i in idx]
        b = [self.b(int(i)) for i in idx]
        return from_lists(self.name + "[subset]", a, b, dict(self.meta))

    def lists(self):
        return [self.a(i) for i in range(self.n)], [self.b(i) for i in range(self.n)]


def _offsets(lens: np.ndarray) -> np.ndarray:
    off = np.zeros(lens.shape[0], np.int64)
    if lens.shape[0] > 1:
        np.cumsum(lens[:-1].astype(np.int64), out=off[1:])
    return off


def from_lists(name, a_list, b_list, meta=None) -> PairSet:
    a_len = np.array([len(x) for x in a_list], np.int32)
    b_len = np.array([len(x) for x in b_list], np.int32)
    a_buf = np.frombuffer(b"".join(a_list), np.uint8).copy() if a_list else np.zeros(0, np.uint8)
    b_buf = np.frombuffer(b"".join(b_list), np.uint8).copy() if b_list else np.zeros(0, np.uint8)
    return PairSet(name, a_buf, _offsets(a_len), a_len, b_buf, _offsets(b_len), b_len, meta or {})


_LUT = np.zeros(256, np.int64)
_LUT[ACGT] = np.arange(4)


def random_bases(rng, n: int) -> np.ndarray:
    return ACGT[rng.integers(0, 4, size=n, dtype=np.uint8)]


def mutate_point(rng, src: np.ndarray, src_len: np.ndarray, rate, mix):
    """Vectorised 1-base-indel mutation of many sequences at once.

    ``src`` is the concatenation of sequences with lengths ``src_len``; ``rate``
    is a scalar or one rate per sequence; ``mix`` = (p_sub, p_ins, p_del).
    Returns (buffer, lengths) of the mutated sequences."""
    total = src.shape[0]
    nseq = src_len.shape[0]
    src_off = _offsets(src_len)
    if np.isscalar(rate):
        ev = np.nonzero(rng.random(total) < rate)[0]
    else:
        seq_id = np.repeat(np.arange(nseq, dtype=np.int64), src_len)
        ev = np.nonzero(rng.random(total) < np.asarray(rate)[seq_id])[0]
        del seq_id
    typ = rng.choice(3, size=ev.size, p=np.asarray(mix, float))
    reps = np.ones(total, np.int8)
    reps[ev[typ == 1]] = 2
    reps[ev[typ == 2]] = 0
    out = np.repeat(src, reps)
    start = np.cumsum(reps, dtype=np.int64) - reps
    sub = ev[typ == 0]
    if sub.size:
        shift = rng.integers(1, 4, size=sub.size)
        out[start[sub]] = ACGT[(_LUT[src[sub]] + shift) % 4]
    ins = ev[typ == 1]
    if ins.size:
        out[start[ins] + 1] = random_bases(rng, ins.size)
    # per-sequence output length = source length + insertions - deletions
    seq_of = lambda pos: np.searchsorted(src_off, pos, side="right") - 1
    out_len = src_len.astype(np.int64).copy()
    np.add.at(out_len, seq_of(ins), 1)
    np.add.at(out_len, seq_of(ev[typ == 2]), -1)
    return out, out_len.astype(np.int32)


def mutate_runs(rng, s: np.ndarray, rate: float, mix, geom_p=None) -> np.ndarray:
    """Mutation of one sequence with optional geometric indel lengths."""
    L = s.shape[0]
    pos = np.nonzero(rng.random(L) < rate)[0]
    typ = rng.choice(3, size=pos.size, p=np.asarray(mix, float))
    pieces = []
    cur = 0
    for p, t in zip(pos.tolist(), typ.tolist()):
        if p < cur:
            continue                       # inside a deleted run
        pieces.append(s[cur:p])
        run = 1 if geom_p is None else int(rng.geometric(geom_p))
        if t == 0:
            c = int(_LUT[s[p]])
            pieces.append(ACGT[[(c + int(rng.integers(1, 4))) % 4]])
            cur = p + 1
        elif t == 1:
            pieces.append(s[p:p + 1])
            pieces.append(random_bases(rng, run))
            cur = p + 1
        else:
            cur = p + run
    pieces.append(s[cur:])
    return np.concatenate(pieces) if pieces else s.copy()


def _pairs(name, a_buf, a_len, b_buf, b_len, meta):
    return PairSet(name, a_buf, _offsets(a_len), a_len.astype(np.int32), b_buf,
                   _offsets(b_len), b_len.astype(np.int32), meta)


def wfa_150bp_2pct(n=10_000, seed=1) -> PairSet:
    rng = np.random.default_rng(seed)
    plen = np.full(n, 150, np.int32)
    pat = random_bases(rng, int(plen.sum()))
    txt, tlen = mutate_point(rng, pat, plen, 0.02, (1 / 3, 1 / 3, 1 / 3))
    return _pairs("wfa_150bp_2pct", pat, plen, txt, tlen, {"smax": 64, "with_cigar": True})


def sw_uneven_200k(n=200_000, seed=2) -> PairSet:
    rng = np.random.default_rng(seed)
    qlen = np.rint(np.exp(rng.uniform(np.log(50), np.log(1000), size=n))).astype(np.int64)
    q = random_bases(rng, int(qlen.sum()))
    core, core_len = mutate_point(rng, q, qlen, 0.05, (0.6, 0.2, 0.2))
    lf = rng.integers(0, 501, size=n)
    rf = rng.integers(0, 501, size=n)
    tlen = lf + core_len + rf
    # assemble target = flank + core + flank with vectorised scatter
    t = np.empty(int(tlen.sum()), np.uint8)
    toff = _offsets(tlen)
    core_off = _offsets(core_len)
    flank = random_bases(rng, int(lf.sum() + rf.sum()))
    fl_off = _offsets(lf + rf)
    seg_lf = np.repeat(np.arange(n), lf)
    idx_lf = toff[seg_lf] + (np.arange(int(lf.sum())) - _offsets(lf)[seg_lf])
    t[idx_lf] = flank[fl_off[seg_lf] + (np.arange(int(lf.sum())) - _offsets(lf)[seg_lf])]
    seg_c = np.repeat(np.arange(n), core_len)
    within_c = np.arange(int(core_len.sum())) - core_off[seg_c]
    t[toff[seg_c] + lf[seg_c] + within_c] = core
    seg_r = np.repeat(np.arange(n), rf)
    within_r = np.arange(int(rf.sum())) - _offsets(rf)[seg_r]
    t[toff[seg_r] + lf[seg_r] + core_len[seg_r] + within_r] = flank[fl_off[seg_r] + lf[seg_r] + within_r]
    return _pairs("sw_uneven_200k", t, tlen, q, qlen, {"scoring": (2, -3, 3, 1), "with_cigar": True})


def wfa_long_1k_10k(n=2_000, seed=3) -> PairSet:
    rng = np.random.default_rng(seed)
    L = np.rint(np.exp(rng.uniform(np.log(1000), np.log(10000), size=n))).astype(np.int64)
    e = np.exp(rng.uniform(np.log(0.01), np.log(0.15), size=n))
    pats, txts = [], []
    for i in range(n):
        s = random_bases(rng, int(L[i]))
        pats.append(s)
        txts.append(mutate_runs(rng, s, float(e[i]), (1 / 3, 1 / 3, 1 / 3), geom_p=0.5))
    plen = np.array([x.shape[0] for x in pats], np.int32)
    tlen = np.array([x.shape[0] for x in txts], np.int32)
    return _pairs("wfa_long_1k_10k", np.concatenate(pats), plen, np.concatenate(txts), tlen,
                  {"smax": 2048, "with_cigar": True})


def mixture_rates(rng, n):
    comp = rng.choice(3, size=n, p=[0.70, 0.25, 0.05])
    lo = np.array([0.0, 0.02, 0.10])[comp]
    hi = np.array([0.02, 0.10, 0.30])[comp]
    return rng.uniform(lo, hi)


def wfa_mixed(n=1_000_000, seed=4) -> PairSet:
    rng = np.random.default_rng(seed)
    plen = rng.integers(150, 251, size=n).astype(np.int64)
    pat = random_bases(rng, int(plen.sum()))
    rate = mixture_rates(rng, n)
    txt, tlen = mutate_point(rng, pat, plen, rate, (1 / 3, 1 / 3, 1 / 3))
    return _pairs("wfa_mixed_1m", pat, plen, txt, tlen, {"smax": 64, "with_cigar": True,
                                                          "rate": rate})


def sw_long_4k(n=4_096, seed=5) -> PairSet:
    rng = np.random.default_rng(seed)
    qlen = np.rint(np.exp(rng.uniform(np.log(2000), np.log(30000), size=n))).astype(np.int64)
    q = random_bases(rng, int(qlen.sum()))
    core, core_len = mutate_point(rng, q, qlen, 0.10, (0.5, 0.25, 0.25))
    core_off = _offsets(core_len)
    lf = rng.integers(0, 5001, size=n)
    rf = rng.integers(0, 5001, size=n)
    ts = []
    for i in range(n):
        c = core[core_off[i]:core_off[i] + core_len[i]]
        ts.append(np.concatenate([random_bases(rng, int(lf[i])), c, random_bases(rng, int(rf[i]))]))
    tlen = np.array([x.shape[0] for x in ts], np.int32)
    return _pairs("sw_long_4k", np.concatenate(ts), tlen, q, qlen,
                  {"scoring": (2, -3, 3, 1), "with_cigar": True})


WORKLOADS = {
    "wfa_150bp_2pct": wfa_150bp_2pct,
    "sw_uneven_200k": sw_uneven_200k,
    "wfa_long_1k_10k": wfa_long_1k_10k,
    "wfa_mixed_1m": wfa_mixed,
    "sw_long_4k": sw_long_4k,
}


# ------------------------------------------------------------ gene families --
_STOPS1 = {b"TAA", b"TAG", b"TGA"}
_SENSE = [bytes(c) for c in (a + b + c for a in (b"A", b"C", b"G", b"T") for b in (b"A", b"C", b"G", b"T")
                             for c in (b"A", b"C", b"G", b"T")) if bytes(c) not in _STOPS1 | {b"AGA", b"AGG"}]


def gene_family(n_records=200, codons=300, seed=6):
    """A seeded protein-coding gene family for one-reference-against-many work.

    Returns (records, baits): lists of (id, sequence bytes).  The bait file
    holds a clean CDS (ATG, `codons` sense codons, TAA) and a fragment of it
    shifted by one base with an inserted stop; the records are copies of the
    CDS at 0-4 % substitutions with, by class: nothing else; an in-frame
    3-base deletion; a 1- or 2-base indel (frameshift); a premature stop;
    a 40-70 % fragment; bases outside ACGT; 0-200 bp flanks; or an unrelated
    random sequence."""
    rng = np.random.default_rng(seed)
    sense = np.array([np.frombuffer(c, np.uint8) for c in _SENSE])
    cds = np.concatenate([np.frombuffer(b"ATG", np.uint8),
                          sense[rng.integers(0, len(_SENSE), size=codons)].reshape(-1),
                          np.frombuffer(b"TAA", np.uint8)])
    frag = np.concatenate([random_bases(rng, 1), cds[30: len(cds) // 2], np.frombuffer(b"TGA", np.uint8),
                           cds[len(cds) // 2: -60]])
    baits = [("bait_frag shifted fragment", frag.tobytes()), ("bait_cds clean CDS", cds.tobytes())]
    records = []
    for r in range(n_records):
        cls = r % 9
        s = cds.copy()
        rate = float(rng.uniform(0.0, 0.04))
        sub = np.nonzero(rng.random(s.shape[0]) < rate)[0]
        s[sub] = ACGT[(_LUT[s[sub]] + rng.integers(1, 4, size=sub.size)) % 4]
        if cls == 1:
            k = 3 * int(rng.integers(10, codons - 10))
            s = np.concatenate([s[:k], s[k + 3:]])
        elif cls == 2:
            k = int(rng.integers(30, s.shape[0] - 30))
            d = int(rng.integers(1, 3))
            s = np.concatenate([s[:k], s[k + d:]]) if rng.random() < 0.5 else \
                np.concatenate([s[:k], random_bases(rng, d), s[k:]])
        elif cls == 3:
            k = 3 * int(rng.integers(20, codons - 20))
            s[k:k + 3] = np.frombuffer(b"TAG", np.uint8)
        elif cls == 4:
            L = int(s.shape[0] * rng.uniform(0.4, 0.7))
            a = int(rng.integers(0, s.shape[0] - L))
            s = s[a:a + L]
        elif cls == 5:
            s[rng.integers(0, s.shape[0], size=int(rng.integers(1, 6)))] = ord("N")
        elif cls == 6:
            s = np.concatenate([random_bases(rng, int(rng.integers(0, 200))), s,
                                random_bases(rng, int(rng.integers(0, 200)))])
        elif cls == 7:
            s = random_bases(rng, int(rng.integers(300, 1200)))
        records.append((f"rec{r:04d} class{cls}", s.tobytes()))
    return records, baits


def write_fasta(path, records, width=60, crlf=False):
    """Write (id-and-description, sequence) records as FASTA, `width` bases per line."""
    end = b"\r\n" if crlf else b"\n"
    with open(path, "wb") as f:
        for head, seq in records:
            f.write(b">" + head.encode() + end)
            for k in range(0, len(seq), width):
                f.write(seq[k:k + width] + end)
