"""The CPU oracle (oracle/ga_oracle.c) against the reference's own outputs.

tests/golden/ was produced by the reference's kernels compiled for the host
(tests/golden/make_golden.py); every field of every result must match."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import workloads


def _enc(s):
    return s.encode("latin-1")


def test_oracle_wfa_matches_reference_golden(wfa_golden):
    for rec in wfa_golden:
        pats = [_enc(p) for p, _ in rec["pairs"]]
        txts = [_enc(t) for _, t in rec["pairs"]]
        got = oracle.wfa_batch(pats, txts, smax=rec["smax"], with_cigar=rec["with_cigar"], threads=4)
        assert got.status == "ok", rec["name"]
        for i, want in enumerate(rec["results"]):
            assert got.score[i] == want["score"], (rec["name"], i)
            assert got.resolved[i] == bool(want["resolved"]), (rec["name"], i)
            assert got.cigars[i].decode() == want["cigar"], (rec["name"], i)
            assert got.rescore_ok[i] == bool(want["rescore_ok"]), (rec["name"], i)
            assert got.wellformed_ok[i] == bool(want["wellformed_ok"]), (rec["name"], i)
        assert got.resolved_count == rec["resolved_count"]
        assert got.unresolved_count == rec["unresolved_count"]


def test_oracle_sw_matches_reference_golden(sw_golden):
    fields = ["score", "start_i", "start_j", "end_i", "end_j"]
    flags = ["resolved", "rescore_ok", "wellformed_ok", "too_large"]
    for rec in sw_golden:
        ts = [_enc(t) for t, _ in rec["pairs"]]
        ps = [_enc(p) for _, p in rec["pairs"]]
        got = oracle.sw_batch(ts, ps, scoring=tuple(rec["scoring"]), with_cigar=rec["with_cigar"], threads=4)
        assert got.status == rec["status"], rec["name"]
        for i, want in enumerate(rec["results"]):
            for f in fields:
                assert getattr(got, f)[i] == want[f], (rec["name"], i, f)
            for f in flags:
                assert getattr(got, f)[i] == bool(want[f]), (rec["name"], i, f)
            assert got.cigars[i].decode() == want["cigar"], (rec["name"], i)


def test_oracle_wfa_score_equals_levenshtein():
    ps = workloads.wfa_150bp_2pct(n=300, seed=11)
    pats, txts = ps.lists()
    got = oracle.wfa_batch(pats, txts, smax=64, with_cigar=True)
    ed = oracle.edit_distance(pats, txts)
    assert np.array_equal(got.score, np.where(ed <= 64, ed, -1))
    assert got.rescore_ok.all() and got.wellformed_ok.all()


def test_oracle_validation_refusals():
    b = oracle.wfa_batch([b"ACGT"], [b"ACGT"], smax=512)
    assert b.status == "invalid_argument" and b.error == "smax out of range [0, 511]"
    b = oracle.wfa_batch([b"ACGT"], [b"ACGT"], smax=-1)
    assert b.status == "invalid_argument"
    b = oracle.wfa_batch([(None, 5)], [b"ACGT"], smax=8)
    assert b.error == "null pointer with non-zero length"
    for sc in [(0, -1, 2, 1), (2, 2, 5, 2), (2, -3, 0, 2), (2, -3, 5, 0), (2, -3, 1, 2)]:
        assert oracle.sw_batch([b"ACGT"], [b"ACGT"], scoring=sc).status == "invalid_argument"
    b = oracle.sw_batch([b"ACGT"], [b"ACGT"], scoring=(2, -3, 1, 2), with_cigar=False)
    assert b.status == "ok" and b.score[0] == 8
    b = oracle.sw_batch([b"ACGT", b"ACGT"], [b"ACGT", b"ACGT"], scoring=[(2, -3, 5, 2), (1, -1, 2, 1)])
    assert b.error == "all requests in an SW batch must share one scoring scheme"
    big_t, big_p = b"A" * 8192, b"A" * 8193
    b = oracle.sw_batch([big_t], [big_p])
    assert b.too_large[0] and not b.resolved[0] and b.score[0] == -1


def test_oracle_wfa_matches_reference_on_real_sequences(real_golden):
    """Human and chimp mitochondrial genomes (repeats, the human N, real
    divergence), cut as the reference's real-sequence test cuts them: the
    oracle equals the reference's kernels field by field, and a pair is
    unresolved exactly when its edit distance exceeds smax."""
    for rec in real_golden:
        pats = [_enc(p) for p, _ in rec["pairs"]]
        txts = [_enc(t) for _, t in rec["pairs"]]
        got = oracle.wfa_batch(pats, txts, smax=rec["smax"], with_cigar=rec["with_cigar"], threads=4)
        assert got.status == "ok", rec["name"]
        for i, want in enumerate(rec["results"]):
            assert got.score[i] == want["score"], (rec["name"], i)
            assert got.cigars[i].decode() == want["cigar"], (rec["name"], i)
            assert got.rescore_ok[i] == bool(want["rescore_ok"]), (rec["name"], i)
            assert got.wellformed_ok[i] == bool(want["wellformed_ok"]), (rec["name"], i)
            d, smax = rec["edit_distance"][i], rec["smax"][i]
            assert (got.score[i] == d) if d <= smax else (got.score[i] == -1), (rec["name"], i)
        assert got.resolved_count == rec["resolved_count"]
