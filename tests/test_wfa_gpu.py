"""WFA on the GPU through the C ABI, bit-exact against the reference.

Golden batches (produced by the reference's own kernels), the oracle on seeded
workloads, edge cases, batch semantics and the full-size property checks."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, workloads
from helpers import assert_wfa_equal, wfa_gpu

pytestmark = pytest.mark.gpu


def _enc(s):
    return s.encode("latin-1")


def test_device_present():
    assert api.device_available(), "the GPU tests need a CUDA device"


def test_wfa_golden(wfa_golden):
    for rec in wfa_golden:
        pats = [_enc(p) for p, _ in rec["pairs"]]
        txts = [_enc(t) for _, t in rec["pairs"]]
        got = wfa_gpu(pats, txts, smax=np.array(rec["smax"]), with_cigar=np.array(rec["with_cigar"]))
        assert got.status == api.Status.ok, (rec["name"], got.error)
        res = got.res
        for i, want in enumerate(rec["results"]):
            assert res["score"][i] == want["score"], (rec["name"], i)
            assert bool(res["resolved"][i]) == bool(want["resolved"]), (rec["name"], i)
            assert got.cigar(i).decode() == want["cigar"], (rec["name"], i)
            assert bool(res["rescore_ok"][i]) == bool(want["rescore_ok"]), (rec["name"], i)
            assert bool(res["wellformed_ok"][i]) == bool(want["wellformed_ok"]), (rec["name"], i)
        assert got.resolved_count == rec["resolved_count"], rec["name"]


@pytest.mark.parametrize("with_cigar", [True, False])
def test_wfa_150bp_vs_oracle(with_cigar):
    ps = workloads.wfa_150bp_2pct(n=10_000, seed=1)
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=64, with_cigar=with_cigar)
    got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                 smax=64, with_cigar=with_cigar)
    assert_wfa_equal(got, want, "wfa_150bp_2pct")


def test_wfa_mixed_divergence_vs_oracle():
    ps = workloads.wfa_mixed(n=20_000, seed=44)
    pats, txts = ps.lists()
    for smax in (8, 64, 200):
        want = oracle.wfa_batch(pats, txts, smax=smax, with_cigar=True)
        got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                     smax=smax, with_cigar=True)
        assert_wfa_equal(got, want, f"wfa_mixed smax={smax}")


def test_wfa_non_acgt_bytes_vs_oracle():
    rng = np.random.default_rng(5)
    alpha = np.frombuffer(b"ACGTNnacgt-", np.uint8)
    pats, txts = [], []
    for i in range(3000):
        L = int(rng.integers(0, 300))
        p = alpha[rng.integers(0, 4 if i % 3 else len(alpha), size=L)].tobytes()
        t = bytearray(p)
        for _ in range(int(rng.integers(0, 6))):
            if t:
                t[int(rng.integers(0, len(t)))] = int(alpha[rng.integers(0, len(alpha))])
        pats.append(p)
        txts.append(bytes(t))
    want = oracle.wfa_batch(pats, txts, smax=32, with_cigar=True)
    got = wfa_gpu(pats, txts, smax=32)
    assert_wfa_equal(got, want, "non-acgt")


def test_wfa_edge_cases():
    cases = [(b"", b""), (b"", b"ACGT"), (b"ACGT", b""), (b"A" * 600, b""), (b"", b"C" * 700),
             (b"ACGT", b"ACGT"), (b"A", b"C"), (b"A" * 1000, b"A" * 1000), (b"A" * 1000, b"A" * 999 + b"C"),
             (b"ACGT" * 100, b"TGCA" * 100)]
    pats = [c[0] for c in cases]
    txts = [c[1] for c in cases]
    for smax in (0, 1, 5, 64, 511):
        for wc in (True, False):
            want = oracle.wfa_batch(pats, txts, smax=smax, with_cigar=wc)
            got = wfa_gpu(pats, txts, smax=smax, with_cigar=wc)
            assert_wfa_equal(got, want, f"edge smax={smax} cigar={wc}")


def test_wfa_batch_semantics_min_smax_and_any_cigar():
    ps = workloads.wfa_mixed(n=600, seed=7)
    pats, txts = ps.lists()
    smaxs = np.where(np.arange(600) % 50 == 3, 4, 200)
    wc = np.arange(600) % 5 == 0
    want = oracle.wfa_batch(pats, txts, smax=smaxs, with_cigar=wc)
    got = wfa_gpu(pats, txts, smax=smaxs, with_cigar=wc)
    assert_wfa_equal(got, want, "min smax")
    assert (got.res["score"] <= 4).all()


def test_wfa_object_api_documented_example():
    r = api.align(api.AlignRequest(b"ACGTACGT", 8, b"ACGTTCGT", 8, smax=32))
    assert r.resolved and r.score == 1 and r.cigar == "MMMMXMMM"
    assert r.rescore_ok and r.wellformed_ok
    r = api.align(api.AlignRequest(b"", 0, b"ACGT", 4, smax=8))
    assert r.resolved and r.score == 4 and r.cigar == "IIII"


def test_wfa_ext_large_smax_vs_oracle():
    ps = workloads.wfa_long_1k_10k(n=60, seed=31)
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=2048, with_cigar=True, max_smax=4096)
    got = wfa_gpu(pats, txts, smax=2048, max_smax=4096)
    assert_wfa_equal(got, want, "long smax 2048")


def test_wfa_full_size_properties():
    """At the full 1M-pair size: every resolved CIGAR re-scores to its score and
    consumes both sequences (the library's own check), and scores match the
    O(nm) DP on a sample."""
    ps = workloads.wfa_mixed(n=1_000_000, seed=4)
    got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                 smax=64, with_cigar=True)
    res = got.res
    assert got.status == api.Status.ok
    ok = res["resolved"].astype(bool)
    assert ok.mean() > 0.99
    assert res["rescore_ok"][ok].all() and res["wellformed_ok"][ok].all()
    assert (res["cigar_len"][ok] >= np.maximum(ps.a_len, ps.b_len)[ok]).all()
    idx = np.random.default_rng(0).choice(ps.n, 2000, replace=False)
    sub = ps.subset(idx)
    pats, txts = sub.lists()
    ed = oracle.edit_distance(pats, txts)
    assert np.array_equal(res["score"][idx], np.where(ed <= 64, ed, -1))


def test_wfa_fault_injection_reports_device_error():
    pats, txts = [b"ACGT", b"AC"], [b"ACGA", b"AC"]
    for step in (1, 2, 3, 4, 5):
        api.load().ga_debug_fail_next(step)
        got = wfa_gpu(pats, txts, smax=8)
        assert got.status == api.Status.device_error and got.error
        assert (got.res["score"] == -1).all() and not got.res["resolved"].any()
        assert got.resolved_count == 0 and got.unresolved_count == 0
    got = wfa_gpu(pats, txts, smax=8)                   # the next call is clean
    assert got.status == api.Status.ok and list(got.res["score"]) == [1, 0]


def test_wfa_concurrent_calls():
    import threading
    ps = workloads.wfa_150bp_2pct(n=2000, seed=9)
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=64, with_cigar=True)
    errs = []

    def run(k):
        try:
            sl = slice(k * 500, (k + 1) * 500)
            got = wfa_gpu(pats[sl], txts[sl], smax=64)
            assert np.array_equal(got.res["score"], want.score[sl])
            for i in range(500):
                assert got.cigar(i) == want.cigars[k * 500 + i]
        except Exception as e:            # surfaced below
            errs.append(e)
    ts = [threading.Thread(target=run, args=(k,)) for k in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs, errs
