"""Shared helpers for the parity tests (test infrastructure)."""
import numpy as np

from genoaligner_gb300 import api, workloads


def packed(a_list, b_list):
    """Two byte-string lists -> the buffers/offsets/lengths the packed API takes."""
    ps = workloads.from_lists("t", a_list, b_list)
    return ps


def wfa_gpu(pats, txts, smax=64, with_cigar=True, max_smax=0, learned=False):
    ps = packed(pats, txts)
    r = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                               smax=smax, with_cigar=with_cigar, max_smax=max_smax, learned=learned)
    return r


def sw_gpu(texts, pats, scoring=(2, -3, 5, 2), with_cigar=True, trace_cell_limit=0):
    ps = packed(texts, pats)
    return api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                     scoring=scoring, with_cigar=with_cigar,
                                     trace_cell_limit=trace_cell_limit)


def assert_wfa_equal(got, want, label=""):
    """got: PackedResult from the C ABI; want: oracle.WfaBatch."""
    assert got.status.name == want.status, (label, got.status, want.status, got.error)
    if want.status != "ok":
        assert got.error == want.error, label
        return
    r = got.res
    bad = np.nonzero(r["score"] != want.score)[0]
    assert bad.size == 0, (label, "score", bad[:10], r["score"][bad[:10]], want.score[bad[:10]])
    assert np.array_equal(r["resolved"].astype(bool), want.resolved), label
    assert np.array_equal(r["rescore_ok"].astype(bool), want.rescore_ok), label
    assert np.array_equal(r["wellformed_ok"].astype(bool), want.wellformed_ok), label
    for i in range(len(want.cigars)):
        c = got.cigar(i)
        assert c == want.cigars[i], (label, i, c[:80], want.cigars[i][:80])
    assert got.resolved_count == want.resolved_count and got.unresolved_count == want.unresolved_count


def assert_sw_equal(got, want, label=""):
    assert got.status.name == want.status, (label, got.status, want.status, got.error)
    if want.status != "ok":
        assert got.error == want.error, label
        return
    r = got.res
    for f in ("score", "start_i", "start_j", "end_i", "end_j"):
        bad = np.nonzero(r[f] != getattr(want, f))[0]
        assert bad.size == 0, (label, f, bad[:10], r[f][bad[:10]], getattr(want, f)[bad[:10]])
    for f in ("resolved", "rescore_ok", "wellformed_ok", "too_large"):
        assert np.array_equal(r[f].astype(bool), getattr(want, f)), (label, f)
    for i in range(len(want.cigars)):
        assert got.cigar(i) == want.cigars[i], (label, i)
    assert got.resolved_count == want.resolved_count and got.unresolved_count == want.unresolved_count
