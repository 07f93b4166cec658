"""The host entries move sequences to the device two ways: when the caller's
sequences of each kind lie in request order in one dense span (the packed
buffers of this API, FASTA arenas), and the device reads host memory through
the host's page tables, the spans are copied as laid out and moved into place
by a device kernel; otherwise each sequence is copied into pinned staging.
The same batch laid out both ways gives the oracle's results either way."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, workloads
from helpers import assert_sw_equal, assert_wfa_equal

pytestmark = pytest.mark.gpu


def _reversed_layout(ps):
    """The same pairs with each buffer's sequences stored in reverse request
    order, so the sides' addresses fall from one request to the next."""
    def rev(buf, off, ln):
        pieces = [buf[int(off[i]):int(off[i]) + int(ln[i])] for i in range(ln.shape[0])][::-1]
        new = np.concatenate(pieces) if pieces else buf[:0]
        starts = np.zeros(ln.shape[0], np.int64)
        at = 0
        for i in range(ln.shape[0] - 1, -1, -1):
            starts[i] = at
            at += int(ln[i])
        return new, starts
    a_buf, a_off = rev(ps.a_buf, ps.a_off, ps.a_len)
    b_buf, b_off = rev(ps.b_buf, ps.b_off, ps.b_len)
    return workloads.PairSet(ps.name + "[reversed]", a_buf, a_off, ps.a_len, b_buf, b_off, ps.b_len, ps.meta)


def test_wfa_spans_and_staging_agree():
    ps = workloads.wfa_150bp_2pct(n=20000, seed=71)          # 6 MB of sequence: above the span threshold
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=64, with_cigar=True)
    for layout in (ps, _reversed_layout(ps)):
        got = api.align_batch_packed(layout.a_buf, layout.a_off, layout.a_len, layout.b_buf, layout.b_off,
                                     layout.b_len, smax=64, with_cigar=True)
        assert_wfa_equal(got, want, layout.name)


def test_sw_spans_and_staging_agree():
    ps = workloads.sw_uneven_200k(n=5000, seed=72)          # 5.4 MB of sequence: above the span threshold
    ts, pp = ps.lists()
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=True)
    for layout in (ps, _reversed_layout(ps)):
        got = api.align_sw_batch_packed(layout.a_buf, layout.a_off, layout.a_len, layout.b_buf, layout.b_off,
                                        layout.b_len, scoring=(2, -3, 3, 1), with_cigar=True)
        assert_sw_equal(got, want, layout.name)
