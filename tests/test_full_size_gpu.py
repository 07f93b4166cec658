"""Every benchmarked workload against the oracle at the size it is benchmarked.

The uneven SW batch (200,000 pairs), the long WFA batch (2,000 pairs at smax
2048) and the mixed WFA batch (1,000,000 pairs, plain and learned forms) are
compared whole, field by field: score, resolved flag, span, CIGAR and the
result checks.  The long SW batch (4,096 pairs of up to 1.2 Gcells) is
compared on a stratified subset at its own pair sizes -- its 64 largest pairs
(whole-block items and the 512 x 512 long shape) and 64 more drawn at random
-- under both the built-in kernel setting and the one the autotuner keeps on
that batch; the oracle there runs on as many threads as host memory allows
(its direction table is (m+1)(n+1) bytes per pair in flight)."""
import os

import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, cost_model, workloads
from helpers import assert_sw_equal, assert_wfa_equal

pytestmark = pytest.mark.gpu

SCORING = (2, -3, 3, 1)


def _threads():
    return os.cpu_count() or 1


def test_sw_uneven_full_batch_vs_oracle():
    ps = workloads.sw_uneven_200k()
    ts, pp = ps.lists()
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, threads=_threads())
    got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                    scoring=SCORING, with_cigar=True)
    assert_sw_equal(got, want, "sw_uneven_200k full")


def test_wfa_long_full_batch_vs_oracle_plain_and_learned():
    ps = workloads.wfa_long_1k_10k()
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=2048, with_cigar=True, threads=_threads(), max_smax=2048)
    assert cost_model.load_default()
    for learned in (False, True):
        got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=2048,
                                     with_cigar=True, max_smax=2048, learned=learned)
        assert_wfa_equal(got, want, f"wfa_long_1k_10k full, learned={learned}")


def test_wfa_mixed_full_batch_vs_oracle_plain_and_learned():
    ps = workloads.wfa_mixed()
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=64, with_cigar=True, threads=_threads())
    assert cost_model.load_default()
    for learned in (False, True):
        got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=64,
                                     with_cigar=True, learned=learned)
        assert_wfa_equal(got, want, f"wfa_mixed 1M full, learned={learned}")


def _mem_threads(largest_cells):
    """Oracle threads such that the direction tables in flight stay within
    half of the host's available memory."""
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError):
        avail = 16 << 30
    return int(max(1, min(_threads(), avail // 2 // max(1, int(largest_cells * 1.1)))))


def test_sw_long_stratified_subset_vs_oracle():
    full = workloads.sw_long_4k()
    cells = full.a_len.astype(np.int64) * full.b_len.astype(np.int64)
    order = np.argsort(-cells, kind="stable")
    rng = np.random.default_rng(55)
    rest = order[64:]
    idx = np.concatenate([order[:64], rng.choice(rest, size=64, replace=False)])
    ps = full.subset(idx)
    ts, pp = ps.lists()
    assert int(cells[order[0]]) > (1 << 27)             # whole-block items are in the subset
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, trace_cell_limit=-1,
                           threads=_mem_threads(int(cells[order[0]])))
    saved = api.tune_get()
    try:
        # the built-in setting, then the one the autotuner keeps on the long
        # batch (every pair in 32 bits, long shape above 2^22 cells, whole-block
        # items above 2^24)
        for setting in (dict(saved), dict(saved, sw_pack16=0, sw_long_log2=22, sw_coop_log2=24)):
            api.tune_set(**setting)
            got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                            scoring=SCORING, with_cigar=True, trace_cell_limit=-1)
            assert_sw_equal(got, want, f"sw_long_4k stratified subset, {setting}")
    finally:
        api.tune_set(**saved)
