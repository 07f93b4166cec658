"""The C-ABI library without a GPU: it loads, exports every symbol the header
declares, and refuses invalid batches before any device work, with the
reference's messages."""
import os
import re

import pytest

from genoaligner_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "genoaligner_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)          # drop comments
    return sorted(set(re.findall(r"\b(ga_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = api.load()
    names = declared_symbols()
    assert len(names) >= 13
    for name in names:
        assert hasattr(L, name), name
    assert set(api.EXPORTS) <= set(names)


def test_provenance_without_device():
    assert api.backend_name() == "cuda-sm_103a"
    assert isinstance(api.device_name(), str)


@pytest.mark.parametrize("smax", [512, -1])
def test_wfa_smax_refused(smax):
    b = api.align_batch([api.AlignRequest(b"ACGT", 4, b"ACGT", 4, smax=smax)])
    assert b.status == api.Status.invalid_argument
    assert b.error == "smax out of range [0, 511]"
    assert len(b.results) == 1 and b.results[0].score == -1


def test_wfa_null_and_negative_refused():
    b = api.align_batch([api.AlignRequest(None, 5, b"ACGT", 4, smax=8)])
    assert b.status == api.Status.invalid_argument and b.error == "null pointer with non-zero length"
    b = api.align_batch([api.AlignRequest(b"ACGT", -1, b"ACGT", 4, smax=8)])
    assert b.status == api.Status.invalid_argument and b.error == "negative length"
    # the first failing request decides, in request order
    b = api.align_batch([api.AlignRequest(b"ACGT", 4, b"ACGT", 4, smax=600),
                         api.AlignRequest(None, 3, b"A", 1)])
    assert b.error == "smax out of range [0, 511]"


def test_ext_accepts_larger_smax_bound():
    b = api.align_batch([api.AlignRequest(b"ACGT", 4, b"ACGT", 4, smax=2048)], max_smax=4096)
    assert b.status != api.Status.invalid_argument


@pytest.mark.parametrize("sc,msg", [
    ((0, -1, 2, 1), "SW scoring: match must be > 0 (the score is 0 for every input otherwise)"),
    ((2, 2, 5, 2), "SW scoring: mismatch must be < match"),
    ((2, -3, 0, 2), "SW scoring: gap costs must be > 0"),
    ((2, -3, 5, 0), "SW scoring: gap costs must be > 0"),
    ((2, -3, 1, 2), "SW scoring: gap_extend > gap_open with with_cigar cannot re-score to its own score "
                    "(api.hpp; RESULTADO_H9_SW2_TRACE.md). Score-only requests may use it"),
])
def test_sw_scheme_refusals(sc, msg):
    b = api.align_sw_batch([api.SWRequest(b"ACGT", 4, b"ACGT", 4, api.SWScoring(*sc))])
    assert b.status == api.Status.invalid_argument and b.error == msg


def test_sw_mixed_scheme_and_null_refused():
    r1 = api.SWRequest(b"ACGT", 4, b"ACGT", 4, api.SWScoring(2, -3, 5, 2))
    r2 = api.SWRequest(b"ACGT", 4, b"ACGT", 4, api.SWScoring(1, -1, 2, 1))
    b = api.align_sw_batch([r1, r2])
    assert b.error == "all requests in an SW batch must share one scoring scheme"
    b = api.align_sw_batch([api.SWRequest(b"ACGT", 4, None, 5)])
    assert b.error == "null pointer with non-zero length"
    b = api.align_sw_batch([api.SWRequest(b"ACGT", -1, b"ACGT", 4)])
    assert b.error == "negative length"


def test_sw_score_only_pattern_limit_refused():
    # 4 warps x 2*(n+1) ints above 48 KiB: the reference's score-only limit
    p = b"A" * 1600
    b = api.align_sw_batch([api.SWRequest(b"ACGT", 4, p, len(p), with_cigar=False)])
    assert b.status == api.Status.invalid_argument
    assert b.error.startswith("pattern_len exceeds this device's shared-memory limit")


def test_empty_batch_is_ok():
    assert api.align_batch([]).ok()
    assert api.align_sw_batch([]).ok()


def test_no_device_is_device_error():
    if api.device_available():
        pytest.skip("a device is present")
    b = api.align_batch([api.AlignRequest(b"ACGT", 4, b"ACGT", 4, smax=8)])
    assert b.status == api.Status.device_error and b.error
    assert b.resolved_count == 0 and b.unresolved_count == 0


def test_first_failure_across_chunks_in_request_order():
    """Requests are checked in parallel chunks; the error reported is still
    the first failing request's, and every result is the default."""
    reqs = [api.AlignRequest(b"ACGTACGT", 8, b"ACGTTCGT", 8, smax=8) for _ in range(5000)]
    reqs[4500] = api.AlignRequest(b"ACGT", 4, b"ACGT", 4, smax=600)
    reqs[3000] = api.AlignRequest(b"ACGT", -1, b"ACGT", 4, smax=8)
    reqs[3001] = api.AlignRequest(None, 3, b"ACG", 3, smax=8)
    b = api.align_batch(reqs)
    assert b.status == api.Status.invalid_argument and b.error == "negative length"
    assert len(b.results) == 5000 and all(r.score == -1 and not r.resolved for r in b.results)
    assert b.resolved_count == 0 and b.unresolved_count == 0
    sw = [api.SWRequest(b"ACGTACGT", 8, b"ACGT", 4, api.SWScoring(2, -3, 5, 2)) for _ in range(5000)]
    sw[4000] = api.SWRequest(b"ACGT", 4, None, 5, api.SWScoring(2, -3, 5, 2))
    sw[2500] = api.SWRequest(b"ACGT", 4, b"ACGT", 4, api.SWScoring(1, -1, 2, 1))
    b = api.align_sw_batch(sw)
    assert b.error == "all requests in an SW batch must share one scoring scheme"


def test_wfa_cigar_buffer_contract():
    """ga_align_batch needs a CIGAR buffer of ga_align_cigar_bytes bytes when any
    request asks for a CIGAR; a smaller or missing one is refused before any
    device work -- after the request checks, whose error comes first."""
    import ctypes
    import numpy as np
    L = api.load()
    rng = np.random.default_rng(3)
    n = 3000                                            # three request chunks
    p = rng.integers(0, 4, size=n * 20).astype(np.uint8)
    buf = np.frombuffer(b"ACGT", np.uint8)[p]
    off = np.arange(n, dtype=np.int64) * 20
    ln = np.full(n, 20, np.int32)
    res = np.zeros(n, api.RES_DT)

    def call(reqs, cig, nbytes):
        info = api.BatchInfo()
        st = L.ga_align_batch(reqs.ctypes.data, n, res.ctypes.data, cig, nbytes, ctypes.byref(info))
        return st, info.error.decode() if info.error else None

    reqs = api.make_requests(buf, off, ln, buf, off, ln, 8, True)
    need = int(L.ga_align_cigar_bytes(reqs.ctypes.data, n))
    assert need == n * 40
    small = np.empty(need - 1, np.uint8)
    st, err = call(reqs, small.ctypes.data, need - 1)
    assert st == api.GA_INVALID_ARGUMENT and err == "cigar buffer is smaller than the batch needs"
    assert (res["score"] == -1).all()
    st, err = call(reqs, None, 0)
    assert st == api.GA_INVALID_ARGUMENT and err == "cigar buffer is smaller than the batch needs"
    # a failing request decides first
    bad = reqs.copy()
    bad["smax"][2500] = 600
    st, err = call(bad, small.ctypes.data, need - 1)
    assert st == api.GA_INVALID_ARGUMENT and err == "smax out of range [0, 511]"
    # no CIGAR asked for: no buffer needed (past the checks, a device is needed)
    plain = api.make_requests(buf, off, ln, buf, off, ln, 8, False)
    st, err = call(plain, None, 0)
    assert st != api.GA_INVALID_ARGUMENT, err


def test_request_checks_from_many_threads():
    """Host passes from several calling threads at once share the library's
    thread pool (one job at a time, each caller waiting only for the workers
    that joined its job): every call still reports its own batch's first
    failing request."""
    import threading
    import numpy as np
    L = api.load()
    n = 5000
    buf = np.frombuffer(b"ACGT" * 5, np.uint8).copy()
    off = np.zeros(n, np.int64)
    ln = np.full(n, 20, np.int32)
    failures = []

    def worker(t):
        import ctypes
        rng = np.random.default_rng(100 + t)
        res = np.zeros(n, api.RES_DT)
        for _ in range(40):
            reqs = api.make_requests(buf, off, ln, buf, off, ln, 8, False)
            k = int(rng.integers(0, n))
            reqs["smax"][k] = 600
            if k + 1 < n:
                reqs["pattern_len"][k + 1] = -1
            info = api.BatchInfo()
            st = L.ga_align_batch(reqs.ctypes.data, n, res.ctypes.data, None, 0, ctypes.byref(info))
            if st != api.GA_INVALID_ARGUMENT or info.error != b"smax out of range [0, 511]" or \
                    not (res["score"] == -1).all():
                failures.append((t, k, st, info.error))

    ts = [threading.Thread(target=worker, args=(t,)) for t in range(6)]
    for x in ts:
        x.start()
    for x in ts:
        x.join()
    assert not failures, failures[:3]
