"""Smith-Waterman on the GPU through the C ABI, bit-exact against the reference."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, workloads
from helpers import assert_sw_equal, packed, sw_gpu

pytestmark = pytest.mark.gpu


def _enc(s):
    return s.encode("latin-1")


def test_sw_golden(sw_golden):
    for rec in sw_golden:
        ts = [_enc(t) for t, _ in rec["pairs"]]
        ps = [_enc(p) for _, p in rec["pairs"]]
        got = sw_gpu(ts, ps, scoring=tuple(rec["scoring"]), with_cigar=np.array(rec["with_cigar"]))
        assert got.status.name == rec["status"], (rec["name"], got.error)
        res = got.res
        for i, want in enumerate(rec["results"]):
            for f in ("score", "start_i", "start_j", "end_i", "end_j"):
                assert res[f][i] == want[f], (rec["name"], i, f, res[f][i], want[f])
            for f in ("resolved", "rescore_ok", "wellformed_ok", "too_large"):
                assert bool(res[f][i]) == bool(want[f]), (rec["name"], i, f)
            assert got.cigar(i).decode() == want["cigar"], (rec["name"], i)


def test_sw_documented_example():
    r = api.align_sw(api.SWRequest(b"TTTACGTGTT", 10, b"ACGTGT", 6, api.SWScoring(2, -3, 5, 2)))
    assert r.resolved and r.score == 12 and r.cigar == "MMMMMM"
    assert (r.start_i, r.end_i, r.start_j, r.end_j) == (3, 8, 0, 5)


def test_sw_uneven_sample_vs_oracle():
    ps = workloads.sw_uneven_200k(n=3000, seed=21)
    ts, pp = ps.lists()
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=True)
    got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                    scoring=(2, -3, 3, 1), with_cigar=True)
    assert_sw_equal(got, want, "sw_uneven sample")


@pytest.mark.parametrize("scheme", [(2, -3, 3, 1), (1, -1, 2, 1), (2, -3, 5, 2), (5, -4, 10, 1)])
def test_sw_random_vs_oracle(scheme):
    rng = np.random.default_rng(sum(scheme) + 100)
    ts, ps = [], []
    for _ in range(400):
        core = workloads.random_bases(rng, int(rng.integers(1, 700))).tobytes()
        ts.append(workloads.random_bases(rng, int(rng.integers(0, 300))).tobytes() + core +
                  workloads.random_bases(rng, int(rng.integers(0, 300))).tobytes())
        ps.append(core[: max(1, len(core) - int(rng.integers(0, 20)))])
    want = oracle.sw_batch(ts, ps, scoring=scheme, with_cigar=True)
    got = sw_gpu(ts, ps, scoring=scheme)
    assert_sw_equal(got, want, f"random {scheme}")


def test_sw_multiband_vs_oracle():
    """Patterns wider than one band (1024 columns) cross band edges."""
    rng = np.random.default_rng(77)
    ts, ps = [], []
    for k in range(24):
        n = int(rng.integers(1025, 3500))
        core = workloads.random_bases(rng, n).tobytes()
        ts.append(workloads.random_bases(rng, int(rng.integers(0, 200))).tobytes() + core[: n // 2] +
                  workloads.random_bases(rng, 3).tobytes() + core[n // 2:])
        ps.append(core)
    want = oracle.sw_batch(ts, ps, scoring=(2, -3, 3, 1), with_cigar=True)
    got = sw_gpu(ts, ps, scoring=(2, -3, 3, 1))
    assert_sw_equal(got, want, "multiband")


def test_sw_score_only_end_cell_vs_oracle():
    rng = np.random.default_rng(3)
    ts, ps = [], []
    for _ in range(500):
        ts.append(workloads.random_bases(rng, int(rng.integers(0, 400))).tobytes())
        ps.append(workloads.random_bases(rng, int(rng.integers(0, 400))).tobytes())
    for i in range(100):                       # repeats: many tied maxima
        ts.append(b"AC" * int(rng.integers(1, 100)))
        ps.append(b"AC" * int(rng.integers(1, 100)))
    for scheme in [(2, -3, 3, 1), (1, -1, 2, 1), (2, -3, 1, 2)]:
        want = oracle.sw_batch(ts, ps, scoring=scheme, with_cigar=False)
        got = sw_gpu(ts, ps, scoring=scheme, with_cigar=False)
        assert_sw_equal(got, want, f"score-only {scheme}")


def test_sw_too_large_and_ext_limit():
    big_t, big_p = b"A" * 8192, b"A" * 8193
    r = api.align_sw(api.SWRequest(big_t, len(big_t), big_p, len(big_p)))
    assert not r.resolved and r.too_large and r.score == -1
    got = sw_gpu([big_t], [big_p], scoring=(2, -3, 5, 2), trace_cell_limit=-1)
    assert got.status == api.Status.ok and got.res["score"][0] == 2 * 8192
    assert got.res["rescore_ok"][0] and got.res["wellformed_ok"][0]


def _long_pair(rng, qlen, flank, rate, with_n):
    q = workloads.random_bases(rng, qlen)
    core, _ = workloads.mutate_point(rng, q, np.array([qlen]), rate, (0.5, 0.25, 0.25))
    t = np.concatenate([workloads.random_bases(rng, flank), core, workloads.random_bases(rng, flank)])
    if with_n:                                    # a few bytes outside A/C/G/T: the byte-compare path
        t[rng.integers(0, t.shape[0], size=5)] = ord("N")
    return t.tobytes(), q.tobytes()


@pytest.mark.parametrize("scheme,with_n", [((2, -3, 3, 1), True), ((12, -3, 5, 2), False)])
def test_sw_long_pairs_vs_oracle(scheme, with_n):
    """Pairs above 2^24 cells take the 32-bit checkpointed kernel's long shape
    (512-row blocks, 512-column tiles); one below it the short shape."""
    rng = np.random.default_rng(91 if with_n else 92)
    pairs = [_long_pair(rng, 4200, 1000, 0.10, with_n), _long_pair(rng, 3000, 700, 0.10, with_n),
             _long_pair(rng, 1500, 300, 0.10, with_n)]
    ts, pp = [x[0] for x in pairs], [x[1] for x in pairs]
    want = oracle.sw_batch(ts, pp, scoring=scheme, with_cigar=True, trace_cell_limit=-1)
    got = sw_gpu(ts, pp, scoring=scheme, trace_cell_limit=-1)
    assert_sw_equal(got, want, f"long {scheme}")


def test_sw_mixed_with_cigar_batch():
    ps = workloads.sw_uneven_200k(n=300, seed=8)
    ts, pp = ps.lists()
    wc = np.arange(300) % 3 == 0
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=wc)
    got = sw_gpu(ts, pp, scoring=(2, -3, 3, 1), with_cigar=wc)
    assert_sw_equal(got, want, "mixed with_cigar")


def test_sw_fault_injection_reports_device_error():
    for step in (1, 2, 3, 4, 5):
        api.load().ga_debug_fail_next(step)
        got = sw_gpu([b"ACGTACGT"], [b"ACGT"])
        assert got.status == api.Status.device_error
        assert got.res["score"][0] == -1 and not got.res["resolved"][0]
    got = sw_gpu([b"ACGTACGT"], [b"ACGT"])
    assert got.status == api.Status.ok and got.res["score"][0] == 8


def test_sw_large_host_batch_runs_in_ranges_with_same_results():
    """A traceback batch of several Gcells runs as ranges (one per 2 Gcells)
    on their own contexts; results (scores, spans, CIGARs at the right
    offsets, checks) equal the device entry's single run and, on a sample, the
    oracle's."""
    torch = pytest.importorskip("torch")
    ps = workloads.sw_uneven_200k(n=16000, seed=23)
    assert int((ps.a_len.astype(np.int64) * ps.b_len).sum()) >= 4e9
    got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                    scoring=(2, -3, 3, 1), with_cigar=True)
    assert got.status == api.Status.ok
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    sc = torch.empty(b.n, dtype=torch.int32, device="cuda")
    pos = torch.empty(4 * b.n, dtype=torch.int32, device="cuda")
    ln = torch.empty(b.n, dtype=torch.int32, device="cuda")
    cg = torch.empty(b.out_bytes, dtype=torch.uint8, device="cuda")
    api.sw_device(b, (2, -3, 3, 1), True, sc, pos, ln, cg, trace_cell_limit=1 << 26)
    torch.cuda.synchronize()
    s, p4, L = sc.cpu().numpy(), pos.cpu().numpy().reshape(-1, 4), ln.cpu().numpy()
    oo, C = b.out_off.cpu().numpy(), cg.cpu().numpy()
    res = got.res
    assert np.array_equal(res["score"], s)
    for f, k in (("start_i", 0), ("start_j", 1), ("end_i", 2), ("end_j", 3)):
        sel = s > 0
        assert np.array_equal(res[f][sel], p4[sel, k]), f
    assert res["rescore_ok"][s > 0].all() and res["wellformed_ok"][s > 0].all()
    cap = ps.a_len.astype(np.int64) + ps.b_len
    for i in range(0, b.n, 7):
        if s[i] > 0:
            assert got.cigar(i) == C[oo[i] + cap[i] - L[i]: oo[i] + cap[i]].tobytes()
    idx = np.random.default_rng(3).choice(b.n, 200, replace=False)
    sub = ps.subset(idx)
    ts, pp = sub.lists()
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=True)
    assert np.array_equal(res["score"][idx], want.score)
    assert all(got.cigar(int(i)) == want.cigars[q] for q, i in enumerate(idx))


def test_sw_large_score_only_batch_runs_in_ranges_with_same_results():
    """A score-only batch of several Gcells runs as ranges too; scores and end
    cells equal the device entry's single run and, on a sample, the oracle's."""
    torch = pytest.importorskip("torch")
    ps = workloads.sw_uneven_200k(n=16000, seed=24)
    assert int((ps.a_len.astype(np.int64) * ps.b_len).sum()) >= 4e9
    got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                    scoring=(2, -3, 3, 1), with_cigar=False)
    assert got.status == api.Status.ok
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    sc = torch.empty(b.n, dtype=torch.int32, device="cuda")
    pos = torch.empty(4 * b.n, dtype=torch.int32, device="cuda")
    api.sw_device(b, (2, -3, 3, 1), False, sc, pos, None, None)
    torch.cuda.synchronize()
    s, p4 = sc.cpu().numpy(), pos.cpu().numpy().reshape(-1, 4)
    res = got.res
    assert np.array_equal(res["score"], s)
    sel = s > 0
    assert np.array_equal(res["end_i"][sel], p4[sel, 2]) and np.array_equal(res["end_j"][sel], p4[sel, 3])
    idx = np.random.default_rng(4).choice(b.n, 200, replace=False)
    ts, pp = ps.subset(idx).lists()
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=False)
    for f in ("score", "end_i", "end_j", "start_i", "start_j"):
        assert np.array_equal(res[f][idx], getattr(want, f)), f


def test_sw_optimistic_16bit_with_handover():
    """Pure pairs whose all-match score passes 16 bits but whose best fits run
    on the 16-bit kernel (sw_opt16_pct); one whose best reaches the 16-bit
    limit (a 16.5 kb identical pair, score 33,000) is handed to the 32-bit
    kernel.  Results equal the strict rule's run and the oracle's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    pairs = [_long_pair(rng, 17000, 500, 0.08, False), _long_pair(rng, 20000, 300, 0.10, False)]
    q = workloads.random_bases(rng, 16500).tobytes()
    pairs.append((workloads.random_bases(rng, 200).tobytes() + q + workloads.random_bases(rng, 200).tobytes(), q))
    ts, pp = [x[0] for x in pairs], [x[1] for x in pairs]
    scheme = (2, -3, 3, 1)
    ps = workloads.from_lists("t", ts, pp)
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    before = api.tune_get()
    outs = {}
    try:
        for pct in (75, 100):
            api.tune_set(sw_opt16_pct=pct)
            sc = torch.empty(b.n, dtype=torch.int32, device="cuda")
            pos = torch.empty(4 * b.n, dtype=torch.int32, device="cuda")
            ln = torch.empty(b.n, dtype=torch.int32, device="cuda")
            cg = torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda")
            api.profile(True)
            api.sw_device(b, scheme, True, sc, pos, ln, cg, trace_cell_limit=-1)
            torch.cuda.synchronize()
            api.profile(False)
            outs[pct] = (sc.cpu().numpy(), pos.cpu().numpy(), ln.cpu().numpy(), cg.cpu().numpy(),
                         set(api.profile_read()))
    finally:
        api.tune_set(**before)
    assert "sw16x2_trace" in outs[75][4] and "sw32_trace" in outs[75][4]     # 16-bit run, one handed over
    assert "sw16x2_trace" not in outs[100][4]
    for x, y in zip(outs[75][:4], outs[100][:4]):
        assert np.array_equal(x, y)
    want = oracle.sw_batch(ts, pp, scoring=scheme, with_cigar=True, trace_cell_limit=-1)
    assert list(outs[75][0]) == list(want.score)
    assert want.score[2] == 33000


def test_sw_score_only_uneven_and_multiband_vs_oracle():
    """Score-only batches run two pure pairs per warp in 16 bits (multi-band
    patterns included) and the rest in 32 bits; scores and the reference's
    score-only end cells equal the oracle's."""
    ps = workloads.sw_uneven_200k(n=1500, seed=29)
    ts, pp = ps.lists()
    rng = np.random.default_rng(30)
    for k in range(12):                                   # patterns past one 512-column band
        core = workloads.random_bases(rng, int(rng.integers(600, 1400))).tobytes()
        ts.append(workloads.random_bases(rng, 100).tobytes() + core + workloads.random_bases(rng, 80).tobytes())
        pp.append(core)
    for k in range(0, 60, 3):                              # a few bytes outside ACGT
        t = bytearray(ts[k]); t[len(t) // 2] = ord("N"); ts[k] = bytes(t)
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=False)
    got = sw_gpu(ts, pp, scoring=(2, -3, 3, 1), with_cigar=False, trace_cell_limit=-1)
    assert_sw_equal(got, want, "score-only uneven")


def test_sw_device_score_only_vs_oracle():
    """The device entry without traceback: the plan is built on the device
    (16-bit pure pairs two per warp, the rest on the 32-bit score-only
    kernel); score and end cell equal the oracle's, start cells are -1, and
    pairs above the given cell limit get -2."""
    torch = pytest.importorskip("torch")
    ps = workloads.sw_uneven_200k(n=1200, seed=41)
    ts, pp = ps.lists()
    rng = np.random.default_rng(42)
    for k in range(0, 90, 3):                              # bytes outside ACGT: 32-bit kernel
        t = bytearray(ts[k]); t[len(t) // 3] = ord("N"); ts[k] = bytes(t)
    for _ in range(6):                                     # wide patterns: several bands
        core = workloads.random_bases(rng, int(rng.integers(900, 2200))).tobytes()
        ts.append(workloads.random_bases(rng, 50).tobytes() + core)
        pp.append(core)
    ts += [b"", b"ACGT", b"A" * 700]
    pp += [b"ACGT", b"", b"A" * 900]
    # (the device entry has no batch-level shared-memory refusal of the score kernel)
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=False, trace_cell_limit=-1,
                           score_smem_limit=None)
    x = packed(ts, pp)
    b = api.DeviceBatchT(x.a_buf, x.a_off, x.a_len, x.b_buf, x.b_off, x.b_len)
    n = b.n
    sc = torch.empty(n, dtype=torch.int32, device="cuda")
    pos = torch.empty(4 * n, dtype=torch.int32, device="cuda")
    api.sw_device(b, (2, -3, 3, 1), False, sc, pos, None, None)
    torch.cuda.synchronize()
    s, p4 = sc.cpu().numpy(), pos.cpu().numpy().reshape(-1, 4)
    assert np.array_equal(s, want.score)
    pos_ok = want.score > 0
    assert np.array_equal(p4[pos_ok, 2], want.end_i[pos_ok]) and np.array_equal(p4[pos_ok, 3], want.end_j[pos_ok])
    assert (p4[:, 0] == -1).all() and (p4[:, 1] == -1).all()
    assert (p4[~pos_ok, 2:] == -1).all()
    # a cell limit marks the larger pairs too large
    lim = 300 * 300
    api.sw_device(b, (2, -3, 3, 1), False, sc, pos, None, None, trace_cell_limit=lim)
    torch.cuda.synchronize()
    s2 = sc.cpu().numpy()
    big = np.array([len(t) > 0 and len(p) > 0 and (len(t) + 1) * (len(p) + 1) > lim for t, p in zip(ts, pp)])
    assert (s2[big] == -2).all() and np.array_equal(s2[~big], want.score[~big])


@pytest.mark.parametrize("with_cigar", [True, False])
def test_sw_band_edge_widths_vs_oracle(with_cigar):
    """Pattern widths at the forward bands' and tiles' edges (64-column tiles,
    bands of 64 to 512 columns), two pairs of different widths per warp, and
    texts of one row to several checkpoint blocks."""
    rng = np.random.default_rng(55 + with_cigar)
    widths = [1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, 511, 512, 513, 1023, 1024, 1025, 1536, 1537]
    ts, pp = [], []
    for w in widths:
        for tl in (1, 65, int(rng.integers(100, 900))):
            core = workloads.random_bases(rng, w).tobytes()
            mut = bytearray(core)
            for q in rng.integers(0, w, size=max(1, w // 20)):
                mut[q] = ord("ACGT"[int(rng.integers(0, 4))])
            t = workloads.random_bases(rng, int(rng.integers(0, 40))).tobytes() + bytes(mut)
            ts.append(t[:tl] if tl < len(t) else t + workloads.random_bases(rng, tl - len(t)).tobytes())
            pp.append(core)
    # (the extension entry, limit -1: no trace-cell limit and no score-kernel shared-memory refusal)
    want = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=with_cigar, trace_cell_limit=-1,
                           score_smem_limit=None)
    got = sw_gpu(ts, pp, scoring=(2, -3, 3, 1), with_cigar=with_cigar, trace_cell_limit=-1)
    assert got.status == api.Status.ok
    assert_sw_equal(got, want, f"band edges with_cigar={with_cigar}")
