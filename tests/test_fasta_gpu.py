"""FASTA ingest on the GPU: the pinned record arena goes to the device as is
and aligns there (results equal the oracle's), the device 2-bit packing and
non-ACGT masks equal a numpy restatement, and a batch whose requests share one
reference stages that reference once."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, workloads

pytestmark = pytest.mark.gpu


def _pack_ref(arena: np.ndarray):
    """2-bit words and masks of every 32-byte chunk (A 0, C 1, G 2, T 3 under
    ((b >> 1) ^ (b >> 2)) & 3, first byte lowest; mask bit k = byte k not ACGT)."""
    ch = arena.reshape(-1, 32).astype(np.uint64)
    codes = ((ch >> np.uint64(1)) ^ (ch >> np.uint64(2))) & np.uint64(3)
    words = (codes << (np.arange(32, dtype=np.uint64) * np.uint64(2))).sum(axis=1, dtype=np.uint64)
    bad = ~np.isin(arena.reshape(-1, 32), np.frombuffer(b"ACGT", np.uint8))
    masks = (bad.astype(np.uint64) << np.arange(32, dtype=np.uint64)).sum(axis=1, dtype=np.uint64)
    return words.astype(np.uint64), masks.astype(np.uint32)


def test_pack_2bit_device_matches_numpy():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    arena = rng.choice(np.frombuffer(b"ACGTACGTACGTNacgtRY-\x00\xff", np.uint8), size=32 * 5000)
    seq = torch.from_numpy(arena).cuda()
    packed = torch.empty(5000, dtype=torch.int64, device="cuda")
    mask = torch.empty(5000, dtype=torch.int32, device="cuda")
    api.pack_2bit_device(seq, packed, mask)
    torch.cuda.synchronize()
    w, m = _pack_ref(arena)
    assert np.array_equal(packed.cpu().numpy().view(np.uint64), w)
    assert np.array_equal(mask.cpu().numpy().view(np.uint32), m)


def test_fasta_arena_aligns_on_device(tmp_path):
    torch = pytest.importorskip("torch")
    recs, baits = workloads.gene_family(60, 120, 11)
    p = tmp_path / "g.fa"
    workloads.write_fasta(p, recs + baits, width=70, crlf=True)
    fs = api.fasta_read(str(p))
    assert fs.pinned
    seq = torch.empty(fs.arena.nbytes, dtype=torch.uint8, device="cuda")
    fs.upload(seq)
    # pairs: record k (text) against record k + 1 (pattern)
    n = fs.n - 1
    batch = api.DeviceBatchT.from_device_arena(seq, fs.offsets[:-1].copy(), fs.lengths[:-1].copy(),
                                               fs.offsets[1:].copy(), fs.lengths[1:].copy())
    sc = torch.empty(n, dtype=torch.int32, device="cuda")
    pos = torch.empty(4 * n, dtype=torch.int32, device="cuda")
    ln = torch.empty(n, dtype=torch.int32, device="cuda")
    cg = torch.empty(batch.out_bytes, dtype=torch.uint8, device="cuda")
    api.sw_device(batch, (2, -3, 3, 1), True, sc, pos, ln, cg)
    torch.cuda.synchronize()
    ts = [fs.sequence(k) for k in range(n)]
    ps = [fs.sequence(k + 1) for k in range(n)]
    want = oracle.sw_batch(ts, ps, scoring=(2, -3, 3, 1), with_cigar=True, trace_cell_limit=-1)
    assert np.array_equal(sc.cpu().numpy(), want.score)
    L = ln.cpu().numpy()
    oo = batch.out_off.cpu().numpy()
    cgh = cg.cpu().numpy()
    for k in range(n):
        if want.score[k] > 0:
            cap = len(ts[k]) + len(ps[k])
            w = want.cigars[k]
            assert cgh[oo[k] + cap - L[k]: oo[k] + cap].tobytes() == (w if isinstance(w, bytes) else w.encode())


def test_shared_reference_is_staged_once():
    recs, baits = workloads.gene_family(200, 300, 12)
    bait = baits[1][1]
    texts = [s for _, s in recs]
    reqs = [api.SWRequest(t, len(t), bait, len(bait), api.SWScoring(1, -1, 2, 1)) for t in texts]
    got = api.align_sw_batch(reqs)
    h2d_shared, _ = api.last_transfer_bytes()
    # the same requests with a private copy of the bait each
    reqs2 = [api.SWRequest(t, len(t), bytes(bytearray(bait)), len(bait), api.SWScoring(1, -1, 2, 1)) for t in texts]
    got2 = api.align_sw_batch(reqs2)
    h2d_private, _ = api.last_transfer_bytes()
    assert got.ok() and got2.ok()
    assert [(r.score, r.cigar) for r in got.results] == [(r.score, r.cigar) for r in got2.results]
    assert h2d_private - h2d_shared >= 199 * (len(bait) // 32) * 32
    want = oracle.sw_batch(texts, [bait] * len(texts), scoring=(1, -1, 2, 1), with_cigar=True)
    assert [r.score for r in got.results] == list(want.score)
    assert [r.cigar.encode() if isinstance(r.cigar, str) else r.cigar for r in got.results] == \
        [w if isinstance(w, bytes) else w.encode() for w in want.cigars]
