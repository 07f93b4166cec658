"""Smith-Waterman launches sized on the device from the device-built plan.

The host entry enqueues every launch without reading the plan back (sizes are
bounded from the lengths on the host; each kernel takes its exact items and
per-warp memory from the plan on the device) and replays each range's work as
a CUDA graph; a synchronous ga_sw_device call with a cell limit replays the
graph of its launch shape.  Results must equal the oracle's call after call,
including when the pairs behind the same device pointers grow past the memory
the graph was captured with (the kernels flag it and the call runs again
through the read-back path)."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, workloads

pytestmark = pytest.mark.gpu

SCORING = (2, -3, 3, 1)


def _outs(torch, batch):
    n = batch.n
    return (torch.full((n,), -7, dtype=torch.int32, device="cuda"),
            torch.full((4 * n,), -7, dtype=torch.int32, device="cuda"),
            torch.full((n,), -7, dtype=torch.int32, device="cuda"),
            torch.zeros(max(batch.out_bytes, 1), dtype=torch.uint8, device="cuda"))


def _check(batch, outs, want, label):
    sc, pos, ln, cg = (t.cpu().numpy() for t in outs)
    assert np.array_equal(sc, want.score), label
    pos = pos.reshape(-1, 4)
    for k, f in enumerate(("start_i", "start_j", "end_i", "end_j")):
        assert np.array_equal(pos[:, k], getattr(want, f)), (label, f)
    ends = (batch.out_off.cpu().numpy() + batch.a_len.cpu().numpy().astype(np.int64) +
            batch.b_len.cpu().numpy().astype(np.int64))
    for i, c in enumerate(want.cigars):
        assert int(ln[i]) == len(c), (label, i)
        assert cg[ends[i] - len(c):ends[i]].tobytes() == c, (label, i)


def test_sw_device_sync_calls_replay_one_graph():
    torch = pytest.importorskip("torch")
    ps = workloads.sw_uneven_200k(n=2000, seed=31)
    ts, pp = ps.lists()
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    outs = _outs(torch, batch)
    for call in range(3):
        for t in outs:
            t.fill_(-7 if t.dtype == torch.int32 else 0)
        api.sw_device(batch, SCORING, True, *outs, stream=None, trace_cell_limit=1 << 26)
        _check(batch, outs, want, f"call {call}")


def test_sw_device_graph_after_pairs_grow_behind_the_same_pointers():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(32)
    full_t, full_p = [], []
    for _ in range(8):
        q = workloads.random_bases(rng, 2000)
        core, _ = workloads.mutate_point(rng, q, np.array([2000]), 0.05, (0.6, 0.2, 0.2))
        full_t.append(np.concatenate([workloads.random_bases(rng, 200), core]).tobytes())
        full_p.append(q.tobytes())
    ps = workloads.from_lists("grow", full_t, full_p)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    a_full, b_full = batch.a_len.clone(), batch.b_len.clone()
    # first calls on the pairs' first 300 x 150 bases (the graph's memory is
    # sized for them), then on the whole pairs behind the same pointers
    batch.a_len.copy_(torch.clamp(a_full, max=300))
    batch.b_len.copy_(torch.clamp(b_full, max=150))
    small = oracle.sw_batch([t[:300] for t in full_t], [p[:150] for p in full_p], scoring=SCORING, with_cigar=True)
    outs = _outs(torch, batch)
    for call in range(2):
        api.sw_device(batch, SCORING, True, *outs, stream=None, trace_cell_limit=1 << 26)
        _check(batch, outs, small, f"short pairs, call {call}")
    batch.a_len.copy_(a_full)
    batch.b_len.copy_(b_full)
    torch.cuda.synchronize()
    big = oracle.sw_batch(full_t, full_p, scoring=SCORING, with_cigar=True)
    for call in range(2):
        outs = _outs(torch, batch)
        api.sw_device(batch, SCORING, True, *outs, stream=None, trace_cell_limit=1 << 26)
        _check(batch, outs, big, f"grown pairs, call {call}")


def test_sw_host_entry_repeats_replay_the_same_graphs():
    """Two calls of a ranged host batch (each range's device work a graph)
    and a score-only call in between: identical results, equal to the oracle."""
    ps = workloads.sw_uneven_200k(n=30000, seed=33)
    ts, pp = ps.lists()
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True)
    for call in range(2):
        got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                        scoring=SCORING, with_cigar=True)
        assert got.status == api.Status.ok, got.error
        for f in ("score", "start_i", "start_j", "end_i", "end_j"):
            assert np.array_equal(got.res[f], getattr(want, f)), (call, f)
        assert all(got.cigar(i) == want.cigars[i] for i in range(ps.n)), call
        so = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len,
                                       scoring=SCORING, with_cigar=False)
        assert so.status == api.Status.ok and np.array_equal(so.res["score"], want.score), call
