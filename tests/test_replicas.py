"""Replicas on CPU ranks (gloo): the partitioner and the gather give, on k
ranks, exactly the 1-rank results.  The per-range aligner here is the oracle
(the GPU path is exercised by the GPU tests); what is under test is the
partitioning and the reassembly in request order."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from genoaligner_gb300 import replicas, workloads


def test_partition_is_contiguous_and_balanced():
    rng = np.random.default_rng(3)
    w = rng.integers(1, 1000, size=1000)
    for world in (1, 2, 3, 8):
        r = replicas.partition(w, world)
        assert r[0][0] == 0 and r[-1][1] == 1000
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        share = w.sum() / world
        for lo, hi in r:
            assert w[lo:hi].sum() <= share + w.max()


def test_partition_edge_cases():
    assert replicas.partition([], 3) == [(0, 0)] * 3
    assert replicas.partition([5], 2) in ([(0, 1), (1, 1)], [(0, 0), (0, 1)])
    r = replicas.partition([0, 0, 0, 0], 2)
    assert r[0][0] == 0 and r[-1][1] == 4
    with pytest.raises(ValueError):
        replicas.partition([1, -1], 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_q):
    import torch.distributed as dist

    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ps = workloads.sw_uneven_200k(n=120, seed=11)
        ts, pp = ps.lists()

        def align_range(lo, hi):
            r = oracle.sw_batch(ts[lo:hi], pp[lo:hi], scoring=(2, -3, 3, 1), with_cigar=True, threads=1)
            return [(int(r.score[i]), r.cigars[i]) for i in range(hi - lo)]

        res = replicas.run_replicated(align_range, ps.n, replicas.sw_weights(ps.a_len, ps.b_len), rank, world,
                                      gather=replicas.torch_gather)
        if rank == 0:
            out_q.put(res)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_replicated_results_equal_single_rank(world):
    import oracle
    ps = workloads.sw_uneven_200k(n=120, seed=11)
    ts, pp = ps.lists()
    one = oracle.sw_batch(ts, pp, scoring=(2, -3, 3, 1), with_cigar=True, threads=1)
    want = [(int(one.score[i]), one.cigars[i]) for i in range(ps.n)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == want
