"""ga_wfa_device_noalloc: the WFA entry for callers that cannot allocate device
memory (their memory belongs to a pool allocator, or they cannot afford
cudaMalloc's synchronisation).  It must return exactly what the allocating
entry ga_wfa_device returns, call after call, although every call reuses the
same 16 MiB scratch array; and it must refuse batches that do not fit.

Kept in its own file so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

from genoaligner_gb300 import api, workloads

pytestmark = pytest.mark.gpu


def _noalloc():
    L = api.load()
    f = L.ga_wfa_device_noalloc
    f.argtypes = [ctypes.POINTER(api.DeviceBatch), ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_char_p)]
    f.restype = ctypes.c_int32
    return f


def _outputs(torch, batch, fill):
    sc = torch.full((batch.n,), fill, dtype=torch.int32, device="cuda")
    ln = torch.full((batch.n,), fill, dtype=torch.int32, device="cuda")
    cg = torch.zeros(max(batch.out_bytes, 1), dtype=torch.uint8, device="cuda")
    return sc, ln, cg


def test_noalloc_matches_allocating_entry_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    f = _noalloc()
    batches = [workloads.wfa_150bp_2pct(n=3000, seed=17), workloads.wfa_mixed(n=4000, seed=18)]
    for call, ps in enumerate(batches + batches[:1]):         # three calls in a row, two different batches
        batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
        ref = _outputs(torch, batch, -7)
        api.wfa_device(batch, 64, True, *ref)
        got = _outputs(torch, batch, -9)
        err = ctypes.c_char_p()
        st = f(ctypes.byref(batch.c), 64, 1, got[0].data_ptr(), got[1].data_ptr(), got[2].data_ptr(), None,
               ctypes.byref(err))
        assert st == api.GA_OK, (call, err.value)
        torch.cuda.synchronize()
        assert torch.equal(got[0], ref[0]), call
        assert torch.equal(got[1], ref[1]), call
        assert torch.equal(got[2], ref[2]), call
        assert int((got[0] >= 0).sum()) > 0.9 * ps.n


def test_noalloc_score_only_matches():
    torch = pytest.importorskip("torch")
    f = _noalloc()
    ps = workloads.wfa_mixed(n=2000, seed=19)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    ref = _outputs(torch, batch, -7)
    api.wfa_device(batch, 32, False, *ref)
    for _ in range(2):
        got = _outputs(torch, batch, -9)
        err = ctypes.c_char_p()
        st = f(ctypes.byref(batch.c), 32, 0, got[0].data_ptr(), got[1].data_ptr(), got[2].data_ptr(), None,
               ctypes.byref(err))
        assert st == api.GA_OK, err.value
        torch.cuda.synchronize()
        assert torch.equal(got[0], ref[0])


def test_noalloc_refuses_oversized_batch():
    torch = pytest.importorskip("torch")
    f = _noalloc()
    ps = workloads.wfa_150bp_2pct(n=200, seed=20)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    got = _outputs(torch, batch, -9)
    err = ctypes.c_char_p()
    # smax 1100: four wavefront stacks need 4 * 1101^2 * 4 bytes, above 16 MiB
    st = f(ctypes.byref(batch.c), 1100, 1, got[0].data_ptr(), got[1].data_ptr(), got[2].data_ptr(), None,
           ctypes.byref(err))
    assert st == api.GA_INVALID_ARGUMENT
    assert b"16 MiB" in err.value
    assert int((got[0] == -9).sum()) == ps.n                  # nothing ran


def test_noalloc_on_a_caller_stream_and_large_smax():
    """A call on the caller's own stream returns once enqueued; after that
    stream is synchronised the results equal the allocating entry's.  A trace
    call at smax 600 (four stacks of 601^2 ints, most of the scratch) checks
    the slot arithmetic near the array's end."""
    torch = pytest.importorskip("torch")
    f = _noalloc()
    ps = workloads.wfa_mixed(n=3000, seed=21)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    s = torch.cuda.Stream()
    for smax in (64, 600):
        ref = _outputs(torch, batch, -7)
        api.wfa_device(batch, smax, True, *ref)
        for _ in range(2):
            got = _outputs(torch, batch, -9)
            torch.cuda.synchronize()
            err = ctypes.c_char_p()
            st = f(ctypes.byref(batch.c), smax, 1, got[0].data_ptr(), got[1].data_ptr(), got[2].data_ptr(),
                   ctypes.c_void_p(s.cuda_stream), ctypes.byref(err))
            assert st == api.GA_OK, (smax, err.value)
            s.synchronize()
            assert torch.equal(got[0], ref[0]), smax
            assert torch.equal(got[1], ref[1]), smax
            assert torch.equal(got[2], ref[2]), smax


def test_noalloc_empty_batch_and_refusals():
    torch = pytest.importorskip("torch")
    f = _noalloc()
    ps = workloads.wfa_150bp_2pct(n=64, seed=22)
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    got = _outputs(torch, batch, -9)
    err = ctypes.c_char_p()
    empty = api.DeviceBatch(batch.c.seq, batch.c.seq_bytes, batch.c.a_off, batch.c.a_len, batch.c.b_off,
                            batch.c.b_len, batch.c.out_off, 0, 0)
    assert f(ctypes.byref(empty), 64, 1, None, None, None, None, ctypes.byref(err)) == api.GA_OK
    # an arena that does not start on a 16-byte boundary
    odd = api.DeviceBatch(batch.c.seq + 8, batch.c.seq_bytes - 8, batch.c.a_off, batch.c.a_len, batch.c.b_off,
                          batch.c.b_len, batch.c.out_off, batch.n, 0)
    st = f(ctypes.byref(odd), 64, 1, got[0].data_ptr(), got[1].data_ptr(), got[2].data_ptr(), None,
           ctypes.byref(err))
    assert st == api.GA_INVALID_ARGUMENT and b"16-byte" in err.value
    # smax beyond the device entries' bound, and a negative arena size
    st = f(ctypes.byref(batch.c), api.GA_MAX_SMAX_DEVICE + 1, 0, got[0].data_ptr(), None, None, None,
           ctypes.byref(err))
    assert st == api.GA_INVALID_ARGUMENT
    neg = api.DeviceBatch(batch.c.seq, -32, batch.c.a_off, batch.c.a_len, batch.c.b_off, batch.c.b_len,
                          batch.c.out_off, batch.n, 0)
    st = f(ctypes.byref(neg), 64, 0, got[0].data_ptr(), None, None, None, ctypes.byref(err))
    assert st == api.GA_INVALID_ARGUMENT
    torch.cuda.synchronize()
    assert int((got[0] == -9).sum()) == ps.n                  # nothing ran
