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
