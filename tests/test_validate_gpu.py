"""The result checks on the device (ga_wfa_validate_device,
ga_sw_validate_device) agree with the oracle's restatement of the reference's
validate / sw_validate on the kernels' own CIGARs and on altered ones (ops
swapped, flipped, dropped: each altered CIGAR stays inside its slot)."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, workloads

pytestmark = pytest.mark.gpu


def _alter(rng, cig: bytes) -> bytes:
    c = bytearray(cig)
    k = int(rng.integers(0, 5))
    if not c:
        return bytes(c)
    q = int(rng.integers(0, len(c)))
    if k == 0:
        c[q] = {77: 88, 88: 77, 73: 68, 68: 73}.get(c[q], 77)     # M<->X, I<->D
    elif k == 1:
        del c[q]                                                  # one op fewer
    elif k == 2:
        c[q] = ord("Z")                                           # not an op
    elif k == 3 and q + 1 < len(c):
        c[q], c[q + 1] = c[q + 1], c[q]                           # two ops swapped
    return bytes(c)


def _slots(b, n):
    oo = b.out_off.cpu().numpy()
    cap = b.a_len.cpu().numpy().astype(np.int64) + b.b_len.cpu().numpy()
    return oo, cap


def test_wfa_checks_on_device_match_oracle():
    torch = pytest.importorskip("torch")
    ps = workloads.wfa_mixed(n=3000, seed=31)
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    sc = torch.empty(b.n, dtype=torch.int32, device="cuda")
    ln = torch.empty(b.n, dtype=torch.int32, device="cuda")
    cg = torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda")
    api.wfa_device(b, 64, True, sc, ln, cg)
    torch.cuda.synchronize()
    pats, txts = ps.lists()
    s, L, C = sc.cpu().numpy(), ln.cpu().numpy().copy(), cg.cpu().numpy().copy()
    oo, cap = _slots(b, b.n)
    rng = np.random.default_rng(5)
    for i in range(b.n):                      # alter every other CIGAR, in place at the end of its slot
        if i % 2 and L[i] > 0:
            old = C[oo[i] + cap[i] - L[i]: oo[i] + cap[i]].tobytes()
            new = _alter(rng, old)
            C[oo[i] + cap[i] - len(new): oo[i] + cap[i]] = np.frombuffer(new, np.uint8)
            L[i] = len(new)
    ln.copy_(torch.from_numpy(L))
    cg.copy_(torch.from_numpy(C))
    fl = torch.empty(b.n, dtype=torch.uint8, device="cuda")
    api.wfa_validate_device(b, sc, ln, cg, fl)
    torch.cuda.synchronize()
    f = fl.cpu().numpy()
    bad = 0
    for i in range(b.n):
        if s[i] < 0 or L[i] <= 0:
            assert f[i] == 0
            continue
        cig = C[oo[i] + cap[i] - L[i]: oo[i] + cap[i]].tobytes()
        rs, wf = oracle.wfa_validate(cig, int(s[i]), pats[i], txts[i])
        assert (f[i] & 1, f[i] >> 1) == (rs, wf), i
        bad += not (rs and wf)
    assert bad > 100                           # the altered ones do fail


def test_sw_checks_on_device_match_oracle():
    torch = pytest.importorskip("torch")
    scheme = (2, -3, 3, 1)
    ps = workloads.sw_uneven_200k(n=2000, seed=32)
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    sc = torch.empty(b.n, dtype=torch.int32, device="cuda")
    pos = torch.empty(4 * b.n, dtype=torch.int32, device="cuda")
    ln = torch.empty(b.n, dtype=torch.int32, device="cuda")
    cg = torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda")
    api.sw_device(b, scheme, True, sc, pos, ln, cg)
    torch.cuda.synchronize()
    ts, pp = ps.lists()
    s, P4 = sc.cpu().numpy(), pos.cpu().numpy().reshape(-1, 4)
    L, C = ln.cpu().numpy().copy(), cg.cpu().numpy().copy()
    oo, cap = _slots(b, b.n)
    rng = np.random.default_rng(6)
    for i in range(b.n):
        if i % 2 and L[i] > 0:
            old = C[oo[i] + cap[i] - L[i]: oo[i] + cap[i]].tobytes()
            new = _alter(rng, old)
            C[oo[i] + cap[i] - len(new): oo[i] + cap[i]] = np.frombuffer(new, np.uint8)
            L[i] = len(new)
    ln.copy_(torch.from_numpy(L))
    cg.copy_(torch.from_numpy(C))
    fl = torch.empty(b.n, dtype=torch.uint8, device="cuda")
    api.sw_validate_device(b, scheme, sc, pos, ln, cg, fl)
    torch.cuda.synchronize()
    f = fl.cpu().numpy()
    bad = 0
    for i in range(b.n):
        if s[i] <= 0 or L[i] <= 0:
            assert f[i] == 0
            continue
        cig = C[oo[i] + cap[i] - L[i]: oo[i] + cap[i]].tobytes()
        si, sj, ei, ej = (int(v) for v in P4[i])
        rs, wf = oracle.sw_validate(cig, ts[i], si, ei, pp[i], sj, ej, scheme, int(s[i]))
        assert (f[i] & 1, f[i] >> 1) == (rs, wf), i
        bad += not (rs and wf)
    assert bad > 100
