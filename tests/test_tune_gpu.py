"""The autotuner on the GPU: every kernel setting gives the same results (and
the oracle's), the search keeps the fastest candidate it timed, and a saved
setting loads back."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, cost_model, workloads

pytestmark = pytest.mark.gpu


def _sw_batch():
    """Uneven 16-bit pairs, pairs with bytes outside ACGT (32-bit kernel) and
    pairs of 2^20 .. 2^23 cells (long shape at low thresholds)."""
    ps = workloads.sw_uneven_200k(n=1500, seed=41)
    ts, pp = ps.lists()
    rng = np.random.default_rng(42)
    for k in range(40):
        t = bytearray(ts[k])
        t[int(rng.integers(0, len(t)))] = ord("N")
        ts[k] = bytes(t)
    for q in (1200, 2100, 2900):
        core = workloads.random_bases(rng, q)
        mut, _ = workloads.mutate_point(rng, core, np.array([q]), 0.08, (0.6, 0.2, 0.2))
        ts.append(workloads.random_bases(rng, 400).tobytes() + mut.tobytes() + workloads.random_bases(rng, 400).tobytes())
        pp.append(core.tobytes())
    return ts, pp


def _device(ts, pp):
    ps = workloads.from_lists("t", ts, pp)
    return api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)


def _sw_outputs(torch, b):
    return (torch.empty(b.n, dtype=torch.int32, device="cuda"), torch.empty(4 * b.n, dtype=torch.int32, device="cuda"),
            torch.empty(b.n, dtype=torch.int32, device="cuda"), torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda"))


def _host(torch, outs):
    torch.cuda.synchronize()
    return tuple(o.cpu().numpy() for o in outs)


def _check_sw(res, want, b, ts, pp):
    sc, pos, ln, cg = res
    oo = b.out_off.cpu().numpy()
    for i in range(b.n):
        assert sc[i] == want.score[i], i
        if sc[i] > 0:
            cap = len(ts[i]) + len(pp[i])
            cig = cg[oo[i] + cap - ln[i]: oo[i] + cap].tobytes()
            w = want.cigars[i]
            assert cig == (w if isinstance(w, bytes) else w.encode()), i


@pytest.fixture
def restore_tune():
    before = api.tune_get()
    yield
    api.tune_set(**before)


def test_every_sw_setting_gives_the_same_results(restore_tune):
    torch = pytest.importorskip("torch")
    ts, pp = _sw_batch()
    scheme = (2, -3, 3, 1)
    want = oracle.sw_batch(ts, pp, scoring=scheme, with_cigar=True, trace_cell_limit=-1)
    b = _device(ts, pp)
    first = None
    combos = [(p, w, lg, 40) for p in (1, 0) for w in (2, 4) for lg in (16, 20, 24, 30)]
    # whole-block pairs: every long-shape pair (above 2^16 / 2^20 cells) on a block's 4 warps
    combos += [(1, 2, 16, 16), (0, 2, 16, 16), (0, 2, 20, 18), (0, 4, 16, 20)]
    for pack16, window, long_log2, coop in combos:
        api.tune_set(sw_pack16=pack16, sw_window=window, sw_long_log2=long_log2, sw_coop_log2=coop)
        outs = _sw_outputs(torch, b)
        api.sw_device(b, scheme, True, *outs)
        res = _host(torch, outs)
        if first is None:
            first = res
            _check_sw(res, want, b, ts, pp)
        else:
            for x, y in zip(first, res):
                assert np.array_equal(x, y), (pack16, window, long_log2, coop)


def test_autotune_sw_keeps_its_fastest_candidate(restore_tune):
    torch = pytest.importorskip("torch")
    ts, pp = _sw_batch()
    scheme = (2, -3, 3, 1)
    b = _device(ts, pp)
    outs = _sw_outputs(torch, b)
    chosen, trials = api.autotune_sw(b, scheme, *outs, reps=1)
    assert len(trials) >= 3
    assert {t["sw_pack16"] for t, _ in trials} == {0, 1}
    # coordinate search: the kept setting is the fastest of the last sweep
    last = [t for t, _ in trials if all(t[f] == chosen[f] for f in ("sw_pack16", "sw_window"))]
    assert chosen in last
    assert api.tune_get() == chosen
    want = oracle.sw_batch(ts, pp, scoring=scheme, with_cigar=True, trace_cell_limit=-1)
    _check_sw(_host(torch, outs), want, b, ts, pp)


def test_every_wfa_lane_setting_gives_the_same_results(restore_tune):
    torch = pytest.importorskip("torch")
    assert cost_model.load_default()
    ps = workloads.wfa_mixed(n=20_000, seed=73)
    b = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)
    base = None
    for lane, group in ((0, 32), (0, 16), (0, 8), (4, 8), (15, 16), (31, 32), (31, 8)):
        api.tune_set(wfa_lane_smax=lane, wfa_group=group)
        sc = torch.full((b.n,), -7, dtype=torch.int32, device="cuda")
        ln = torch.zeros(b.n, dtype=torch.int32, device="cuda")
        cg = torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda")
        api.wfa_device(b, 64, True, sc, ln, cg, learned=True)
        res = _host(torch, (sc, ln, cg))
        small, big, _ = api.wfa_route_stats()
        if lane == 0:
            assert small == 0
        else:
            assert small > 0
        if base is None:
            base = res
        else:
            for x, y in zip(base, res):
                assert np.array_equal(x, y), (lane, group)
    sc = torch.full((b.n,), -7, dtype=torch.int32, device="cuda")
    ln = torch.zeros(b.n, dtype=torch.int32, device="cuda")
    cg = torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda")
    chosen, trials = api.autotune_wfa(b, 64, True, sc, ln, cg, reps=1)
    assert api.tune_get() == chosen and len(trials) == 7      # 5 lane bounds, then the 2 other group sizes
    assert min(trials, key=lambda x: x[1])[0] == chosen
    for x, y in zip(base, _host(torch, (sc, ln, cg))):
        assert np.array_equal(x, y)


def test_saved_setting_loads_back(tmp_path, restore_tune):
    api.tune_set(sw_pack16=0, sw_window=4, sw_long_log2=20, wfa_lane_smax=8, sw_coop_log2=25, sw_opt16_pct=60,
                 wfa_group=16)
    p = tmp_path / "tune.txt"
    api.tune_save(str(p))
    api.tune_set(**api.tune_default())
    api.tune_load(str(p))
    assert api.tune_get() == {"sw_pack16": 0, "sw_window": 4, "sw_long_log2": 20, "wfa_lane_smax": 8,
                              "sw_coop_log2": 25, "sw_opt16_pct": 60, "wfa_group": 16}
    assert api.device_name() in p.read_text()
