"""The learned cost model on the GPU: exactness of the sketch bound, gradients
of the hand-written backward kernel against a float64 reference, training,
and the rule that routing never changes a result."""
import numpy as np
import pytest

import oracle
from oracle import mlp_ref
from genoaligner_gb300 import api, cost_model, workloads

pytestmark = pytest.mark.gpu


def _batch(ps):
    return api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len)


def test_lower_bound_never_exceeds_distance():
    ps = workloads.wfa_mixed(n=3000, seed=71)
    f, lb = api.wfa_features(_batch(ps))
    pats, txts = ps.lists()
    ed = oracle.edit_distance(pats, txts)
    lb = lb.cpu().numpy()
    assert (lb <= ed).all()
    assert (lb > 0).mean() > 0.5                 # the bound is not vacuous
    feat = f.cpu().numpy()
    assert np.allclose(feat[:, 64], ps.a_len / 256.0) and np.allclose(feat[:, 65], ps.b_len / 256.0)


def test_mlp_forward_and_gradient_match_float64_reference():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    params = api.cost_model_init(seed=3)
    params[-2:] = [1.0, -0.5]
    api.cost_model_set(params)
    x = rng.normal(0, 1, size=(300, 66)).astype(np.float32)
    t = rng.normal(2, 1, size=(300, 2)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    tt = torch.from_numpy(t).cuda()
    y = api.mlp_forward(xt).cpu().numpy()
    y_ref, _ = mlp_ref.forward(params, x)
    assert np.allclose(y, y_ref, rtol=1e-4, atol=1e-4)
    g, loss = api.mlp_gradient(xt, tt)
    g_ref, loss_ref = mlp_ref.gradient(params, x, t)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref) + 1e-4
    # tolerance: fp32 accumulation over a batch of 300 against float64
    err = np.abs(g - g_ref)
    assert err.max() <= 1e-3 * np.abs(g_ref).max() + 1e-5, (err.max(), np.abs(g_ref).max())
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert rel < 1e-4, rel


def test_tensor_core_forward_matches_bf16_reference():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    params = api.cost_model_init(seed=4)
    api.cost_model_set(params)
    x = (rng.integers(-40, 41, size=(1000, 66)) / 8.0).astype(np.float32)    # count differences / 8
    x[:, 64:] = rng.uniform(0.5, 1.0, size=(1000, 2))
    y = api.mlp_forward_fast(torch.from_numpy(x).cuda()).cpu().numpy()
    y_ref = mlp_ref.forward_bf16_activations(params, x)
    # tolerance: fp32 accumulation order against float64, on bf16-rounded operands
    scale = np.abs(y_ref).max()
    assert np.abs(y - y_ref).max() <= 2e-3 * scale + 1e-3, (np.abs(y - y_ref).max(), scale)


def test_training_reduces_loss():
    ps = cost_model.training_pairs(n=60_000, seed=77)
    feat, targ, dist, lb = cost_model.labels_and_features(ps)
    rec = cost_model.train(feat, targ, epochs=2, batch=2048, lr=3e-3, seed=5)
    first, last = np.mean(rec["losses"][:5]), np.mean(rec["losses"][-5:])
    assert last < 0.2 * first, (first, last)
    ev = cost_model.evaluate(feat, dist, lb)
    assert ev["mae_distance"] < ev["mae_distance_lower_bound_only"]


@pytest.mark.parametrize("model", ["zero", "trained"])
def test_learned_routing_is_bit_exact(model):
    torch = pytest.importorskip("torch")
    if model == "zero":
        api.cost_model_set(np.zeros(api.cost_model_nparams(), np.float32))   # predicts d = 0: many escalations
    else:
        assert cost_model.load_default(), "the committed model is missing"
    ps = workloads.wfa_mixed(n=40_000, seed=72)
    b = _batch(ps)
    for smax, trace in ((64, True), (20, True), (64, False)):
        out = []
        for learned in (False, True):
            sc = torch.full((b.n,), -7, dtype=torch.int32, device="cuda")
            ln = torch.zeros(b.n, dtype=torch.int32, device="cuda")
            cg = torch.zeros(b.out_bytes, dtype=torch.uint8, device="cuda")
            api.wfa_device(b, smax, trace, sc, ln, cg, learned=learned)
            torch.cuda.synchronize()
            out.append((sc.cpu().numpy(), ln.cpu().numpy(), cg.cpu().numpy()))
        (s0, l0, c0), (s1, l1, c1) = out
        assert np.array_equal(s0, s1), (model, smax, trace)
        if trace:
            assert np.array_equal(l0, l1) and np.array_equal(c0, c1), (model, smax, trace)
        small, big, esc = api.wfa_route_stats()
        assert small + big <= b.n
        if model == "zero" and smax == 64:
            assert esc[0] > 0                     # the poor model escalates, results unchanged
        if model == "trained" and smax == 64:
            # the routed path computes its features from the 2-bit arena: a
            # wrong feature order there would show up as mispredictions
            assert small > 0.5 * b.n, (small, big)
            assert esc[0] < 0.05 * (small + big), esc


def test_learned_host_entry_matches_oracle():
    assert cost_model.load_default()
    ps = workloads.wfa_mixed(n=5000, seed=73)
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=64, with_cigar=True)
    got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=64,
                                 with_cigar=True, learned=True)
    assert got.status == api.Status.ok
    assert np.array_equal(got.res["score"], want.score)
    assert all(got.cigar(i) == want.cigars[i] for i in range(ps.n))
    assert np.array_equal(got.res["rescore_ok"].astype(bool), want.rescore_ok)


def test_trained_model_beats_lower_bound_rule():
    """What the trained network gains over routing without it: its distance
    estimate is closer and far fewer pairs escalate past their first smax."""
    assert cost_model.load_default()
    hold = workloads.wfa_mixed(n=100_000, seed=4041)
    feat, targ, dist, lb = cost_model.labels_and_features(hold)
    ev = cost_model.evaluate(feat, dist, lb)
    assert ev["mae_distance"] < 0.5 * ev["mae_distance_lower_bound_only"], ev
    assert ev["escalation_rate"] < ev["escalation_rate_lower_bound_only"], ev
    assert ev["escalation_rate"] < 0.05, ev


def test_learned_whole_block_items_match_oracle():
    """Long, divergent pairs at smax 2048: the warp queue's items estimated at
    s >= 256 run on whole blocks of the warp kernel; scores and CIGARs equal
    the oracle's and the plain path's."""
    assert cost_model.load_default()
    ps = workloads.wfa_long_1k_10k(n=48, seed=33)
    pats, txts = ps.lists()
    want = oracle.wfa_batch(pats, txts, smax=2048, with_cigar=True, max_smax=4096)
    assert (want.score >= 256).sum() >= 5
    got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=2048,
                                 with_cigar=True, max_smax=4096, learned=True)
    assert got.status == api.Status.ok
    assert np.array_equal(got.res["score"], want.score)
    assert all(got.cigar(i) == want.cigars[i] for i in range(ps.n))
    assert np.array_equal(got.res["rescore_ok"].astype(bool), want.rescore_ok)
    small, big, rest = api.wfa_route_stats()
    assert rest[1] >= 3, rest                              # pairs that ran on whole blocks
    plain = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=2048,
                                   with_cigar=True, max_smax=4096, learned=False)
    assert np.array_equal(plain.res["score"], got.res["score"])


@pytest.mark.parametrize("group", [8, 16, 32])
def test_warp_queue_group_sizes_match_oracle(group):
    """The warp queue's pairs on groups of 8 or 16 lanes (several pairs per
    warp, stepping through the wavefronts together) or on whole warps: pairs
    with bytes outside ACGT (byte compare), empty sides, pairs longer than the
    lane queue takes, unresolved pairs and the mixed batch's divergent ones,
    every field against the oracle."""
    assert cost_model.load_default()
    before = api.tune_get()
    ps = workloads.wfa_mixed(n=4000, seed=74)
    pats, txts = ps.lists()
    rng = np.random.default_rng(75)
    bases = np.frombuffer(b"ACGT", np.uint8)
    for k in range(0, 200, 5):                        # an N or a lower-case base in one side
        b = bytearray(txts[k])
        b[int(rng.integers(0, len(b)))] = ord("N") if k % 2 else ord("a")
        txts[k] = bytes(b)
    pats[200], txts[200] = b"", b"ACGTACGT"
    pats[201], txts[201] = b"ACGTA", b""
    pats[202], txts[202] = b"", b""
    for k in range(210, 260):                         # 300-600 bases, 5-12 % point changes
        L = int(rng.integers(300, 601))
        s = bases[rng.integers(0, 4, L)].tobytes()
        t = bytearray(s)
        for i in rng.choice(L, size=int(L * rng.uniform(0.05, 0.12)), replace=False):
            t[i] = bases[(bases.tolist().index(t[i]) + 1 + int(rng.integers(0, 3))) % 4]
        pats[k], txts[k] = s, bytes(t)
    for k in range(260, 280):                         # unrelated: unresolved at smax 64
        pats[k] = bases[rng.integers(0, 4, 180)].tobytes()
        txts[k] = bases[rng.integers(0, 4, 200)].tobytes()
    ps = workloads.from_lists("wfa_group_cases", pats, txts)
    want = oracle.wfa_batch(pats, txts, smax=64, with_cigar=True)
    assert (want.score < 0).sum() >= 20 and (want.score > 30).sum() >= 50
    try:
        for lane in (0, 31):
            api.tune_set(wfa_lane_smax=lane, wfa_group=group)
            got = api.align_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, smax=64,
                                         with_cigar=True, learned=True)
            assert got.status == api.Status.ok
            assert np.array_equal(got.res["score"], want.score), (group, lane)
            assert all(got.cigar(i) == want.cigars[i] for i in range(ps.n)), (group, lane)
            assert np.array_equal(got.res["rescore_ok"].astype(bool), want.rescore_ok), (group, lane)
    finally:
        api.tune_set(**before)
