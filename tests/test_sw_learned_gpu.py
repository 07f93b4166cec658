"""The SW variant model: the cost model's network in model slot 1, choosing
which pure pairs beyond the proven 16-bit bound try the 16-bit kernel.

Routing must never change a result (oracle-checked with the committed model
and with an all-zero model that sends every pure pair to the 16-bit kernel,
so the long pairs are handed over to the 32-bit kernel); the two model slots
are independent; the trained model takes more of the pairs that fit 16 bits
than the proven bound does, with few hand-overs."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import api, cost_model, sw_model, workloads
from helpers import assert_sw_equal

pytestmark = pytest.mark.gpu

SCORING = (2, -3, 3, 1)


def _subset():
    full = workloads.sw_long_4k()
    rng = np.random.default_rng(61)
    q = full.b_len
    mid = np.nonzero((q > 15000) & (q < 21000))[0]          # beyond the bound, may fit 16 bits
    small = np.nonzero(q < 6000)[0]
    idx = np.concatenate([rng.choice(mid, 10, replace=False), rng.choice(small, 14, replace=False)])
    return full.subset(idx)


@pytest.mark.parametrize("model", ["trained", "zero"])
def test_sw_learned_routing_is_bit_exact(model):
    torch = pytest.importorskip("torch")
    if model == "trained" and not sw_model.load_default():
        pytest.skip("no committed SW variant model")
    if model == "zero":
        with api.model_slot(1):
            api.cost_model_set(np.zeros(api.cost_model_nparams(), np.float32))
    ps = _subset()
    ts, pp = ps.lists()
    want = oracle.sw_batch(ts, pp, scoring=SCORING, with_cigar=True, trace_cell_limit=-1)
    got = api.align_sw_batch_packed(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, scoring=SCORING,
                                    with_cigar=True, trace_cell_limit=-1, learned=True)
    assert_sw_equal(got, want, f"host entry, {model} model")
    batch = api.DeviceBatchT(ps.a_buf, ps.a_off, ps.a_len, ps.b_buf, ps.b_off, ps.b_len, device="cuda")
    outs = [torch.full((ps.n,), -7, dtype=torch.int32, device="cuda"),
            torch.full((4 * ps.n,), -7, dtype=torch.int32, device="cuda"),
            torch.full((ps.n,), -7, dtype=torch.int32, device="cuda"),
            torch.zeros(batch.out_bytes, dtype=torch.uint8, device="cuda")]
    api.sw_device(batch, SCORING, True, *outs, trace_cell_limit=-1, learned=True)
    torch.cuda.synchronize()
    assert np.array_equal(outs[0].cpu().numpy(), want.score), model
    pos = outs[1].cpu().numpy().reshape(-1, 4)
    assert np.array_equal(pos[:, 2], want.end_i) and np.array_equal(pos[:, 0], want.start_i), model


def test_model_slots_are_independent():
    pytest.importorskip("torch")
    a = api.cost_model_init(5)
    b = api.cost_model_init(6)
    api.cost_model_set(a)
    with api.model_slot(1):
        api.cost_model_set(b)
        assert np.array_equal(api.cost_model_get(), b)
    assert np.array_equal(api.cost_model_get(), a)
    cost_model.load_default()


def test_trained_sw_model_takes_more_fitting_pairs_than_the_bound():
    pytest.importorskip("torch")
    if not sw_model.load_default():
        pytest.skip("no committed SW variant model")
    q = sw_model.routing_quality(sw_model.training_pairs(n=1024, seed=2003))
    assert q["fit_16bit"] > q["taken_by_bound"]
    assert q["fit_but_left_by_model"] < q["fit_but_left_by_bound"]
    assert q["taken_but_handed_over_by_model"] <= 0.05 * max(1, q["taken_by_model"])
