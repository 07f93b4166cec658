"""WFA on real sequences: the human and chimp mitochondrial genomes cut into
the batches of the reference's real-sequence test (fragments, the
repeat-rich control region, human/chimp windows that stay unresolved at smax
64 and 200 and resolve at 100 bp, the whole genomes at smax 511, a window
around the human N), through the host entry, plain and learned.  Expected:
the reference's own kernels' outputs (tests/golden/real_golden.json.gz,
tests/golden/make_real_golden.py), field by field."""
import numpy as np
import pytest

from genoaligner_gb300 import api, cost_model
from helpers import wfa_gpu

pytestmark = pytest.mark.gpu


def _enc(s):
    return s.encode("latin-1")


@pytest.mark.parametrize("learned", [False, True])
def test_real_sequences_match_reference(real_golden, learned):
    if learned:
        assert cost_model.load_default()
    resolved_100bp = 0
    for rec in real_golden:
        pats = [_enc(p) for p, _ in rec["pairs"]]
        txts = [_enc(t) for _, t in rec["pairs"]]
        got = wfa_gpu(pats, txts, smax=np.array(rec["smax"]), with_cigar=np.array(rec["with_cigar"]),
                      learned=learned)
        assert got.status == api.Status.ok, (rec["name"], got.error)
        res = got.res
        for i, want in enumerate(rec["results"]):
            assert res["score"][i] == want["score"], (rec["name"], i)
            assert bool(res["resolved"][i]) == bool(want["resolved"]), (rec["name"], i)
            assert got.cigar(i).decode() == want["cigar"], (rec["name"], i)
            assert bool(res["rescore_ok"][i]) == bool(want["rescore_ok"]), (rec["name"], i)
            assert bool(res["wellformed_ok"][i]) == bool(want["wellformed_ok"]), (rec["name"], i)
            d, smax = rec["edit_distance"][i], rec["smax"][i]
            assert bool(res["resolved"][i]) == (d <= smax), (rec["name"], i)
        assert got.resolved_count == rec["resolved_count"], rec["name"]
        assert got.unresolved_count == rec["unresolved_count"], rec["name"]
        if "100 bp" in rec["name"]:
            resolved_100bp = got.resolved_count
    assert resolved_100bp > 0              # a batch that resolves nothing proves nothing
