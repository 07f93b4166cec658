"""The traceback walk of the 16-bit SW kernel on pairs shaped to stress its
shortcuts: long identical stretches (the walk hops diagonally from checkpoint
row to checkpoint row, 64 rows at a time, without recomputing windows),
indels placed on and next to checkpoint rows, mismatch-only stretches, and
local alignments that start exactly on or just past a checkpoint row (where
a hop must stop at H = 0).  Every field against the oracle."""
import numpy as np
import pytest

import oracle
from genoaligner_gb300 import workloads
from helpers import assert_sw_equal, sw_gpu

pytestmark = pytest.mark.gpu

BASES = np.frombuffer(b"ACGT", np.uint8)


def rand(rng, n):
    return BASES[rng.integers(0, 4, n)].tobytes()


def flip(s, i):
    b = bytearray(s)
    b[i] = ord("C") if b[i] != ord("C") else ord("A")
    return bytes(b)


def crafted():
    rng = np.random.default_rng(2024)
    core = rand(rng, 3000)
    texts, pats = [], []
    texts.append(core); pats.append(core)                                  # identical: hops all the way
    t = core[:640] + core[641:]; texts.append(t); pats.append(core)       # a deletion on a checkpoint row
    t = core[:639] + b"G" + core[639:]; texts.append(t); pats.append(core)  # an insertion just before one
    t = core
    for k in range(100, 3000, 97):
        t = flip(t, k)
    texts.append(t); pats.append(core)                                     # mismatches only
    for start in (64, 65, 128, 129, 192):                                  # local start on / past a checkpoint row
        texts.append(rand(rng, start) + core[:1500]); pats.append(core[:1500])
    texts.append(rand(rng, 200) + core[:2000] + rand(rng, 300)); pats.append(core[:2000])
    t = core[:1000] + rand(rng, 64) + core[1064:]; texts.append(t); pats.append(core)   # a 64-base mismatch block
    return texts, pats


@pytest.mark.parametrize("scoring", [(2, -3, 3, 1), (1, -1, 2, 1), (2, -3, 5, 2)])
def test_walk_shortcuts_match_oracle(scoring):
    texts, pats = crafted()
    want = oracle.sw_batch(texts, pats, scoring=scoring, with_cigar=True)
    got = sw_gpu(texts, pats, scoring=scoring, with_cigar=True)
    assert_sw_equal(got, want, str(scoring))
