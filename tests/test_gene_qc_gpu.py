"""The gene QC tool on the GPU (FASTA ingest -> one SW batch of records
against a bait -> CIGAR checks on the device) writes the same TSV, byte for
byte, as the reference's tools/gene_qc.cpp run on the reference's own SW
(fixtures from tests/golden/make_gene_qc_golden.py)."""
import base64
import gzip
import json
import os

import pytest

from genoaligner_gb300 import gene_qc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cases():
    with gzip.open(os.path.join(ROOT, "tests", "golden", "gene_qc_golden.json.gz"), "rt") as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_gene_qc_tsv_matches_reference_tool(case, tmp_path):
    sp, rp, out = tmp_path / "s.fa", tmp_path / "r.fa", tmp_path / "out.tsv"
    sp.write_bytes(base64.b64decode(case["seqs_fasta"]))
    rp.write_bytes(base64.b64decode(case["ref_fasta"]))
    rc = gene_qc.main([str(sp), "--ref", str(rp), "--emit", str(out), *case["args"]])
    assert rc == 0
    got = out.read_text().splitlines()
    want = case["tsv"].splitlines()
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g == w
