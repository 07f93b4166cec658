"""Writes tests/golden/gene_qc_golden.json.gz: seeded gene-family FASTA inputs
(genoaligner_gb300.workloads.gene_family) and the TSV the reference's own gene
QC tool writes for them -- oracle/_ref/gene_qc_ref, the reference's
tools/gene_qc.cpp built unchanged on its CPU-shim API by `make -C oracle ref`.
Run from the repository root:

    make -C oracle ref && python tests/golden/make_gene_qc_golden.py
"""
import base64
import gzip
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from genoaligner_gb300 import workloads  # noqa: E402

# (name, records, codons, seed, CRLF files, extra tool arguments)
CASES = [
    ("family_code1", 180, 300, 6, False, []),
    ("family_code2_crlf", 90, 200, 7, True, ["--code", "2", "--min-cov", "0.6", "--min-score", "20"]),
    ("family_scoring", 72, 250, 8, False, ["--scoring", "2,-3,5,2"]),
]


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "gene_qc_ref")
    out = []
    with tempfile.TemporaryDirectory() as d:
        for name, n, codons, seed, crlf, extra in CASES:
            recs, baits = workloads.gene_family(n, codons, seed)
            sp, rp, tp = (os.path.join(d, f"{name}.{x}") for x in ("fa", "ref.fa", "tsv"))
            workloads.write_fasta(sp, recs, crlf=crlf)
            workloads.write_fasta(rp, baits, crlf=crlf)
            r = subprocess.run([exe, sp, "--ref", rp, "--emit", tp, *extra], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
            out.append({"name": name, "records": n, "codons": codons, "seed": seed, "crlf": crlf, "args": extra,
                        "seqs_fasta": base64.b64encode(open(sp, "rb").read()).decode(),
                        "ref_fasta": base64.b64encode(open(rp, "rb").read()).decode(),
                        "tsv": open(tp).read(), "stdout": r.stdout, "stderr": r.stderr})
            print(name, r.stderr.strip().splitlines()[-1])
    path = os.path.join(ROOT, "tests", "golden", "gene_qc_golden.json.gz")
    with gzip.open(path, "wt") as f:
        json.dump({"source": "reference tools/gene_qc.cpp via oracle/ref_gene_qc.cpp (CPU shim)", "cases": out}, f)
    print(path)


if __name__ == "__main__":
    main()
