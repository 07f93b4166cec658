"""FASTA ingest without a GPU: the oracle against the reference reader's
fixtures, the library's reader (C ABI record set and the C++ reader API)
against the same fixtures, and the device-ready arena layout."""
import base64
import gzip
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from genoaligner_gb300 import _build, api
from oracle import fasta as ofasta

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _golden():
    with gzip.open(os.path.join(ROOT, "tests", "golden", "fasta_golden.json.gz"), "rt") as f:
        cases = json.load(f)["cases"]
    out = []
    for c in cases:
        recs = [tuple(base64.b64decode(x) for x in r) for r in c["records"]]
        out.append((base64.b64decode(c["input"]), c["ok"], c["error"], recs))
    return out


GOLDEN = _golden()


def test_oracle_matches_reference_reader():
    for data, ok, err, recs in GOLDEN:
        got = ofasta.records(data)
        assert got == (ok, err, recs), data


def test_reference_reader_cases_are_covered():
    oks = [g for g in GOLDEN if g[1]]
    fails = {g[2].split(" (")[0] for g in GOLDEN if not g[1]}
    assert len(oks) > 100
    assert fails >= {"expected '>' at start of a record, found 'A'", "record has a header but no sequence",
                     "no records found", "empty identifier in header"}


def _check_set(fs, recs):
    assert fs.n == len(recs)
    assert fs.ids == [r[0].decode("latin-1") for r in recs]
    assert fs.descriptions == [r[1].decode("latin-1") for r in recs]
    end = 0
    for i, r in enumerate(recs):
        assert fs.offsets[i] % 32 == 0 and fs.offsets[i] >= end
        assert fs.sequence(i) == r[2]
        end = int(fs.offsets[i]) + len(r[2])
        nxt = int(fs.offsets[i + 1]) if i + 1 < fs.n else fs.arena.nbytes - 64
        assert not fs.arena[end:nxt].any()                       # zero padding
    assert fs.arena.nbytes == (int(fs.offsets[-1]) + ((len(recs[-1][2]) + 31) // 32) * 32 + 64 if recs else 64)
    assert not fs.arena[-64:].any()


def test_record_set_matches_reference_reader():
    for data, ok, err, recs in GOLDEN:
        if ok:
            fs = api.fasta_parse(data)
            _check_set(fs, recs)
            fs.close()
        else:
            with pytest.raises(ValueError) as e:
                api.fasta_parse(data)
            assert str(e.value) == err, data


def test_record_set_from_file_and_missing_file(tmp_path):
    p = tmp_path / "x.fa"
    p.write_bytes(b">x\nACGT\n")
    fs = api.fasta_read(str(p))
    assert fs.ids == ["x"] and fs.sequence(0) == b"ACGT"
    missing = str(tmp_path / "definitely_not_here.fa")
    with pytest.raises(ValueError) as e:
        api.fasta_read(missing)
    assert str(e.value) == f"cannot open '{missing}'"


def test_large_multiline_file_matches_oracle(tmp_path):
    rng = np.random.default_rng(5)
    parts, want = [], []
    for r in range(3000):
        n = int(rng.integers(1, 900))
        seq = bytes(rng.choice(np.frombuffer(b"ACGTNacgt", np.uint8), size=n))
        end = [b"\n", b"\r\n"][r % 2]
        lines = [seq[k:k + 60] for k in range(0, n, 60)]
        parts.append(b">r%d desc %d" % (r, r) + end + end.join(lines) + end)
        want.append((b"r%d" % r, b"desc %d" % r, seq))
    data = b"".join(parts)
    p = tmp_path / "big.fa"
    p.write_bytes(data)
    fs = api.fasta_read(str(p))
    _check_set(fs, want)
    assert ofasta.records(data) == (True, "", want)


@pytest.fixture(scope="module")
def cxx_harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    lib = api.load()._name
    out = tmp_path_factory.mktemp("cxx") / "fasta_check"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "fasta_cxx_check.cpp"), "-o", str(out), lib,
                        "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


def test_cxx_reader_api_matches_reference_reader(cxx_harness, tmp_path):
    files = []
    for k, (data, ok, err, recs) in enumerate(GOLDEN):
        p = tmp_path / f"c{k}.fa"
        p.write_bytes(data)
        files.append(str(p))
    res = subprocess.run([cxx_harness, *files], capture_output=True, text=True, check=True).stdout.split("\n")
    at = 0
    for data, ok, err, recs in GOLDEN:
        head = res[at]
        assert head == ("ok " if ok else "fail " + err), (data, head)
        cnt = int(res[at + 1])
        got = [tuple(bytes.fromhex(x) for x in res[at + 2 + q].split(" ")[:3]) for q in range(cnt)]
        assert got == recs, data                           # also the records appended before a failure
        at += 2 + cnt
