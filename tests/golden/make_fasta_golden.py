"""Writes tests/golden/fasta_golden.json.gz: inputs and the reference FASTA
reader's outputs on them, from oracle/_ref/libgaref_fasta.so (the reference's
include/genoaligner/io/fasta.hpp compiled by `make -C oracle ref`).

Inputs: the reader cases of the reference's tests/io/test_fasta.cpp (the same
texts), then seeded random inputs mixing headers, descriptions, blank and
blank-led lines, LF / CRLF / lone CR line ends, lowercase and non-ACGT bytes,
stray '>' and empty records.  Run from the repository root:

    make -C oracle ref && python tests/golden/make_fasta_golden.py
"""
import base64
import ctypes
import gzip
import json
import os
import random

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

CASES = [
    b">seq1 first record\nACGTACGTAC\nGTACGTACGT\nACGT\n>seq2 second\nTTTT\n",
    b">a\r\nACGT\r\nACGT\r\n>b\r\nTT\r\n",
    b"\n>only_id\n\nACGT\n\n\n>with_desc  some words here\nNNNN\n",
    b">masked\nacgtNNNRYSWacgt\n",
    b"ACGT\n",
    b">empty\n>next\nACGT\n",
    b"",
    b">   \nACGT\n",
    b">a\nAC\n>b\nTT\n>c\n",
    b">x\nACGT\n",
]


def random_input(rng: random.Random) -> bytes:
    ends = [b"\n", b"\r\n", b"\r"]
    out = bytearray()
    for _ in range(rng.randint(0, 6)):
        e = rng.choice(ends) if rng.random() < 0.3 else b"\n"
        kind = rng.random()
        if kind < 0.08:
            out += rng.choice([b"", b" ", b"\t", b"  x"]) + e                # blank or blank-led line
        elif kind < 0.12:
            out += rng.choice([b"ACGT", b"N"]) + e                           # sequence before any header
        head = b">" + rng.choice([b"", b" ", b"\t"]) if rng.random() < 0.07 else b">"
        rid = bytes(rng.choice(b"abcXYZ019_.|") for _ in range(rng.randint(0, 6)))
        desc = b""
        if rng.random() < 0.5:
            desc = rng.choice([b" ", b"\t", b"  ", b" \t"]) + bytes(rng.choice(b"ab c\td") for _ in range(rng.randint(0, 8)))
        trail = rng.choice([b"", b"", b" ", b"\t", b" \t "])
        out += head + rid + desc + trail + e
        for _ in range(rng.choice([0, 1, 1, 2, 3, 5])):
            if rng.random() < 0.15:
                out += rng.choice(ends)                                       # blank line inside
            seq = bytes(rng.choice(b"ACGTacgtNRY -") for _ in range(rng.randint(0, 12)))
            out += seq + rng.choice(ends)
    if rng.random() < 0.3 and out.endswith(b"\n"):
        out = out[:-1]                                                        # no final line end
    return bytes(out)


def main():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libgaref_fasta.so"))
    lib.ref_fasta_parse.argtypes = [ctypes.c_char_p, ctypes.c_long, ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.POINTER(ctypes.c_long)]
    lib.ref_fasta_free.argtypes = [ctypes.c_void_p]
    rng = random.Random(20240611)
    inputs = CASES + [random_input(rng) for _ in range(600)]
    out = []
    for data in inputs:
        p = ctypes.c_void_p()
        n = ctypes.c_long()
        assert lib.ref_fasta_parse(data, len(data), ctypes.byref(p), ctypes.byref(n)) == 0
        buf = ctypes.string_at(p, n.value)
        lib.ref_fasta_free(p)
        ok = buf[0] == 1
        e = buf.index(b"\0", 1)
        err = buf[1:e].decode()
        k = e + 1
        cnt = int.from_bytes(buf[k:k + 4], "little")
        k += 4
        recs = []
        for _ in range(cnt):
            a = buf.index(b"\0", k)
            rid = buf[k:a]
            b = buf.index(b"\0", a + 1)
            desc = buf[a + 1:b]
            sl = int.from_bytes(buf[b + 1:b + 9], "little")
            seq = buf[b + 9:b + 9 + sl]
            k = b + 9 + sl
            recs.append([base64.b64encode(x).decode() for x in (rid, desc, seq)])
        out.append({"input": base64.b64encode(data).decode(), "ok": ok, "error": err, "records": recs})
    path = os.path.join(ROOT, "tests", "golden", "fasta_golden.json.gz")
    with gzip.open(path, "wt") as f:
        json.dump({"source": "reference include/genoaligner/io/fasta.hpp via oracle/ref_fasta.cpp",
                   "cases": out}, f)
    print(path, len(out), "cases,", sum(c["ok"] for c in out), "well formed")


if __name__ == "__main__":
    main()
