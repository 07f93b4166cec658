"""FASTA reader oracle (test infrastructure only; never imported by the
product).

A plain-Python restatement of the reference's reader, genoaligner::io::
read_fasta (include/genoaligner/io/fasta.hpp:59-157), pinned against the
reference's own reader compiled here (oracle/ref_fasta.cpp) through the
fixtures in tests/golden/fasta_golden.json.gz.  Returns (ok, error, records)
with records a list of (id, description, sequence) byte strings: the records
the reader appended, also when it fails (the reference pushes a record when it
reads the header, :130, and reports the failure afterwards).
"""
from __future__ import annotations


def read_fasta(data: bytes):
    total = len(data)
    i = 0
    line = 1
    recs = []

    def fail(why, at):
        return False, f"{why} (line {at})", recs

    def eol(i, line):                      # fasta.hpp:86-99: \n, \r\n or a lone \r ends a line
        while i < total:
            c = data[i]
            if c == 0x0A:
                return i + 1, line + 1
            if c == 0x0D:
                i += 1
                if i < total and data[i] == 0x0A:
                    i += 1
                return i, line + 1
            i += 1
        return i, line

    in_record = False
    have_seq = False
    record_line = 0
    while i < total:
        c = data[i]
        if not in_record:                  # fasta.hpp:105-136
            if c in (0x0A, 0x0D, 0x20, 0x09):
                i, line = eol(i, line)     # a blank, CR, LF or tab line start: skip the line
                continue
            if c != 0x3E:
                return fail("expected '>' at start of a record, found '" + chr(c) + "'", line)
            i += 1
            j = i
            while j < total and data[j] not in (0x0A, 0x0D):
                j += 1
            header = data[i:j].rstrip(b" \t")  # trailing spaces and tabs only (:116-117)
            i = j
            sp = min([k for k in (header.find(b" "), header.find(b"\t")) if k >= 0], default=-1)
            if sp < 0:
                rid, desc = header, b""
            else:
                rid = header[:sp]
                rest = header[sp:].lstrip(b" \t")
                desc = rest
            if not rid:
                return fail("empty identifier in header", line)
            recs.append([rid, desc, bytearray()])
            in_record = True
            have_seq = False
            record_line = line
            i, line = eol(i, line)
            continue
        if c == 0x3E:                      # fasta.hpp:138-148
            if not have_seq:
                return fail("record has a header but no sequence", record_line)
            in_record = False
            continue
        if c in (0x0A, 0x0D):
            i, line = eol(i, line)
            continue
        j = i
        while j < total and data[j] not in (0x0A, 0x0D):
            j += 1
        recs[-1][2] += data[i:j]
        have_seq = True
        i = j
    if in_record and not have_seq:         # fasta.hpp:154-155
        return fail("record has a header but no sequence", record_line)
    if not recs:
        return fail("no records found", line)
    return True, "", recs


def records(data: bytes):
    """(ok, error, [(id, description, sequence)]) with immutable bytes."""
    ok, err, recs = read_fasta(data)
    return ok, err, [(bytes(a), bytes(b), bytes(c)) for a, b, c in recs]
