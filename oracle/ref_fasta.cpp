// ref_fasta.cpp -- host build of the reference's FASTA reader.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile (target `ref`) with
// the reference's include/genoaligner/io/fasta.hpp, where it lies under
// REF_ROOT, into oracle/_ref/libgaref_fasta.so; nothing of the reference is
// copied here.  tests/golden/make_fasta_golden.py runs it on the reference's
// own reader cases (tests/io/test_fasta.cpp) and seeded inputs to write the
// FASTA fixtures; it is never part of the product.
#include "include/genoaligner/io/fasta.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

extern "C" {

// Parse `len` bytes with genoaligner::io::read_fasta (through a temporary
// FILE*, as the reference's tests do).  *out gets a malloc'd buffer: 1 byte ok
// flag, then the error string and NUL, then u32 record count and per record
// id NUL, description NUL, u64 sequence length, sequence bytes (records the
// reader appended, also on failure).  Returns 0, or -1 without a temp file.
int ref_fasta_parse(const char* data, long len, char** out, long* out_len)
{
    FILE* f = std::tmpfile();
    if (!f) return -1;
    if (len > 0) std::fwrite(data, 1, (size_t)len, f);
    std::rewind(f);
    std::vector<genoaligner::io::FastaRecord> recs;
    std::string err;
    const bool ok = genoaligner::io::read_fasta(f, &recs, &err);
    std::fclose(f);
    std::string buf;
    buf.push_back(ok ? 1 : 0);
    buf += err;
    buf.push_back('\0');
    const unsigned n = (unsigned)recs.size();
    buf.append(reinterpret_cast<const char*>(&n), 4);
    for (const auto& r : recs) {
        buf += r.id;
        buf.push_back('\0');
        buf += r.description;
        buf.push_back('\0');
        const unsigned long long sl = r.sequence.size();
        buf.append(reinterpret_cast<const char*>(&sl), 8);
        buf += r.sequence;
    }
    *out = static_cast<char*>(std::malloc(buf.size()));
    std::memcpy(*out, buf.data(), buf.size());
    *out_len = (long)buf.size();
    return 0;
}

void ref_fasta_free(char* p) { std::free(p); }

}  // extern "C"
