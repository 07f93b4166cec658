// Test harness (built by tests/test_fasta.py): reads each file named on the
// command line with genoaligner::io::read_fasta_file from the library and
// prints, per file, "ok|fail <error>" then one line per record appended:
// hex(id) hex(description) hex(sequence).
#include <genoaligner/io/fasta.hpp>

#include <cstdio>
#include <string>
#include <vector>

static void hex(const std::string& s)
{
    for (unsigned char c : s) std::printf("%02x", c);
    std::printf(" ");
}

int main(int argc, char** argv)
{
    for (int a = 1; a < argc; ++a) {
        std::vector<genoaligner::io::FastaRecord> recs;
        std::string err;
        const bool ok = genoaligner::io::read_fasta_file(argv[a], &recs, &err);
        std::printf("%s %s\n%zu\n", ok ? "ok" : "fail", err.c_str(), recs.size());
        for (const auto& r : recs) {
            hex(r.id);
            hex(r.description);
            hex(r.sequence);
            std::printf("\n");
        }
    }
    return 0;
}
