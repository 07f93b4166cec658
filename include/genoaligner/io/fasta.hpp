// genoaligner/io/fasta.hpp -- FASTA reading, drop-in for the reference's
// include/genoaligner/io/fasta.hpp (same names, record fields and rules).
//
// Rules kept from the reference (its tests/io/test_fasta.cpp pins them):
//   - FASTA only, no gzip; sequences are raw bytes, not validated as ACGT,
//     case preserved, line breaks removed;
//   - multi-line records are joined; \n, \r\n and a lone \r end a line; blank
//     lines between and inside records are skipped;
//   - the header's first space/tab-delimited token is the id, the rest (after
//     the separating blanks, trailing blanks removed) the description;
//   - an empty id, a record with no sequence, a byte other than '>' where a
//     record must start, and a file with no record are errors; a failed read
//     reports false and its reason (records already appended stay appended, as
//     in the reference: the caller discards them).
//
// Here the reader is compiled into libgenoaligner_gb300 (csrc/fasta.cpp), and
// the same parser also fills the pinned, device-ready arena of the C ABI's
// ga_fasta_* entries (include/genoaligner_gb300.h).
#ifndef GENOALIGNER_IO_FASTA_HPP
#define GENOALIGNER_IO_FASTA_HPP

#include <cstdio>
#include <string>
#include <vector>

namespace genoaligner {
namespace io {

struct FastaRecord {
    std::string id;           // first whitespace-delimited token of the header
    std::string description;  // the remainder of the header line (may be empty)
    std::string sequence;     // raw bytes, line breaks removed, case preserved
};

// Read every record from an open FILE* (to its end).  Returns false on a
// malformed file with the reason (and its line) in *error.
bool read_fasta(FILE* in, std::vector<FastaRecord>* out, std::string* error);

// Open a path and read it; false if it cannot be opened or is malformed.
bool read_fasta_file(const std::string& path, std::vector<FastaRecord>* out, std::string* error);

}  // namespace io
}  // namespace genoaligner

#endif  // GENOALIGNER_IO_FASTA_HPP
