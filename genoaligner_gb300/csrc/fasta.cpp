// fasta.cpp -- FASTA ingest: the reference's reader API (genoaligner::io,
// include/genoaligner/io/fasta.hpp of the reference) and the C ABI's
// device-ready record set (ga_fasta_*).
//
// One parser serves both.  It scans the input once, keeping for each record
// its header fields and the spans of its sequence lines (the reader rules of
// the reference's read_fasta, include/genoaligner/io/fasta.hpp:61-151: line
// ends \n, \r\n or a lone \r; between records a line starting with a blank or
// a tab is skipped whole; the id is the header's first space/tab token, the
// description the rest after the separating blanks, trailing blanks removed;
// an empty id, a record without sequence, a byte other than '>' where a record
// starts, and an input without records are errors, with the reference's
// messages and line numbers).  The record set then copies those spans, in
// parallel, into one arena in the layout the device entries take: every
// sequence at a 32-byte-aligned offset, zero padding, 64 spare bytes.  The
// arena is pinned host memory when a CUDA device is present, so a single
// cudaMemcpyAsync moves it to the device at full bus speed.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/genoaligner/io/fasta.hpp"
#include "engine.hpp"

namespace ga {

struct FaSpan { int64_t src, dst, len; };          // one sequence line: input offset, offset in the record, bytes

struct FaParse {
    std::vector<std::string> id, desc;
    std::vector<int64_t> seq_len;                  // per record
    std::vector<int64_t> first_span;               // per record, into spans (+ one end entry)
    std::vector<FaSpan> spans;
    std::string error;                             // empty when the input is well formed
};

// The scan.  On an error the records met so far stay in P (the reference
// appends a record when its header is read, before it knows the record is
// complete), and P.error holds the reason.
static void fa_scan(const char* data, int64_t total, FaParse& P)
{
    int64_t i = 0;
    long line = 1;
    auto fail = [&](const std::string& why, long at) { P.error = why + " (line " + std::to_string(at) + ")"; };
    auto eol = [&]() {                             // past the end of the current line
        while (i < total) {
            const char c = data[i];
            if (c == '\n') { ++i; ++line; return; }
            if (c == '\r') {
                ++i;
                if (i < total && data[i] == '\n') ++i;
                ++line;
                return;
            }
            ++i;
        }
    };
    auto line_end = [&](int64_t from) -> int64_t {   // first \n or \r at or after from
        const void* nl = std::memchr(data + from, '\n', (size_t)(total - from));
        const int64_t k = nl ? (int64_t)((const char*)nl - data) : total;
        const void* cr = std::memchr(data + from, '\r', (size_t)(k - from));
        return cr ? (int64_t)((const char*)cr - data) : k;
    };
    bool in_record = false, have_seq = false;
    long record_line = 0;
    while (i < total) {
        const char c = data[i];
        if (!in_record) {
            if (c == '\n' || c == '\r' || c == ' ' || c == '\t') { eol(); continue; }
            if (c != '>') {
                fail(std::string("expected '>' at start of a record, found '") + c + "'", line);
                break;
            }
            ++i;
            const int64_t e = line_end(i);
            int64_t h1 = e;
            while (h1 > i && (data[h1 - 1] == ' ' || data[h1 - 1] == '\t')) --h1;
            int64_t sp = i;
            while (sp < h1 && data[sp] != ' ' && data[sp] != '\t') ++sp;
            if (sp == i) {
                fail("empty identifier in header", line);
                break;
            }
            int64_t ds = sp;
            while (ds < h1 && (data[ds] == ' ' || data[ds] == '\t')) ++ds;
            P.id.emplace_back(data + i, (size_t)(sp - i));
            P.desc.emplace_back(data + ds, (size_t)(h1 - ds));
            P.seq_len.push_back(0);
            P.first_span.push_back((int64_t)P.spans.size());
            in_record = true;
            have_seq = false;
            record_line = line;
            i = e;
            eol();
            continue;
        }
        if (c == '>') {
            if (!have_seq) {
                fail("record has a header but no sequence", record_line);
                break;
            }
            in_record = false;
            continue;
        }
        if (c == '\n' || c == '\r') { eol(); continue; }
        const int64_t e = line_end(i);
        P.spans.push_back(FaSpan{i, P.seq_len.back(), e - i});
        P.seq_len.back() += e - i;
        have_seq = true;
        i = e;
    }
    if (P.error.empty()) {
        if (in_record && !have_seq) fail("record has a header but no sequence", record_line);
        else if (P.id.empty()) fail("no records found", line);
    }
    P.first_span.push_back((int64_t)P.spans.size());
}

static bool read_all(FILE* in, std::string& data)
{
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), in)) > 0) data.append(buf, n);
    return !std::ferror(in);
}

static bool read_path(const char* path, std::string& data, std::string& err)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        err = std::string("cannot open '") + path + "'";
        return false;
    }
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long sz = std::ftell(f);
        if (sz > 0) data.reserve((size_t)sz);
        std::rewind(f);
    }
    const bool ok = read_all(f, data);
    std::fclose(f);
    if (!ok) err = "read error (line 0)";
    return ok;
}

}  // namespace ga

// ------------------------------------------------ the reference's reader --
namespace genoaligner {
namespace io {

static bool to_records(const char* data, int64_t total, std::vector<FastaRecord>* out, std::string* error)
{
    ga::FaParse P;
    ga::fa_scan(data, total, P);
    const size_t base = out->size();
    out->resize(base + P.id.size());
    for (size_t r = 0; r < P.id.size(); ++r) {
        FastaRecord& rec = (*out)[base + r];
        rec.id = std::move(P.id[r]);
        rec.description = std::move(P.desc[r]);
        rec.sequence.resize((size_t)P.seq_len[r]);
        for (int64_t s = P.first_span[r]; s < P.first_span[r + 1]; ++s)
            std::memcpy(&rec.sequence[(size_t)P.spans[s].dst], data + P.spans[s].src, (size_t)P.spans[s].len);
    }
    if (!P.error.empty()) {
        if (error) *error = P.error;
        return false;
    }
    return true;
}

bool read_fasta(FILE* in, std::vector<FastaRecord>* out, std::string* error)
{
    if (!in) { if (error) *error = "null FILE*"; return false; }
    if (!out) { if (error) *error = "null output vector"; return false; }
    std::string data;
    if (!ga::read_all(in, data)) { if (error) *error = "read error (line 0)"; return false; }
    return to_records(data.data(), (int64_t)data.size(), out, error);
}

bool read_fasta_file(const std::string& path, std::vector<FastaRecord>* out, std::string* error)
{
    std::string data, err;
    if (!ga::read_path(path.c_str(), data, err)) { if (error) *error = err; return false; }
    if (!out) { if (error) *error = "null output vector"; return false; }
    return to_records(data.data(), (int64_t)data.size(), out, error);
}

}  // namespace io
}  // namespace genoaligner

// ------------------------------------------------------ the C ABI's set --
struct ga_fasta {
    uint8_t* arena = nullptr;
    int64_t arena_bytes = 0;
    bool pinned = false;
    std::vector<int64_t> off;
    std::vector<int32_t> len;
    std::vector<std::string> id, desc;
    ~ga_fasta()
    {
        if (!arena) return;
        if (pinned) cudaFreeHost(arena);
        else std::free(arena);
    }
};

namespace ga {

static thread_local std::string t_fa_err;

static const char* fa_fail(const std::string& why, const char** err)
{
    t_fa_err = why;
    if (err) *err = t_fa_err.c_str();
    return t_fa_err.c_str();
}

static int32_t fa_build(const char* data, int64_t total, ga_fasta** out, const char** err)
{
    FaParse P;
    fa_scan(data, total, P);
    if (!P.error.empty()) {
        fa_fail(P.error, err);
        return GA_INVALID_ARGUMENT;
    }
    const int64_t n = (int64_t)P.id.size();
    if (n > INT32_MAX) {
        fa_fail("more than 2^31-1 records", err);
        return GA_INVALID_ARGUMENT;
    }
    std::unique_ptr<ga_fasta> F(new ga_fasta());
    F->off.resize(n);
    F->len.resize(n);
    int64_t at = 0;
    for (int64_t r = 0; r < n; ++r) {
        if (P.seq_len[r] > INT32_MAX) {
            fa_fail("record " + P.id[r] + " is longer than 2^31-1 bytes", err);
            return GA_INVALID_ARGUMENT;
        }
        F->off[r] = at;
        F->len[r] = (int32_t)P.seq_len[r];
        at += (P.seq_len[r] + 31) & ~(int64_t)31;
    }
    F->arena_bytes = at + 64;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) == cudaSuccess && dev > 0 &&
        cudaHostAlloc(reinterpret_cast<void**>(&F->arena), (size_t)F->arena_bytes, cudaHostAllocDefault) == cudaSuccess) {
        F->pinned = true;
    } else {
        cudaGetLastError();
        F->arena = static_cast<uint8_t*>(std::aligned_alloc(64, (size_t)((F->arena_bytes + 63) & ~(int64_t)63)));
    }
    if (!F->arena) {
        fa_fail("host allocation failed", err);
        return GA_DEVICE_ERROR;
    }
    // padding first (tails of the records and the spare bytes), then the lines
    uint8_t* A = F->arena;
    parallel_for(n, 4096, [&](int64_t lo, int64_t hi) {
        for (int64_t r = lo; r < hi; ++r) {
            const int64_t end = r + 1 < n ? F->off[r + 1] : at;
            std::memset(A + F->off[r] + F->len[r], 0, (size_t)(end - F->off[r] - F->len[r]));
        }
    });
    std::memset(A + at, 0, 64);
    std::vector<int64_t> span_rec(P.spans.size());
    for (int64_t r = 0; r < n; ++r)
        for (int64_t s = P.first_span[r]; s < P.first_span[r + 1]; ++s) span_rec[s] = r;
    parallel_for((int64_t)P.spans.size(), 1024, [&](int64_t lo, int64_t hi) {
        for (int64_t s = lo; s < hi; ++s) {
            const FaSpan& sp = P.spans[s];
            std::memcpy(A + F->off[span_rec[s]] + sp.dst, data + sp.src, (size_t)sp.len);
        }
    });
    F->id = std::move(P.id);
    F->desc = std::move(P.desc);
    *out = F.release();
    return GA_OK;
}

}  // namespace ga

using namespace ga;

extern "C" {

int32_t ga_fasta_parse(const char* data, int64_t bytes, ga_fasta** out, const char** err)
{
    if (!out || (bytes > 0 && !data) || bytes < 0) {
        fa_fail("invalid arguments", err);
        return GA_INVALID_ARGUMENT;
    }
    *out = nullptr;
    return fa_build(data, bytes, out, err);
}

int32_t ga_fasta_read(const char* path, ga_fasta** out, const char** err)
{
    if (!out || !path) {
        fa_fail("invalid arguments", err);
        return GA_INVALID_ARGUMENT;
    }
    *out = nullptr;
    std::string data, e;
    if (!read_path(path, data, e)) {
        fa_fail(e, err);
        return GA_INVALID_ARGUMENT;
    }
    return fa_build(data.data(), (int64_t)data.size(), out, err);
}

int32_t ga_fasta_count(const ga_fasta* f) { return f ? (int32_t)f->len.size() : 0; }

const char* ga_fasta_id(const ga_fasta* f, int32_t i)
{
    return (f && i >= 0 && i < (int32_t)f->id.size()) ? f->id[i].c_str() : nullptr;
}

const char* ga_fasta_description(const ga_fasta* f, int32_t i)
{
    return (f && i >= 0 && i < (int32_t)f->desc.size()) ? f->desc[i].c_str() : nullptr;
}

const uint8_t* ga_fasta_arena(const ga_fasta* f, int64_t* bytes)
{
    if (bytes) *bytes = f ? f->arena_bytes : 0;
    return f ? f->arena : nullptr;
}

const int64_t* ga_fasta_offsets(const ga_fasta* f) { return f ? f->off.data() : nullptr; }
const int32_t* ga_fasta_lengths(const ga_fasta* f) { return f ? f->len.data() : nullptr; }
int32_t ga_fasta_pinned(const ga_fasta* f) { return f && f->pinned ? 1 : 0; }

int32_t ga_fasta_upload(const ga_fasta* f, void* device_arena, void* stream)
{
    if (!f || !device_arena) return GA_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(device_arena, f->arena, (size_t)f->arena_bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

void ga_fasta_free(ga_fasta* f) { delete f; }

}  // extern "C"
