// noalloc.cu -- WFA over a device-resident batch without any device allocation.
//
// Some callers cannot call cudaMalloc at the moment they need an alignment:
// an application whose device memory is fully handed to its own pool
// allocator (a fresh cudaMalloc there fails or fragments the pool), or a
// latency-bound loop that cannot take cudaMalloc's implicit device-wide
// synchronisation.  ga_wfa_device_noalloc serves them: the caller passes the
// inputs and outputs, and every piece of scratch the WFA kernels need (the
// 2-bit sequence arena with its per-chunk masks, purity flags, the per-warp wavefront stacks, the work
// counter and error word) lives in one file-scope __device__ array of
// NOALLOC_SCRATCH_BYTES, which each GPU that loads this library holds until the
// process exits.  Batches whose scratch does not fit are refused.
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "../../include/genoaligner_gb300.h"
#include "kernels.cuh"

namespace ga {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)16 << 20;   // 16 MiB per GPU
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch.  In host code the array's name is a
// host-side stand-in, so only the address cudaGetSymbolAddress returns may be
// handed to a kernel.  The address belongs to the CUDA context the library's
// module is loaded in: it is looked up on the first call made in a context
// (with its device current) and kept with that context's unique id
// (cuCtxGetId, reached through cudaGetDriverEntryPointByVersion, so the
// library does not link the driver library).  A call in another context --
// after cudaDeviceReset, or with a context of the caller's own made current --
// looks it up again.  When the driver entry points cannot be had, every call
// looks the address up (cudaGetSymbolAddress allocates nothing).
constexpr int NOALLOC_MAX_DEVICES = 64;
struct ScratchAddr {
    unsigned char* addr = nullptr;
    unsigned long long ctx_id = 0;
};
static std::mutex g_noalloc_mu;
static ScratchAddr g_noalloc_addr[NOALLOC_MAX_DEVICES];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current context; false when there is
// none or the driver entry points are unavailable.
static bool current_ctx_id(unsigned long long* id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return false;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

static unsigned char* noalloc_scratch(int dev)
{
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return nullptr;
    unsigned long long id = 0;
    bool have_id = current_ctx_id(&id);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    ScratchAddr& s = g_noalloc_addr[dev];
    if (s.addr && have_id && s.ctx_id == id) return s.addr;
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return nullptr;
    }
    // the lookup makes the device's primary context current if none was
    if (!have_id) have_id = current_ctx_id(&id);
    s.addr = have_id ? static_cast<unsigned char*>(p) : nullptr;
    s.ctx_id = id;
    return static_cast<unsigned char*>(p);
}

static inline size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace ga

using namespace ga;

extern "C" int32_t ga_wfa_device_noalloc(const ga_device_batch* b, int32_t smax, int32_t trace,
                                         int32_t* out_score, int32_t* out_len, char* out_cigar, void* stream,
                                         const char** err)
{
    if (!b || b->n < 0 || b->seq_bytes < 0 ||
        (b->n > 0 && (!b->seq || !b->a_off || !b->a_len || !b->b_off || !b->b_len || !out_score ||
                      (trace && (!out_len || !out_cigar || !b->out_off))))) {
        if (err) *err = "invalid device batch";
        return GA_INVALID_ARGUMENT;
    }
    if (smax < 0 || smax > GA_MAX_SMAX_DEVICE) {
        if (err) *err = "smax out of range [0, GA_MAX_SMAX_DEVICE]";
        return GA_INVALID_ARGUMENT;
    }
    if (((uintptr_t)b->seq & 15) != 0) {
        if (err) *err = "device batch arena must be 16-byte aligned";
        return GA_INVALID_ARGUMENT;
    }
    if (b->n == 0) return GA_OK;

    // scratch layout: [counter, error word | purity flags | 2-bit arena | wavefront stacks]
    const size_t head = 256;
    const size_t pure_bytes = round256(2 * (size_t)b->n);
    const size_t packed_bytes = round256((size_t)packed_arena_words(b->seq_bytes) * sizeof(uint64_t));
    const size_t fixed = head + pure_bytes + packed_bytes;
    const size_t slot_bytes = (size_t)((int64_t)smax + 1) * (size_t)((int64_t)smax + 1) * sizeof(int32_t);
    if (fixed + (trace ? 4 * slot_bytes : 0) > NOALLOC_SCRATCH_BYTES) {
        if (err) *err = "batch needs more than the 16 MiB no-allocation scratch: split it or use ga_wfa_device";
        return GA_INVALID_ARGUMENT;
    }

    int dev = -1, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "no CUDA device is available";
        return GA_DEVICE_ERROR;
    }
    unsigned char* base = noalloc_scratch(dev);
    if (!base) {
        if (err) *err = "cannot resolve the no-allocation scratch on this device";
        return GA_DEVICE_ERROR;
    }
    int32_t* ctr = reinterpret_cast<int32_t*>(base);
    uint8_t* pure = base + head;
    uint64_t* packed = reinterpret_cast<uint64_t*>(base + head + pure_bytes);
    int32_t* stk = trace ? reinterpret_cast<int32_t*>(base + fixed) : nullptr;

    int slots = (int)std::min<int64_t>(wfa_max_slots(smax, trace != 0, sms), ((int64_t)b->n + 3) / 4 * 4);
    if (trace) {
        const int64_t fit = (int64_t)((NOALLOC_SCRATCH_BYTES - fixed) / slot_bytes) / 4 * 4;
        slots = (int)std::min<int64_t>(slots, fit);
    }
    // pairs per counter increment, as the allocating entry takes them
    const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(16, (int64_t)b->n / ((int64_t)slots * 8)));
    cudaStream_t st = (cudaStream_t)stream;
    // the counter and error word keep the previous call's values: clear them
    if (cudaMemsetAsync(ctr, 0, head, st) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "device memset failed";
        return GA_DEVICE_ERROR;
    }
    PairDesc D;
    D.seq = b->seq; D.packed = packed; D.pure = pure;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len;
    D.out_off = b->out_off; D.n = b->n;
    WfaArgs A;
    A.D = D; A.smax = smax; A.trace = trace ? 1 : 0;
    A.out_score = out_score; A.out_len = out_len; A.out_cigar = out_cigar;
    A.stack = stk; A.stack_slot = ((int64_t)smax + 1) * ((int64_t)smax + 1);
    A.counter = ctr; A.err = ctr + 1;
    A.chunk = chunk;
    if (launch_pack(D, b->seq_bytes, packed, pure, st) != cudaSuccess || launch_wfa(A, slots, st) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "kernel launch failed";
        return GA_DEVICE_ERROR;
    }
    if (!stream && cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "device execution failed";
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}
