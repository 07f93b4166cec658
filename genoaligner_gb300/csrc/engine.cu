// engine.cu -- host engine and C ABI of the GB300 pairwise aligner.
//
// Per call: validate the requests exactly as the reference's API does
// (src/api/api.cpp:246-266, 600-616, 515-536), lay the sequences out in a
// pinned staging arena at 32-byte-aligned offsets (the layout the kernels
// take), copy once to the device, run the kernels on the call's own stream,
// copy the outputs back once, and materialise results on the host thread pool.
// Contexts (stream + grow-only device and pinned arenas) are pooled, so a
// steady stream of calls allocates nothing; concurrent calls take different
// contexts.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "engine.hpp"
#include "kernels.cuh"
#include "tune.hpp"

namespace ga {

// ------------------------------------------------------------ accounting --
static std::atomic<long long> g_launches{0};
static thread_local long long t_launches = 0;     // the calling thread's share of g_launches

// Per-kernel event timing, on only between ga_profile(1) and ga_profile(0).
struct ProfRec { int id; cudaEvent_t a, b; };
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<ProfRec> g_prof_open;      // begin recorded, end pending
static std::vector<ProfRec> g_prof_done;
static double g_prof_ms[K_COUNT];
static long long g_prof_n[K_COUNT];
thread_local ProfRec t_prof_cur{-1, nullptr, nullptr};

void launch_begin(int kernel_id, cudaStream_t st)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ++t_launches;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (!g_prof_on) return;
    ProfRec r{kernel_id, nullptr, nullptr};
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, st);
    t_prof_cur = r;
}

static bool profiling_on()
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    return g_prof_on;
}

// Launches replayed through a CUDA graph count like direct ones.
static void note_graph_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void launch_end(int kernel_id, cudaStream_t st)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (!g_prof_on || t_prof_cur.id != kernel_id) return;
    cudaEventRecord(t_prof_cur.b, st);
    g_prof_done.push_back(t_prof_cur);
    t_prof_cur = ProfRec{-1, nullptr, nullptr};
}

int device_sms()
{
    constexpr int MAX_DEV = 64;
    static std::atomic<int> cache[MAX_DEV];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev < MAX_DEV) {
        if (const int v = cache[dev].load(std::memory_order_relaxed)) return v;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
        cudaGetLastError();
        return 1;
    }
    if (dev < MAX_DEV) cache[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

int blocks_per_sm(const void* func, int threads, size_t smem)
{
    static std::mutex mu;
    static std::map<std::tuple<int, const void*, int, size_t>, int> cache;
    static std::map<std::pair<int, const void*>, size_t> limit;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return 1; }
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, func, threads, smem);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    if (smem > 0) {
        // (the opt-in limit counts dynamic memory only, but a launch needs it
        // whenever dynamic plus static memory pass 48 KB: raise it always)
        size_t& lim = limit[std::make_pair(dev, func)];
        if (smem > lim && cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                              cudaSuccess)
            lim = smem;
        cudaGetLastError();
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 0;
    }
    per_sm = std::max(per_sm, 1);
    cache[key] = per_sm;
    return per_sm;
}

// Host-to-device / device-to-host bytes of the calling thread's last batch call.
thread_local int64_t t_h2d = 0, t_d2h = 0;

static std::atomic<int> g_fail_next{0};

// ----------------------------------------------------------- thread pool --
// One job at a time: the calling thread and every worker that wakes while the
// job is open take chunks of `grain` from a shared counter.  The job closes
// when the caller runs out of chunks; the caller then waits only for the
// workers that joined it (a worker that wakes after the close skips the job).
// A worker that finishes a job watches for the next one for SPIN_US before it
// sleeps: a call's host passes come tens of microseconds apart, and waking
// sleeping threads costs about as much as a small pass itself.  While a call
// runs its ranges on threads of their own (quiet() > 0) the workers sleep at
// once instead, leaving the cores to those threads.
class Pool {
public:
    static constexpr int SPIN_US = 200;
    std::atomic<int>& quiet() { return quiet_; }
    Pool()
    {
        unsigned hc = std::thread::hardware_concurrency();
        int nw = (int)(hc == 0 ? 1 : hc) - 1;
        if (nw > 63) nw = 63;
        for (int i = 0; i < nw; ++i) threads_.emplace_back([this] { worker(); });
    }
    ~Pool()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_.store(true);
            gen_.fetch_add(1);
        }
        cv_.notify_all();
        for (auto& t : threads_) t.join();
    }
    void run(int64_t n, int64_t grain, const std::function<void(int64_t, int64_t)>& fn)
    {
        if (n <= 0) return;
        if (grain < 1) grain = 1;
        if (threads_.empty() || n <= grain) { fn(0, n); return; }
        std::lock_guard<std::mutex> one(job_mu_);          // one parallel job at a time
        bool wake;
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &fn;
            n_ = n;
            grain_ = grain;
            next_.store(0);
            open_ = true;
            joined_ = 0;
            gen_.fetch_add(1);
            wake = sleeping_ > 0;
        }
        if (wake) cv_.notify_all();
        drain();
        std::unique_lock<std::mutex> lk(mu_);
        open_ = false;                                      // every chunk is taken
        done_cv_.wait(lk, [&] { return joined_ == 0; });    // and the joined workers' chunks are done
        fn_ = nullptr;
    }

private:
    void drain()
    {
        for (;;) {
            const int64_t lo = next_.fetch_add(grain_);
            if (lo >= n_) break;
            (*fn_)(lo, std::min(n_, lo + grain_));
        }
    }
    void worker()
    {
        uint64_t seen = 0;
        for (;;) {
            // watch for a new job for a while, then sleep until one comes
            const auto t0 = std::chrono::steady_clock::now();
            for (int it = 0; gen_.load() == seen && quiet_.load() == 0; ++it) {
                if ((it & 63) == 63 &&
                    std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(SPIN_US))
                    break;
                std::this_thread::yield();
            }
            {
                std::unique_lock<std::mutex> lk(mu_);
                if (gen_.load() == seen) {
                    ++sleeping_;
                    cv_.wait(lk, [&] { return gen_.load() != seen; });
                    --sleeping_;
                }
                if (stop_.load()) return;
                seen = gen_.load();
                if (!open_) continue;                       // woke after the job closed
                ++joined_;
            }
            drain();
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (--joined_ == 0) done_cv_.notify_all();
            }
        }
    }
    std::vector<std::thread> threads_;
    std::mutex mu_, job_mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int64_t, int64_t)>* fn_ = nullptr;
    int64_t n_ = 0, grain_ = 1;
    std::atomic<int64_t> next_{0};
    std::atomic<uint64_t> gen_{0};
    std::atomic<bool> stop_{false};
    std::atomic<int> quiet_{0};
    int joined_ = 0, sleeping_ = 0;
    bool open_ = false;
};

static Pool& pool()
{
    static Pool* p = new Pool();   // never destroyed: worker threads outlive static teardown safely
    return *p;
}

void parallel_for(int64_t n, int64_t grain, const std::function<void(int64_t, int64_t)>& fn)
{
    pool().run(n, grain, fn);
}

// Held while a call runs its ranges on threads of its own: the pool's idle
// workers sleep instead of watching for the next job.
struct PoolQuiet {
    PoolQuiet() { pool().quiet().fetch_add(1); }
    ~PoolQuiet() { pool().quiet().fetch_sub(1); }
};

void expand_cigar(const uint8_t* src, int len, char* dst)
{
    // four ops per packed byte: one 4-byte store per byte from a 256-entry table
    static const auto table = [] {
        std::vector<uint32_t> t(256);
        const char ops[4] = {'M', 'X', 'I', 'D'};
        for (int b = 0; b < 256; ++b) {
            unsigned char c[4];
            for (int k = 0; k < 4; ++k) c[k] = (unsigned char)ops[(b >> (2 * k)) & 3];
            std::memcpy(&t[(size_t)b], c, 4);
        }
        return t;
    }();
    int t = 0;
    for (; t + 4 <= len; t += 4) std::memcpy(dst + t, &table[src[t >> 2]], 4);
    if (t < len) {
        const uint32_t w = table[src[t >> 2]];
        std::memcpy(dst + t, &w, (size_t)(len - t));
    }
}

// -------------------------------------------------------------- contexts --
struct Ctx {
    int device = -1;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;     // last work enqueued on a caller's stream
    bool pending = false;
    char* dev = nullptr;
    size_t dev_cap = 0;
    uint64_t dev_gen = 0;           // bumped whenever the device arena is reallocated
    cudaGraphExec_t gexec = nullptr;  // the learned WFA path, captured once per launch shape
    std::vector<uint64_t> gkey;
    int glaunches = 0;                // library kernels in gexec
    cudaGraphExec_t swexec = nullptr; // the SW device work of a call or range, captured once per launch shape
    std::vector<uint64_t> swkey;
    int swlaunches = 0;               // library kernels in swexec
    char* host = nullptr;
    size_t host_cap = 0;
    int tag = -1;                   // range index of a ranged SW call that created it, else -1
    int prio = 0;                   // the stream's priority
};

// Stream priority of range `tag` of a ranged call: range 0 the greatest, each
// later range one step lower (as far as the device's range goes), so the
// earlier ranges' blocks are scheduled first and those ranges finish first --
// their results copy back and are written out while the later ranges run.
// Other calls: the default priority.
static int ctx_priority(int tag)
{
    if (tag < 0) return 0;
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return std::min(least, greatest + tag);
}

static std::mutex g_ctx_mu;
static std::vector<Ctx*> g_ctx_free;

static const char* E_NODEV = "no CUDA device is available";

// A free context of the current device: the one tagged `tag` if free (range
// k of a ranged SW call takes the context range k had before, whose arena is
// already sized for such a range; growing an arena frees the old one, which
// waits for the whole device), else the most recently released one (a caller
// on one thread keeps reusing one warm arena), else a new one.
static Ctx* acquire_ctx(const char** err, int tag = -1)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        *err = E_NODEV;
        return nullptr;
    }
    {
        std::lock_guard<std::mutex> lk(g_ctx_mu);
        long pick = -1;
        for (size_t i = g_ctx_free.size(); i-- > 0;) {
            if (g_ctx_free[i]->device != dev) continue;
            if (g_ctx_free[i]->tag == tag) { pick = (long)i; break; }
            if (pick < 0 && (tag < 0 || g_ctx_free[i]->tag < 0)) pick = (long)i;
        }
        if (pick >= 0) {
            Ctx* c = g_ctx_free[(size_t)pick];
            g_ctx_free.erase(g_ctx_free.begin() + pick);
            if (tag >= 0) c->tag = tag;
            if (c->pending) { cudaEventSynchronize(c->done); c->pending = false; }
            // a range's context needs its range's priority (a call alone runs at any)
            const int prio = tag >= 0 ? ctx_priority(tag) : c->prio;
            if (prio != c->prio) {                     // the stream of another priority: a new one
                cudaStream_t ns = nullptr;
                if (cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio) == cudaSuccess) {
                    cudaStreamSynchronize(c->stream);
                    cudaStreamDestroy(c->stream);
                    c->stream = ns;
                    c->prio = prio;
                } else {
                    cudaGetLastError();
                }
            }
            return c;
        }
    }
    Ctx* c = new Ctx();
    c->device = dev;
    c->tag = tag;
    c->prio = ctx_priority(tag);
    if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, c->prio) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        *err = E_NODEV;
        return nullptr;
    }
    return c;
}

static void release_ctx(Ctx* c)
{
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    g_ctx_free.push_back(c);
}

// Device bytes the idle contexts of `dev` hold in their arenas.
static size_t idle_dev_bytes(int dev)
{
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    size_t s = 0;
    for (Ctx* c : g_ctx_free)
        if (c->device == dev) s += c->dev_cap;
    return s;
}

// Free idle contexts' arenas on `dev` (least recently used first) until
// `need` bytes are free on the device or none is left.
static void trim_idle(int dev, size_t need)
{
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    for (Ctx* c : g_ctx_free) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); fr = 0; }
        if (fr >= need) return;
        if (c->device != dev || !c->dev) continue;
        if (c->pending) { cudaEventSynchronize(c->done); c->pending = false; }
        cudaStreamSynchronize(c->stream);
        cudaFree(c->dev);
        c->dev = nullptr;
        c->dev_cap = 0;
        ++c->dev_gen;
    }
}

static bool ensure_dev(Ctx* c, size_t bytes)
{
    if (bytes <= c->dev_cap) return true;
    if (c->dev) { cudaStreamSynchronize(c->stream); cudaFree(c->dev); c->dev = nullptr; c->dev_cap = 0; }
    size_t want = std::max(bytes, (size_t)(c->dev_cap * 3 / 2));
    want = (want + ((size_t)1 << 20) - 1) & ~(((size_t)1 << 20) - 1);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); fr = 0; }
    const size_t margin = (size_t)256 << 20;
    if (fr < want + margin) trim_idle(c->device, want + margin);   // idle contexts' arenas give way
    if (cudaMalloc(&c->dev, want) != cudaSuccess) {
        cudaGetLastError();
        trim_idle(c->device, (size_t)-1);
        if (cudaMalloc(&c->dev, bytes) != cudaSuccess) { cudaGetLastError(); c->dev = nullptr; return false; }
        want = bytes;
    }
    c->dev_cap = want;
    ++c->dev_gen;
    return true;
}

static bool ensure_host(Ctx* c, size_t bytes)
{
    if (bytes <= c->host_cap) return true;
    if (c->host) { cudaStreamSynchronize(c->stream); cudaFreeHost(c->host); c->host = nullptr; c->host_cap = 0; }
    size_t want = std::max(bytes, (size_t)(c->host_cap * 3 / 2));
    want = (want + ((size_t)1 << 20) - 1) & ~(((size_t)1 << 20) - 1);
    if (cudaHostAlloc(&c->host, want, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        c->host = nullptr;
        return false;
    }
    c->host_cap = want;
    return true;
}

// Carves aligned sub-buffers out of one arena; a first pass with base null
// only measures.
struct Carve {
    char* base;
    size_t off = 0;
    explicit Carve(char* b) : base(b) {}
    template <class T>
    T* take(size_t count, size_t align = 256)
    {
        off = (off + align - 1) & ~(align - 1);
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

static inline int64_t round32(int64_t x) { return (x + 31) & ~(int64_t)31; }

// Requests per chunk of the host passes over a batch's requests.
constexpr int64_t REQ_CHUNK = 1024;
// The WFA entry's chunk: smaller for small batches, whose passes would
// otherwise be a few chunks, each a whole thread's serial work.
static inline int64_t wfa_chunk(int64_t n) { return n < 65536 ? 256 : REQ_CHUNK; }

// Where a batch's own sides of one kind (patterns, or texts) lie in the
// caller's memory, in request order: [first, end) when every side starts at
// or after the previous one's end and less than 4,096 bytes past it -- so
// every page of the span holds part of a side, and the span can be read as
// one block.
struct SideSpan {
    uintptr_t first = 0, end = 0;
    int64_t bytes = 0;
    bool ok = true;
    void add(const void* p, int32_t len)
    {
        if (len <= 0) return;
        const uintptr_t a = (uintptr_t)p;
        if (bytes == 0) first = a;
        else if (a < end || a - end >= 4096) ok = false;
        end = a + (uintptr_t)len;
        bytes += len;
    }
    void join(const SideSpan& o)                 // this span followed by o
    {
        if (o.bytes == 0) return;
        if (bytes == 0) { *this = o; return; }
        ok = ok && o.ok && o.first >= end && o.first - end < 4096;
        end = o.end;
        bytes += o.bytes;
    }
};

// Copies from pageable host memory run at close to the pinned rate where the
// device reaches host memory through the host's page tables (coherent
// host-device links): there the host entries copy dense caller spans straight
// to the device instead of staging every sequence through pinned memory.
static bool pageable_direct()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return false; }
    int v = cache[dev].load();
    if (v == 0) {
        int a = 0;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            a = 0;
        }
        v = a == 1 ? 1 : 2;
        cache[dev].store(v);
    }
    return v == 1;
}
// Below this, staging through pinned memory is cheaper than the span copies
// (each copy from pageable memory waits for the stream): measured on a GB300
// host, 10k x 150 bp (3 MB) 17 us faster staged, 100k (30 MB) 0.28 ms slower.
constexpr int64_t SPAN_MIN_BYTES = (int64_t)4 << 20;

// fn(k, lo, hi) on chunk k = [lo, hi) of [0, n) (chunks of `chunk`
// requests), the chunks in parallel on the host pool; returns the number of
// chunks.
template <class F>
static int64_t for_chunks(int64_t n, F fn, int64_t chunk = REQ_CHUNK)
{
    const int64_t nch = (n + chunk - 1) / chunk;
    parallel_for(nch, 1, [&](int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) fn(k, k * chunk, std::min(n, (k + 1) * chunk));
    });
    return nch;
}

// The first request of [0, n) for which check(i) returns an error (null when
// it passes), as a serial scan finds it, scanned in parallel chunks: its
// status is GA_INVALID_ARGUMENT with *err set, else GA_OK.
template <class F>
static int32_t first_failure(int64_t n, F check, const char** err)
{
    std::vector<int64_t> at((size_t)((n + REQ_CHUNK - 1) / REQ_CHUNK + 1), -1);
    std::vector<const char*> what(at.size(), nullptr);
    const int64_t nch = for_chunks(n, [&](int64_t k, int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i)
            if (const char* e = check(i)) { at[(size_t)k] = i; what[(size_t)k] = e; return; }
    });
    for (int64_t k = 0; k < nch; ++k)
        if (at[(size_t)k] >= 0) { *err = what[(size_t)k]; return GA_INVALID_ARGUMENT; }
    return GA_OK;
}

// The device's CIGAR lengths of pairs [lo, hi) against their slots (pair q's
// slot ends at slot_end[q], the previous one's end is its start), checked
// before any of them is expanded: a length outside [0, slot] means the device
// work did not finish as enqueued, and the call fails instead of writing
// outside the caller's buffer.
static bool lengths_fit(const int32_t* len, const int64_t* slot_end, int64_t lo, int64_t hi)
{
    for (int64_t q = lo; q < hi; ++q) {
        const int64_t cap = slot_end[q] - (q > 0 ? slot_end[q - 1] : 0);
        if (len[q] < 0 || len[q] > cap) return false;
    }
    return true;
}

static bool fail_here(int step)
{
    int want = g_fail_next.load();
    if (want == step && g_fail_next.compare_exchange_strong(want, 0)) return true;
    return false;
}

// ------------------------------------------------------------ validation --
static const char* E_NULL = "null pointer with non-zero length";
static const char* E_NEG = "negative length";
static const char* E_SMAX = "smax out of range [0, 511]";
static const char* E_SMAX_EX = "smax out of range [0, max_smax]";
static const char* E_ALLOC = "device allocation failed";
static const char* E_H2D = "host-to-device copy failed";
static const char* E_LAUNCH = "kernel launch failed";
static const char* E_D2H = "device-to-host copy failed";
static const char* E_SYNC = "device execution failed";
static const char* E_OVERFLOW = "internal error: CIGAR slot overflow";
static const char* E_SCRATCH = "internal error: traceback memory smaller than the plan needs";
static const char* E_HOSTMEM = "pinned host allocation failed";
static const char* E_BADLEN = "internal error: device returned a CIGAR longer than its slot";
static const char* E_CIGBUF = "cigar buffer is smaller than the batch needs";

// -------------------------------------------------------------------- WFA --
// The reference's checks of one WFA request (src/api/api.cpp:234-266), in its
// order: the error of the first it fails, null when it passes.
static const char* wfa_request_error(const ga_align_request& r, int32_t max_smax)
{
    if ((r.pattern_len > 0 && !r.pattern) || (r.text_len > 0 && !r.text)) return E_NULL;
    if (r.pattern_len < 0 || r.text_len < 0) return E_NEG;
    if (r.smax < 0 || r.smax > max_smax) return max_smax == GA_MAX_SMAX ? E_SMAX : E_SMAX_EX;
    return nullptr;
}

// Device scratch of one WFA batch: the 2-bit arena and purity flags, the
// per-warp wavefront stacks, the work counter; for the learned path also the
// queue items, lower bounds, predictions, bucket counts and the queues.
struct WfaScratch {
    uint64_t* packed = nullptr;
    uint8_t* pure = nullptr;
    int32_t* stack = nullptr;
    int32_t* ctr = nullptr;          // 64 ints: plain counter; learned: round counters
    int32_t* item = nullptr;         // queue item per pair (bucket | first smax << 8, or -1)
    int32_t* lb = nullptr;
    float* y = nullptr;
    int32_t* counts = nullptr;       // 2*buckets + 2
    int32_t* starts = nullptr;       // 2*buckets
    int2* big = nullptr;
    int2* small = nullptr;
    int2* esc = nullptr;
    uint16_t* lane_rec = nullptr;
    int slots = 0;                   // warp slots of the WFA (or warp-queue) kernel
    int lane_slots = 0;              // learned: warp slots of the lane kernel
    int64_t stack_slot = 0;
    int warp_smem = 0;
    int group = 32;                  // learned: lanes per warp-queue pair
    int64_t seq_bytes = 0;
    int chunk = 1;
};

// group: the tuned lanes per warp-queue pair (ga_tune.wfa_group).
static void size_wfa(WfaScratch& S, int n, int smax, bool trace, bool learned, int sm_count, int group)
{
    if (learned) {
        prepare_mlp();
        S.group = routed_group(smax, group);
        S.slots = (int)std::min<int64_t>(routed_max_slots(smax, trace, sm_count, S.group), ((int64_t)n + 3) / 4 * 4);
        S.lane_slots = (int)std::min<int64_t>(lane_max_slots(trace, sm_count), ((int64_t)n + 127) / 128 * 4);
        S.stack_slot = routed_stack_slot(smax, S.group);
        S.warp_smem = routed_warp_smem(smax, S.group);
    } else {
        S.slots = (int)std::min<int64_t>(wfa_max_slots(smax, trace, sm_count), ((int64_t)n + 3) / 4 * 4);
        S.stack_slot = (int64_t)(smax + 1) * (smax + 1);
    }
    if (trace) {
        const int64_t budget = (int64_t)16 << 30;     // stack memory cap
        S.slots = (int)std::min<int64_t>(S.slots, std::max<int64_t>(4, budget / (S.stack_slot * 4) / 4 * 4));
    }
    // pairs per counter increment: keep >= 8 grabs per warp
    S.chunk = (int)std::max<int64_t>(1, std::min<int64_t>(16, (int64_t)n / ((int64_t)S.slots * 8)));
}

static void carve_wfa(Carve& k, WfaScratch& S, int n, int64_t arena, bool trace, bool learned)
{
    S.seq_bytes = arena;
    S.packed = k.take<uint64_t>(packed_arena_words(arena));
    S.pure = k.take<uint8_t>(2 * (size_t)n);
    S.ctr = k.take<int32_t>(64, 256);
    S.stack = trace ? k.take<int32_t>((size_t)S.slots * S.stack_slot) : nullptr;
    if (learned) {
        S.item = k.take<int32_t>(n);
        S.lb = k.take<int32_t>(n);
        S.y = k.take<float>(2 * (size_t)n);
        S.counts = k.take<int32_t>(2 * route_buckets() + 4);
        S.starts = k.take<int32_t>(2 * route_buckets());
        S.big = k.take<int2>(n);
        S.small = k.take<int2>(n);
        S.esc = k.take<int2>(n);
        S.lane_rec = trace ? k.take<uint16_t>((size_t)S.lane_slots * lane_rec_slot()) : nullptr;
    }
}

// Every launch of one WFA batch on stream st (inputs already on the device).
// route: 0 plain, 1 queues by the cost model, 2 queues by the lower bound alone.
static cudaError_t enqueue_wfa(const WfaScratch& S, PairDesc D, int smax, bool trace, int route, int lane_smax,
                               int32_t* score, int32_t* len, char* cig, int32_t* err, cudaStream_t st)
{
    D.packed = S.packed;
    D.pure = S.pure;
    WfaArgs A;
    A.D = D; A.smax = smax; A.trace = trace ? 1 : 0;
    A.out_score = score; A.out_len = len; A.out_cigar = cig;
    A.stack = S.stack; A.stack_slot = S.stack_slot; A.counter = S.ctr; A.err = err;
    A.chunk = S.chunk;
    cudaError_t e = cudaMemsetAsync(S.ctr, 0, 64 * sizeof(int32_t), st);
    if (e == cudaSuccess) e = launch_pack(D, S.seq_bytes, S.packed, S.pure, st);
    if (e != cudaSuccess) return e;
    if (route == 0) return launch_wfa(A, S.slots, st);
    const int NB = route_buckets();
    if ((e = cudaMemsetAsync(S.counts, 0, sizeof(int32_t) * (2 * NB + 4), st)) != cudaSuccess) return e;
    if ((e = launch_route_model(D, smax, lane_smax, route == 1, S.item, S.lb, S.y, S.counts, score, len, st)) !=
        cudaSuccess)
        return e;
    if ((e = launch_route(D.n, S.item, S.counts, S.starts, S.big, S.small, st)) != cudaSuccess) return e;
    // ctr layout: [0] warp-queue next, [1] lane-queue next, [2] escalation
    // next, [3] whole-block next, [32] escalation count; counts[2 NB + 2]:
    // whole-block items (the warp queue's first ones)
    RoutedArgs R;
    R.A = A;
    R.warp_smem = S.warp_smem;
    R.group = S.group;
    R.big = S.big;
    R.big_count = S.counts + 2 * NB;
    R.big_next = S.ctr;
    R.small = S.small;
    R.small_count = S.counts + 2 * NB + 1;
    R.small_next = S.ctr + 1;
    R.esc = S.esc;
    R.esc_count = S.ctr + 32;
    R.esc_next = S.ctr + 2;
    R.lane_rec = S.lane_rec;
    R.block_count = S.counts + 2 * NB + 2;
    R.block_next = S.ctr + 3;
    return launch_routed(R, S.lane_slots, S.slots, st);
}

// Replays `exec` when `key` (everything the enqueued launches bake in) is the
// one it was captured for; otherwise captures enqueue() on stream st first.
// `launches` keeps the number of library kernels the graph holds (counted
// once per replay).
static cudaError_t replay_graph(cudaGraphExec_t& exec, std::vector<uint64_t>& have, const std::vector<uint64_t>& key,
                                int& launches, cudaStream_t st, const std::function<cudaError_t()>& enqueue)
{
    if (!exec || have != key) {
        // one capture at a time in the process (the ranges of a ranged call
        // capture their first calls from their own threads); a capture is
        // made once per launch shape, so this costs nothing on replays
        static std::mutex capture_mu;
        std::lock_guard<std::mutex> lk(capture_mu);
        if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
        have.clear();
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        const long long before = t_launches;
        const cudaError_t e1 = enqueue();
        launches = (int)(t_launches - before);              // (nothing ran: captured only)
        g_launches.fetch_sub(launches);
        e = cudaStreamEndCapture(st, &g);
        if (e1 != cudaSuccess || e != cudaSuccess) { if (g) cudaGraphDestroy(g); return e1 != cudaSuccess ? e1 : e; }
        e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { exec = nullptr; return e; }
        have = key;
    }
    note_graph_launches(launches);
    return cudaGraphLaunch(exec, st);
}

// Learned path as one CUDA graph, cached per context by everything the
// launches bake in.
static cudaError_t run_wfa_graph(Ctx* c, const WfaScratch& S, const PairDesc& D, int smax, bool trace, int route,
                                 int lane_smax, int32_t* score, int32_t* len, char* cig, int32_t* err, cudaStream_t st)
{
    const std::vector<uint64_t> key = {c->dev_gen, (uint64_t)D.n, (uint64_t)(uintptr_t)D.seq, (uint64_t)smax,
                                       (uint64_t)trace | (uint64_t)lane_smax << 8 | (uint64_t)route << 16 |
                                           (uint64_t)S.group << 24,
                                       (uint64_t)(uintptr_t)score, (uint64_t)(uintptr_t)cig,
                                       (uint64_t)(uintptr_t)D.a_off, (uint64_t)(uintptr_t)S.packed};
    return replay_graph(c->gexec, c->gkey, key, c->glaunches, st, [&]() {
        return enqueue_wfa(S, D, smax, trace, route, lane_smax, score, len, cig, err, st);
    });
}

static bool profiling_on();

// Where the calling thread's last learned WFA run left its queue counters.
struct RouteRecord {
    Ctx* c = nullptr;
    uint64_t gen = 0;
    const int32_t* counts = nullptr;
    const int32_t* ctr = nullptr;
    const int32_t* item = nullptr;
    int n = 0;
    int64_t seq_bytes = 0;
    int chunk = 1;
};
static thread_local RouteRecord t_route;

static void note_route(Ctx* c, const WfaScratch& S, int n)
{
    t_route.c = c;
    t_route.gen = c->dev_gen;
    t_route.counts = S.counts;
    t_route.ctr = S.ctr;
    t_route.item = S.item;
    t_route.n = n;
}

int route_mode(int requested)
{
    if (requested == 1 && !cost_model_loaded()) return 0;
    return (requested == 1 || requested == 2) ? requested : 0;
}

// One chunk of a WFA batch's requests in the first pass over them: the
// checks, the batch smax and trace flag, and the chunk's sizes -- its own
// sides in the staging arena (a side that repeats the previous request's, same
// pointer and length, is staged once and shares its offset), CIGAR slots,
// packed CIGAR bytes -- and where its last own side of each kind starts.
struct WfaChunk {
    int64_t arena = 0, cig = 0, pkb = 0;
    int64_t tail_a = -1, tail_b = -1;       // from the chunk's arena start; -1: no own side of that kind
    int32_t bad = -1;                       // first request failing the checks
    const char* err = nullptr;
    int smax = INT32_MAX;
    bool trace = false;
    SideSpan sa, sb;                        // where its own patterns and texts lie in the caller's memory
};
// Large host batches run as up to WFA_RANGES contiguous ranges of whole
// chunks, each on its own thread, context and stream (range k's priority k
// steps below range 0's): one range's staging and its results' finish on the
// host overlap the others' copies and kernels.  No side is shared across a
// range start (each range's arena holds all it reads).
constexpr int WFA_RANGES = 4;
constexpr int64_t WFA_RANGE_MIN = 262144;

int32_t wfa_batch(const ga_align_request* reqs, int32_t n, int32_t max_smax, int route,
                  const WfaFinish& fin, const char** err, int64_t cig_cap)
{
    *err = nullptr;
    if (n <= 0) return GA_OK;
    const int64_t CH = wfa_chunk(n);                          // requests per chunk
    const int64_t nch = (n + CH - 1) / CH;
    const int K = n >= WFA_RANGE_MIN ? (int)std::min<int64_t>(WFA_RANGES, nch) : 1;
    std::vector<int64_t> kc((size_t)K + 1);                      // range k: chunks [kc[k], kc[k + 1])
    std::vector<uint8_t> range_start((size_t)nch, 0);
    for (int k = 0; k <= K; ++k) kc[(size_t)k] = nch * k / K;
    for (int k = 0; k < K; ++k) range_start[(size_t)kc[(size_t)k]] = 1;

    // pass 1, in parallel chunks: checks (the first failing request's error,
    // as a serial pass finds it), smax, trace, own sides and sizes
    static thread_local std::vector<uint8_t> own_v;
    static thread_local std::vector<int64_t> slot_v;
    own_v.resize((size_t)n);
    slot_v.resize((size_t)n);
    uint8_t* own = own_v.data();
    int64_t* slot_end = slot_v.data();              // per range: CIGAR slot ends from the range's first slot
    std::vector<WfaChunk> ck((size_t)nch);
    const auto pass1 = [&](int64_t k, int64_t lo, int64_t hi) {
        WfaChunk& C = ck[(size_t)k];
        for (int64_t i = lo; i < hi; ++i) {
            const ga_align_request& r = reqs[i];
            if (C.bad < 0)
                if (const char* e = wfa_request_error(r, max_smax)) { C.bad = (int32_t)i; C.err = e; }
            C.smax = std::min(C.smax, (int)r.smax);
            C.trace |= r.with_cigar != 0;
            const bool fresh = i == 0 || (i == lo && range_start[(size_t)k]);
            const bool oa = fresh || !(r.pattern == reqs[i - 1].pattern && r.pattern_len == reqs[i - 1].pattern_len);
            const bool ob = fresh || !(r.text == reqs[i - 1].text && r.text_len == reqs[i - 1].text_len);
            own[i] = (uint8_t)(oa | ob << 1);
            if (oa) { C.tail_a = C.arena; C.arena += round32(r.pattern_len); C.sa.add(r.pattern, r.pattern_len); }
            if (ob) { C.tail_b = C.arena; C.arena += round32(r.text_len); C.sb.add(r.text, r.text_len); }
            const int64_t cap = (int64_t)r.pattern_len + r.text_len;
            C.cig += cap;
            C.pkb += (cap + 3) / 4;
        }
    };
    for_chunks(n, pass1, CH);
    int smax = INT32_MAX;
    bool trace = false;
    std::vector<int64_t> base((size_t)(3 * (nch + 1))), carry((size_t)(2 * nch));
    int64_t arena = 0, cig = 0, pkb = 0, ca = 0, cb = 0;
    for (int64_t k = 0; k < nch; ++k) {
        const WfaChunk& C = ck[(size_t)k];
        if (C.bad >= 0) {
            *err = C.err;
            return GA_INVALID_ARGUMENT;
        }
        smax = std::min(smax, C.smax);
        trace |= C.trace;
        base[3 * k] = arena; base[3 * k + 1] = cig; base[3 * k + 2] = pkb;
        carry[2 * k] = ca; carry[2 * k + 1] = cb;          // the previous request's side offsets
        if (C.tail_a >= 0) ca = arena + C.tail_a;
        if (C.tail_b >= 0) cb = arena + C.tail_b;
        arena += C.arena; cig += C.cig; pkb += C.pkb;
    }
    base[3 * nch] = arena; base[3 * nch + 1] = cig; base[3 * nch + 2] = pkb;
    if (trace && (cig_cap < 0 || cig > cig_cap)) {
        *err = E_CIGBUF;
        return GA_INVALID_ARGUMENT;
    }
    route = route_mode(route);
    const bool learned = route != 0;
    const ga_tune tuned = tune_current();
    const int lane_smax = tuned.wfa_lane_smax;

    // one range: requests of chunks [kc[k], kc[k + 1]), offsets from the range's own bases
    std::vector<int64_t> rh2d((size_t)K, 0), rd2h((size_t)K, 0);
    auto run_range = [&](int k, const char** rerr) -> int32_t {
        const int64_t c0 = kc[(size_t)k], c1 = kc[(size_t)k + 1];
        const int64_t r0 = std::min<int64_t>(n, c0 * CH), r1 = std::min<int64_t>(n, c1 * CH);
        const int32_t nk = (int32_t)(r1 - r0);
        if (nk <= 0) return GA_OK;
        const int64_t a0 = base[3 * c0], g0 = base[3 * c0 + 1], p0 = base[3 * c0 + 2];
        const int64_t arena_k = base[3 * c1] - a0 + 64;             // + read-past padding
        const int64_t cig_k = trace ? base[3 * c1 + 1] - g0 : 0;
        const int64_t pkb_k = trace ? base[3 * c1 + 2] - p0 : 0;

        // the range's own patterns and texts: copied as the caller laid them
        // out (two spans) and moved into place on the device, or staged here
        SideSpan spa, spb;
        for (int64_t kk = c0; kk < c1; ++kk) { spa.join(ck[(size_t)kk].sa); spb.join(ck[(size_t)kk].sb); }
        const bool span = spa.ok && spb.ok && spa.bytes + spb.bytes >= SPAN_MIN_BYTES && pageable_direct();
        const int64_t span_a = span ? (int64_t)(spa.end - spa.first) : 0, span_b = span ? (int64_t)(spb.end - spb.first) : 0;

        Ctx* c = acquire_ctx(rerr, K > 1 ? k : -1);
        if (!c) return GA_DEVICE_ERROR;
        struct Guard { Ctx* c; ~Guard() { release_ctx(c); } } guard{c};
        WfaScratch S;
        size_wfa(S, nk, smax, trace, learned, c->sm_count, tuned.wfa_group);
        // layout: [a_off a_len b_off b_len out_off pk_off (src_a src_b) | seq] in, [score len checks err |
        // packed CIGARs] back, then (device) the CIGAR slots, the scratch and the caller's spans
        int64_t *ha, *hb, *ho, *hpo, *da, *db, *dout, *dpo, *hsa, *hsb, *dsa, *dsb;
        int32_t *hal, *hbl, *dal, *dbl, *hsc, *hln, *dsc, *dln, *her, *der;
        uint8_t *hseq, *dseq, *hvf, *dvf, *hpk, *dpk, *dspan_a, *dspan_b;
        char* dcg;
        auto io = [&](Carve& q, int64_t** pa, int32_t** pal, int64_t** pb, int32_t** pbl, int64_t** po,
                      int64_t** ppo, int64_t** psa, int64_t** psb, uint8_t** ps, int32_t** psc, int32_t** pln,
                      uint8_t** pvf, int32_t** per, uint8_t** ppk) {
            *pa = q.take<int64_t>(nk); *pal = q.take<int32_t>(nk);
            *pb = q.take<int64_t>(nk); *pbl = q.take<int32_t>(nk);
            *po = q.take<int64_t>(nk); *ppo = q.take<int64_t>(nk);
            *psa = q.take<int64_t>(span ? nk : 0); *psb = q.take<int64_t>(span ? nk : 0);
            *ps = q.take<uint8_t>(arena_k);
            *psc = q.take<int32_t>(nk); *pln = q.take<int32_t>(nk);
            *pvf = q.take<uint8_t>(trace ? nk : 0);
            *per = q.take<int32_t>(1, 4);
            *ppk = q.take<uint8_t>((size_t)pkb_k, 4);
        };
        Carve hk(nullptr), dk(nullptr);
        io(hk, &ha, &hal, &hb, &hbl, &ho, &hpo, &hsa, &hsb, &hseq, &hsc, &hln, &hvf, &her, &hpk);
        io(dk, &da, &dal, &db, &dbl, &dout, &dpo, &dsa, &dsb, &dseq, &dsc, &dln, &dvf, &der, &dpk);
        dcg = dk.take<char>(cig_k + 1);
        carve_wfa(dk, S, nk, arena_k, trace, learned);
        dspan_a = dk.take<uint8_t>((size_t)span_a);
        dspan_b = dk.take<uint8_t>((size_t)span_b);
        if (fail_here(1) || !ensure_dev(c, dk.off)) { *rerr = E_ALLOC; return GA_DEVICE_ERROR; }
        if (!ensure_host(c, hk.off)) { *rerr = E_HOSTMEM; return GA_DEVICE_ERROR; }
        {
            Carve h(c->host), d(c->dev);
            io(h, &ha, &hal, &hb, &hbl, &ho, &hpo, &hsa, &hsb, &hseq, &hsc, &hln, &hvf, &her, &hpk);
            io(d, &da, &dal, &db, &dbl, &dout, &dpo, &dsa, &dsb, &dseq, &dsc, &dln, &dvf, &der, &dpk);
            dcg = d.take<char>(cig_k + 1);
            carve_wfa(d, S, nk, arena_k, trace, learned);
            dspan_a = d.take<uint8_t>((size_t)span_a);
            dspan_b = d.take<uint8_t>((size_t)span_b);
        }

        // pass 2, in the same chunks: offsets and the staging of every own side
        parallel_for(c1 - c0, 1, [&](int64_t j0, int64_t j1) {
            for (int64_t kk = c0 + j0; kk < c0 + j1; ++kk) {
                const int64_t lo = kk * CH, hi = std::min<int64_t>(n, lo + CH);
                int64_t at = base[3 * kk] - a0, cg = base[3 * kk + 1] - g0, pk = base[3 * kk + 2] - p0;
                int64_t cur_a = carry[2 * kk] - a0, cur_b = carry[2 * kk + 1] - a0;
                for (int64_t i = lo; i < hi; ++i) {
                    const ga_align_request& r = reqs[i];
                    const int64_t q = i - r0;
                    if (span) { hsa[q] = -1; hsb[q] = -1; }
                    if (own[i] & 1) {
                        cur_a = at;
                        at += round32(r.pattern_len);
                        if (r.pattern_len > 0) {
                            if (span) hsa[q] = (int64_t)((uintptr_t)r.pattern - spa.first);
                            else std::memcpy(hseq + cur_a, r.pattern, (size_t)r.pattern_len);
                        }
                    }
                    if (own[i] & 2) {
                        cur_b = at;
                        at += round32(r.text_len);
                        if (r.text_len > 0) {
                            if (span) hsb[q] = (int64_t)((uintptr_t)r.text - spb.first);
                            else std::memcpy(hseq + cur_b, r.text, (size_t)r.text_len);
                        }
                    }
                    ha[q] = cur_a; hal[q] = r.pattern_len;
                    hb[q] = cur_b; hbl[q] = r.text_len;
                    const int64_t cap = (int64_t)r.pattern_len + r.text_len;
                    ho[q] = cg; cg += cap;
                    slot_end[i] = cg;
                    hpo[q] = pk; pk += (cap + 3) / 4;
                }
            }
        });
        if (!span) std::memset(hseq + arena_k - 64, 0, 64);
        // descriptors (+ the arena when staged here), contiguous; the spans from the caller's memory
        const size_t in_bytes = (size_t)((char*)(span ? hseq : hseq + arena_k) - c->host);
        rh2d[(size_t)k] = (int64_t)in_bytes + span_a + span_b;
        PairDesc D;
        D.seq = dseq; D.packed = nullptr; D.pure = nullptr;
        D.a_off = da; D.a_len = dal; D.b_off = db; D.b_len = dbl; D.out_off = dout; D.n = nk;
        bool ok = !fail_here(2) &&
                  cudaMemcpyAsync(c->dev, c->host, in_bytes, cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
                  cudaMemsetAsync(der, 0, sizeof(int32_t), c->stream) == cudaSuccess;
        if (ok && span) {
            ok = (span_a == 0 || cudaMemcpyAsync(dspan_a, (const void*)spa.first, (size_t)span_a,
                                                 cudaMemcpyHostToDevice, c->stream) == cudaSuccess) &&
                 (span_b == 0 || cudaMemcpyAsync(dspan_b, (const void*)spb.first, (size_t)span_b,
                                                 cudaMemcpyHostToDevice, c->stream) == cudaSuccess) &&
                 launch_gather_sides(D, dseq, dspan_a, dspan_b, dsa, dsb, c->stream) == cudaSuccess &&
                 cudaMemsetAsync(dseq + arena_k - 64, 0, 64, c->stream) == cudaSuccess;
        }
        if (!ok) {
            cudaGetLastError();
            *rerr = E_H2D;
            return GA_DEVICE_ERROR;
        }
        cudaError_t le;
        if (fail_here(3)) le = cudaErrorLaunchFailure;
        else if (learned && !profiling_on())
            le = run_wfa_graph(c, S, D, smax, trace, route, lane_smax, dsc, dln, dcg, der, c->stream);
        else le = enqueue_wfa(S, D, smax, trace, route, lane_smax, dsc, dln, dcg, der, c->stream);
        if (learned) note_route(c, S, nk);
        if (le == cudaSuccess && trace) le = launch_wfa_validate(D, dsc, dln, dcg, dvf, c->stream);
        if (le == cudaSuccess && trace) le = launch_cigar_pack(D, dln, dcg, dpo, dpk, c->stream);
        if (le != cudaSuccess) {
            cudaGetLastError();
            *rerr = E_LAUNCH;
            return GA_DEVICE_ERROR;
        }
        // outputs are contiguous on both sides: score, len, checks, err, packed CIGARs
        const size_t out_bytes = (size_t)((char*)(dpk + pkb_k) - (char*)dsc);
        rd2h[(size_t)k] = (int64_t)out_bytes;
        if (fail_here(4) || cudaMemcpyAsync(hsc, dsc, out_bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) {
            cudaGetLastError();
            *rerr = E_D2H;
            return GA_DEVICE_ERROR;
        }
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
            cudaGetLastError();
            *rerr = E_SYNC;
            return GA_DEVICE_ERROR;
        }
        if (*her != 0) { *rerr = E_OVERFLOW; return GA_DEVICE_ERROR; }
        if (trace && fail_here(5)) hln[0] = INT32_MAX;       // test hook: a length past its slot
        WfaView v{hsc, hln, hpk, hpo, slot_end + r0, trace, trace ? hvf : nullptr, r0, g0};
        std::atomic<bool> bad{false};
        parallel_for(nk, CH, [&](int64_t lo, int64_t hi) {
            if (trace && !lengths_fit(hln, slot_end + r0, lo, hi)) { bad = true; return; }
            fin(r0 + lo, r0 + hi, v);
        });
        if (bad) { *rerr = E_BADLEN; return GA_DEVICE_ERROR; }
        return GA_OK;
    };
    std::vector<int32_t> st((size_t)K, GA_OK);
    std::vector<const char*> errs((size_t)K, nullptr);
    if (K == 1) {
        st[0] = run_range(0, &errs[0]);
    } else {
        int dev = 0;
        cudaGetDevice(&dev);
        PoolQuiet quiet;
        std::vector<std::thread> th;
        for (int k = 0; k + 1 < K; ++k)
            th.emplace_back([&, k] {
                cudaSetDevice(dev);
                st[(size_t)k] = run_range(k, &errs[(size_t)k]);
            });
        st[(size_t)K - 1] = run_range(K - 1, &errs[(size_t)K - 1]);   // this thread keeps the last range's route record
        for (std::thread& x : th) x.join();
    }
    t_h2d = t_d2h = 0;
    for (int k = 0; k < K; ++k) { t_h2d += rh2d[(size_t)k]; t_d2h += rd2h[(size_t)k]; }
    for (int k = 0; k < K; ++k)
        if (st[(size_t)k] != GA_OK) {
            *err = errs[(size_t)k];
            return st[(size_t)k];
        }
    return GA_OK;
}

// --------------------------------------------------------------------- SW --
static const char* E_SW_MATCH = "SW scoring: match must be > 0 (the score is 0 for every input otherwise)";
static const char* E_SW_MISMATCH = "SW scoring: mismatch must be < match";
static const char* E_SW_GAPS = "SW scoring: gap costs must be > 0";
static const char* E_SW_GEGO =
    "SW scoring: gap_extend > gap_open with with_cigar cannot re-score to its own score (api.hpp; "
    "RESULTADO_H9_SW2_TRACE.md). Score-only requests may use it";
static const char* E_SW_MIXED = "all requests in an SW batch must share one scoring scheme";
static const char* E_SW_SMEM =
    "pattern_len exceeds this device's shared-memory limit for the score kernel (see api.hpp "
    "supported-size limits)";

int32_t sw_check(const ga_sw_request* reqs, int32_t n, const char** err)
{
    if (n <= 0) return GA_OK;
    const ga_sw_scoring s0 = reqs[0].scoring;
    return first_failure(n, [&](int64_t i) -> const char* {
        const ga_sw_request& r = reqs[i];
        if ((r.text_len > 0 && !r.text) || (r.pattern_len > 0 && !r.pattern)) return E_NULL;
        if (r.text_len < 0 || r.pattern_len < 0) return E_NEG;
        const ga_sw_scoring& s = r.scoring;
        if (s.match <= 0) return E_SW_MATCH;
        if (s.mismatch >= s.match) return E_SW_MISMATCH;
        if (s.gap_open <= 0 || s.gap_extend <= 0) return E_SW_GAPS;
        if (r.with_cigar && s.gap_extend > s.gap_open) return E_SW_GEGO;
        if (s.match != s0.match || s.mismatch != s0.mismatch || s.gap_open != s0.gap_open ||
            s.gap_extend != s0.gap_extend) return E_SW_MIXED;
        return nullptr;
    }, err);
}

// Work plan of one SW batch, as the device planner left it (sw_plan.cu):
// per list its length in the flattened work array and the largest per-warp
// memory of its items; the band-edge slot; the 16-bit list's largest item;
// pairs taken on the optimistic 16-bit rule and their 32-bit memory.
struct SwPlan {
    int64_t ints[SP_LISTS] = {0, 0, 0};
    int64_t dir[SP_LISTS] = {0, 0, 0};
    int64_t edge_slot = 2;
    int64_t max16_cells = 0;
    int64_t n_opt = 0, dir_opt = 0;
};

// The plan, built on the device (sw_plan.cu) into `dwork`, its record into dres.
static cudaError_t enqueue_plan_sw(const PairDesc& D, const ga_sw_scoring& sc, bool trace, int64_t cell_limit,
                                   int32_t too_large_score, int32_t* out_score, int32_t* dwork, int32_t* scratch,
                                   long long* dres, const ga_tune& T, cudaStream_t st, const uint8_t* try16 = nullptr)
{
    SwPlanArgs A;
    A.D = D;
    A.match = sc.match; A.mismatch = sc.mismatch; A.gap_open = sc.gap_open; A.gap_extend = sc.gap_extend;
    A.cell_limit = cell_limit;
    A.use16 = T.sw_pack16 ? 1 : 0;
    A.window = T.sw_window;
    A.opt16_pct = T.sw_opt16_pct;
    A.long_log2 = T.sw_long_log2;
    A.too_large_score = too_large_score;
    A.score_only = trace ? 0 : 1;
    A.out_score = out_score;
    A.work = dwork;
    A.res = dres;
    A.try16 = try16;
    return launch_sw_plan(A, scratch, st);
}

// The same, then its record read back into P's list lengths and sizes.
static cudaError_t device_plan_sw(const PairDesc& D, const ga_sw_scoring& sc, bool trace, int64_t cell_limit,
                                  int32_t too_large_score, int32_t* out_score, int32_t* dwork, int32_t* scratch,
                                  long long* dres, long long* hres, const ga_tune& T, cudaStream_t st, SwPlan& P,
                                  const uint8_t* try16 = nullptr)
{
    cudaError_t e =
        enqueue_plan_sw(D, sc, trace, cell_limit, too_large_score, out_score, dwork, scratch, dres, T, st, try16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hres, dres, sizeof(long long) * SP_RES, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    P = SwPlan();
    for (int l = 0; l < SP_LISTS; ++l) {
        P.ints[l] = hres[SP_INTS + l];
        P.dir[l] = (hres[SP_DIR + l] + 3) / 4 * 4;
    }
    P.edge_slot = std::max<int64_t>(2, hres[SP_EDGE]);
    P.max16_cells = hres[SP_MAXC16];
    P.n_opt = hres[SP_NOPT];
    P.dir_opt = (hres[SP_DIROPT] + 3) / 4 * 4;
    return cudaSuccess;
}

// Upper bounds of the device-built plan from the requests' lengths alone, for
// launches enqueued without reading the plan back.  Purity is not known on the
// host, so every pair counts in the 16-bit list when its lengths allow it and
// in its 32-bit list as well; per-warp memory is the largest any of those
// pairs (or items) can need.  The kernels take the exact figures from the
// plan on the device (plan_view); these only size the grids and the memory.
static SwPlan bound_plan_sw(const ga_sw_request* reqs, int32_t n, bool trace, int64_t cell_limit, const ga_tune& T,
                            bool learned)
{
    SwPlan P;
    const ga_sw_scoring sc = reqs[0].scoring;
    int maxM16 = 0, maxN16 = 0;
    int64_t n16 = 0, cnt[SP_LISTS] = {0, 0, 0}, edge = 2;
    for (int32_t i = 0; i < n; ++i) {
        const int m = reqs[i].text_len, nn = reqs[i].pattern_len;
        if (cell_limit >= 0 && m > 0 && nn > 0 && ((int64_t)m + 1) * ((int64_t)nn + 1) > cell_limit) continue;
        const bool strict = T.sw_pack16 && sw16_eligible(m, nn, sc.match, sc.mismatch, sc.gap_open, sc.gap_extend);
        // (the SW model may send any pair to the 16-bit kernel)
        const bool u16 = strict || (trace && T.sw_pack16 &&
                                    (learned ? (m > 0 && nn > 0 &&
                                                sw16_scheme_ok(sc.match, sc.mismatch, sc.gap_open, sc.gap_extend))
                                             : sw16_eligible_opt(m, nn, sc.match, sc.mismatch, sc.gap_open,
                                                                 sc.gap_extend, T.sw_opt16_pct)));
        if (u16) {
            ++n16;
            maxM16 = std::max(maxM16, m);
            maxN16 = std::max(maxN16, nn);
            if (!strict) {
                ++P.n_opt;
                P.dir_opt = std::max(P.dir_opt, sw32ck_dir_words(m, nn, 0));
            }
        }
        const int l = (trace && sw32ck_long(m, nn, T.sw_long_log2)) ? SP_L32LONG : SP_L32;
        ++cnt[l];
        if (trace) P.dir[l] = std::max(P.dir[l], sw32ck_dir_words(m, nn, T.sw_long_log2));
        edge = std::max<int64_t>(edge, 2 * (int64_t)std::max(m, 0));
    }
    P.ints[SP_L16] = 2 * ((n16 + 1) / 2);
    P.dir[SP_L16] = n16 ? (trace ? sw16ck_dir_words(maxM16, maxN16, T.sw_window) : sw16so_dir_words(maxM16, maxN16)) : 0;
    P.max16_cells = (int64_t)maxM16 * maxN16;
    P.ints[SP_L32] = cnt[SP_L32];
    P.ints[SP_L32LONG] = cnt[SP_L32LONG];
    for (int l = 0; l < SP_LISTS; ++l) P.dir[l] = (P.dir[l] + 3) / 4 * 4;
    P.dir_opt = (P.dir_opt + 3) / 4 * 4;
    P.edge_slot = edge;
    return P;
}

// Device memory the checkpoint / direction tables of one call may take:
// 60 % of what is free now plus the call's own arena (which it may replace)
// and the idle contexts' arenas (which give way to it, trim_idle),
// between 4 GB and 200 GB, shared by `parts` concurrent calls.  Long pairs
// need tens of MB per resident warp, so this bounds how many run at once.
static int64_t sw_dir_budget(const Ctx* c, int parts)
{
    size_t fr = 0, tot = 0;
    int64_t avail = (int64_t)96 << 30;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess)
        avail = ((int64_t)fr + (int64_t)c->dev_cap + (int64_t)idle_dev_bytes(c->device)) * 6 / 10;
    else cudaGetLastError();
    avail /= std::max(1, parts);
    return std::max<int64_t>((int64_t)4 << 30, std::min<int64_t>(avail, (int64_t)200 << 30));
}

// Slots (resident warps) per launch and the direction-table words the launches
// need (they run one after another on one stream and share the table).
struct SwSlots {
    int s[SP_LISTS] = {0, 0, 0};
    int s_esc = 0;                                    // the 32-bit launch for pairs handed over by the 16-bit kernel
    int64_t dir_words = 0, max_slots = 4;
};

static SwSlots size_sw(const SwPlan& P, bool trace, const ga_tune& T, int sm_count, int64_t budget)
{
    SwSlots S;
    for (int l = 0; l < SP_LISTS; ++l) {
        if (P.ints[l] <= 0) continue;
        // warp slots come in blocks of 4
        int s;
        if (l == SP_L16) {
            s = trace ? sw16ck_max_slots(sm_count, T.sw_window) : sw16so_max_slots(sm_count);
            s = (int)std::min<int64_t>(s, (P.ints[l] / 2 + 3) / 4 * 4);
        } else {
            s = trace ? sw32ck_max_slots(l == SP_L32LONG, sm_count) : sw_max_slots(sm_count);
            s = (int)std::min<int64_t>(s, (P.ints[l] + 3) / 4 * 4);
        }
        if (P.dir[l] > 0) s = (int)std::min<int64_t>(s, std::max<int64_t>(4, budget / (P.dir[l] * 4) / 4 * 4));
        S.s[l] = s;
        S.dir_words = std::max(S.dir_words, (int64_t)s * P.dir[l]);
        S.max_slots = std::max<int64_t>(S.max_slots, s);
    }
    if (trace && P.n_opt > 0 && P.dir_opt > 0) {
        int s = sw32ck_max_slots(true, sm_count);
        s = (int)std::min<int64_t>(s, (P.n_opt + 3) / 4 * 4);
        s = (int)std::min<int64_t>(s, std::max<int64_t>(4, budget / (P.dir_opt * 4) / 4 * 4));
        S.s_esc = s;
        S.dir_words = std::max(S.dir_words, (int64_t)s * P.dir_opt);
        S.max_slots = std::max<int64_t>(S.max_slots, s);
    }
    return S;
}

// Enqueue every SW launch of a plan.  `dwork` holds the plan's lists
// concatenated in list order; `ctr` has 8 zeroed ints; esc_list (n ints)
// takes the pairs the 16-bit kernel hands to the 32-bit one.
// With dplan set (plan mode), P holds bounds (bound_plan_sw) and every launch
// takes its items and per-warp memory from the device-built record dplan
// (plan_view), its memory bounded by the dir_words / edge ints S sized.
static cudaError_t launch_plan(const SwPlan& P, const SwSlots& S, const PairDesc& D, const ga_sw_scoring& sc,
                               bool trace, const ga_tune& T, const int32_t* dwork, int32_t* out_score, int32_t* out_pos,
                               int32_t* out_len, char* out_cigar, uint32_t* dirs, int32_t* edge, int32_t* ctr,
                               int32_t* err, cudaStream_t st, int32_t* esc_list, const long long* dplan = nullptr)
{
    const int64_t dir_cap = S.dir_words, edge_cap = S.max_slots * P.edge_slot;
    // ctr: [l] list l's item counter, [6] pairs handed over, [7] their counter
    const bool opt = trace && P.n_opt > 0 && esc_list && S.s_esc > 0;
    const int64_t coop = T.sw_coop_log2 < 40 ? ((int64_t)1 << T.sw_coop_log2) : -1;
    int64_t base = 0;
    if (P.ints[SP_L16] > 0) {
        Sw16Args A;
        A.D = D; A.work = dwork; A.nwork = (int32_t)(P.ints[SP_L16] / 2);
        A.match = sc.match; A.mismatch = sc.mismatch; A.gap_open = sc.gap_open; A.gap_extend = sc.gap_extend;
        A.out_score = out_score; A.out_pos = out_pos; A.out_len = out_len; A.out_cigar = out_cigar;
        A.dirs = dirs; A.dir_slot = P.dir[SP_L16]; A.edge = edge; A.edge_slot = P.edge_slot;
        A.counter = ctr + SP_L16; A.err = err;
        A.coop_cells = coop;
        if (dplan) { A.plan = dplan; A.plan_list = SP_L16; A.dir_cap = dir_cap; A.edge_cap = 0; }
        if (opt) {
            A.ovf_limit = sw16_overflow_limit(sc.match);
            A.esc_list = esc_list;
            A.esc_count = ctr + 6;
        }
        const bool blocks = A.coop_cells >= 0 && P.max16_cells > A.coop_cells;
        const cudaError_t e = trace ? launch_sw16ck(A, S.s[SP_L16], T.sw_window, blocks, st)
                                    : launch_sw16so(A, S.s[SP_L16], st);
        if (e != cudaSuccess) return e;
        if (opt) {
            // the pairs the 16-bit kernel handed over, on the 32-bit long shape
            SwArgs B;
            B.D = D; B.work = esc_list; B.nwork = 0; B.nwork_dev = ctr + 6;
            B.match = sc.match; B.mismatch = sc.mismatch; B.gap_open = sc.gap_open; B.gap_extend = sc.gap_extend;
            B.out_score = out_score; B.out_pos = out_pos; B.out_len = out_len; B.out_cigar = out_cigar;
            B.dirs = dirs; B.dir_slot = P.dir_opt; B.edge = edge; B.edge_slot = P.edge_slot;
            B.counter = ctr + 7; B.err = err;
            B.coop_cells = coop;
            if (dplan) { B.plan = dplan; B.plan_list = SP_ESC; B.dir_cap = dir_cap; B.edge_cap = 0; }
            const cudaError_t e2 = launch_sw32ck(B, true, S.s_esc, st);
            if (e2 != cudaSuccess) return e2;
        }
    }
    base += P.ints[SP_L16];
    for (int l = SP_L32; l <= SP_L32LONG; ++l) {
        if (P.ints[l] > 0) {
            SwArgs A;
            A.D = D; A.work = dwork + base; A.nwork = (int32_t)P.ints[l];
            A.match = sc.match; A.mismatch = sc.mismatch; A.gap_open = sc.gap_open; A.gap_extend = sc.gap_extend;
            A.out_score = out_score; A.out_pos = out_pos; A.out_len = out_len; A.out_cigar = out_cigar;
            A.dirs = dirs; A.dir_slot = P.dir[l]; A.edge = edge; A.edge_slot = P.edge_slot;
            A.counter = ctr + l; A.err = err;
            A.coop_cells = l == SP_L32LONG ? coop : -1;
            if (dplan) {
                A.plan = dplan;
                A.plan_list = l;
                A.work = dwork;
                A.dir_cap = trace ? dir_cap : 0;
                A.edge_cap = trace ? 0 : edge_cap;
            }
            const cudaError_t e = trace ? launch_sw32ck(A, l == SP_L32LONG, S.s[l], st) : launch_sw(A, S.s[l], st);
            if (e != cudaSuccess) return e;
        }
        base += P.ints[l];
    }
    return cudaSuccess;
}

// One contiguous range of a checked SW batch: requests [base, base + n) of
// the caller's batch, whose CIGAR slots start at byte cig_base of the caller's
// buffer; `trace` is the whole batch's.  The finish callback gets the batch's
// own indices.  Transfer byte counts go to *h2d / *d2h.  `parts` ranges run
// at once and share the device-memory budget.
static int32_t sw_batch_range(const ga_sw_request* reqs, int32_t n, int64_t base, int64_t cig_base, bool trace,
                              const ga_tune& T, int64_t cell_limit, const SwFinish& fin, const char** err,
                              int64_t* h2d, int64_t* d2h, int parts, int range_tag, bool learned)
{
    *err = nullptr;
    if (n <= 0) return GA_OK;
    const ga_sw_scoring s0 = reqs[0].scoring;

    std::vector<int64_t> a_off(n), b_off(n), out_off(n), slot_end(n), pk_off(n);
    std::vector<uint8_t> own(n, 0);
    int64_t arena = 0, cig = 0, pkb = 0;
    SideSpan spa, spb;                          // where the own texts and patterns lie in the caller's memory
    for (int32_t i = 0; i < n; ++i) {
        const ga_sw_request& r = reqs[i];
        // a side that repeats the previous request's (same pointer and length:
        // one reference against many, or many against one) is staged once
        if (i > 0 && r.text == reqs[i - 1].text && r.text_len == reqs[i - 1].text_len) a_off[i] = a_off[i - 1];
        else { a_off[i] = arena; arena += round32(r.text_len); own[i] |= 1; spa.add(r.text, r.text_len); }
        if (i > 0 && r.pattern == reqs[i - 1].pattern && r.pattern_len == reqs[i - 1].pattern_len) b_off[i] = b_off[i - 1];
        else { b_off[i] = arena; arena += round32(r.pattern_len); own[i] |= 2; spb.add(r.pattern, r.pattern_len); }
        const int64_t cap = (int64_t)r.text_len + r.pattern_len;
        out_off[i] = cig; cig += cap;
        slot_end[i] = cig;
        pk_off[i] = pkb; pkb += (cap + 3) / 4;
    }
    arena += 64;
    if (!trace) cig = pkb = 0;
    // the own sides copied as the caller laid them out (two spans) and moved
    // into place on the device, or staged here
    const bool span = spa.ok && spb.ok && spa.bytes + spb.bytes >= SPAN_MIN_BYTES && pageable_direct();
    const int64_t span_a = span ? (int64_t)(spa.end - spa.first) : 0, span_b = span ? (int64_t)(spb.end - spb.first) : 0;

    Ctx* c = acquire_ctx(err, range_tag);
    if (!c) return GA_DEVICE_ERROR;
    struct Guard { Ctx* c; ~Guard() { release_ctx(c); } } guard{c};

    // Launch sizes from the lengths (bounds of the plan the device builds):
    // every launch is enqueued without reading the plan back.
    const bool route = learned && trace;                 // the SW model picks the 16-bit pairs
    const SwPlan P = bound_plan_sw(reqs, n, trace, trace ? cell_limit : -1, T, route);
    SwSlots S = size_sw(P, trace, T, c->sm_count, sw_dir_budget(c, parts));
    // Ranges that run beside others give their 16-bit persistent kernel three
    // quarters of the device's blocks: the next range's pack and plan kernels
    // then find room while this range runs, instead of waiting for its tail
    // (200,000-pair batch end to end: 30.2 -> 29.7 ms; half the blocks: 30.3).
    if (parts > 1 && S.s[SP_L16] > 0) S.s[SP_L16] = std::max(4, S.s[SP_L16] * 3 / 4 / 4 * 4);

    // Host staging: [descriptors (span offsets) | arena] in, [score pos len
    // checks err | packed CIGARs] back.  Device: the same blocks, then the CIGAR
    // slots, purity flags, the plan's work lists, its scratch and record,
    // counters, band edges, direction tables, the caller's spans.
    int64_t *ha, *hb, *ho, *hpo, *da, *db, *dout, *dpo, *hsa, *hsb, *dsa, *dsb;
    int32_t *hal, *hbl, *dal, *dbl, *hsc, *hpos, *hln, *dsc, *dpos, *dln, *her, *der;
    uint8_t *hseq, *dseq, *hvf, *dvf, *hpk, *dpk, *dspan_a, *dspan_b;
    char* dcg;
    auto io_layout = [&](Carve& k, int64_t** pa, int32_t** pal, int64_t** pb, int32_t** pbl, int64_t** po,
                         int64_t** ppo, int64_t** psa, int64_t** psb, uint8_t** ps, int32_t** psc, int32_t** ppos,
                         int32_t** pln, uint8_t** pvf, int32_t** per, uint8_t** ppk) {
        *pa = k.take<int64_t>(n); *pal = k.take<int32_t>(n);
        *pb = k.take<int64_t>(n); *pbl = k.take<int32_t>(n);
        *po = k.take<int64_t>(n); *ppo = k.take<int64_t>(n);
        *psa = k.take<int64_t>(span ? n : 0); *psb = k.take<int64_t>(span ? n : 0);
        *ps = k.take<uint8_t>(arena);
        *psc = k.take<int32_t>(n); *ppos = k.take<int32_t>(4 * (size_t)n);
        *pln = k.take<int32_t>(n); *pvf = k.take<uint8_t>(n);
        *per = k.take<int32_t>(1, 4);
        *ppk = k.take<uint8_t>((size_t)pkb, 4);
    };
    uint8_t *dpure, *dtry = nullptr;
    int32_t *dwork, *dscr, *dctr, *dedge;
    long long* dres;
    uint32_t* ddirs;
    float *dfeat = nullptr, *dy = nullptr;
    auto dev_layout = [&](char* base) {
        Carve k(base);
        io_layout(k, &da, &dal, &db, &dbl, &dout, &dpo, &dsa, &dsb, &dseq, &dsc, &dpos, &dln, &dvf, &der, &dpk);
        dcg = k.take<char>(cig + 1);
        dpure = k.take<uint8_t>(2 * (size_t)n);
        if (route) {
            dfeat = k.take<float>(66 * (size_t)n);
            dy = k.take<float>(2 * (size_t)n);
            dtry = k.take<uint8_t>((size_t)n);
        }
        dwork = k.take<int32_t>(2 * (size_t)n + 8);
        dscr = k.take<int32_t>((size_t)sw_plan_scratch_ints(n));
        dres = k.take<long long>(SP_RES);
        dctr = k.take<int32_t>(8, 4);
        dedge = k.take<int32_t>((size_t)S.max_slots * P.edge_slot);
        ddirs = (S.dir_words > 0) ? k.take<uint32_t>((size_t)S.dir_words) : nullptr;
        dspan_a = k.take<uint8_t>((size_t)span_a);
        dspan_b = k.take<uint8_t>((size_t)span_b);
        return k.off;
    };
    {
        Carve hk(nullptr);
        io_layout(hk, &ha, &hal, &hb, &hbl, &ho, &hpo, &hsa, &hsb, &hseq, &hsc, &hpos, &hln, &hvf, &her, &hpk);
        if (!ensure_host(c, hk.off)) { *err = E_HOSTMEM; return GA_DEVICE_ERROR; }
    }
    if (fail_here(1) || !ensure_dev(c, dev_layout(nullptr))) { *err = E_ALLOC; return GA_DEVICE_ERROR; }
    {
        Carve k(c->host);
        io_layout(k, &ha, &hal, &hb, &hbl, &ho, &hpo, &hsa, &hsb, &hseq, &hsc, &hpos, &hln, &hvf, &her, &hpk);
    }
    dev_layout(c->dev);
    parallel_for(n, 2048, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            const ga_sw_request& r = reqs[i];
            ha[i] = a_off[i]; hal[i] = r.text_len;
            hb[i] = b_off[i]; hbl[i] = r.pattern_len;
            ho[i] = out_off[i]; hpo[i] = pk_off[i];
            if (span) {
                hsa[i] = (own[i] & 1) && r.text_len > 0 ? (int64_t)((uintptr_t)r.text - spa.first) : -1;
                hsb[i] = (own[i] & 2) && r.pattern_len > 0 ? (int64_t)((uintptr_t)r.pattern - spb.first) : -1;
            } else {
                if ((own[i] & 1) && r.text_len) std::memcpy(hseq + a_off[i], r.text, (size_t)r.text_len);
                if ((own[i] & 2) && r.pattern_len) std::memcpy(hseq + b_off[i], r.pattern, (size_t)r.pattern_len);
            }
        }
    });
    if (!span) std::memset(hseq + arena - 64, 0, 64);
    // descriptors (+ the arena when staged here), contiguous; the spans from the caller's memory
    const size_t in_bytes = (size_t)((char*)(span ? hseq : hseq + arena) - c->host);
    *h2d = (int64_t)in_bytes + span_a + span_b;
    PairDesc D;
    D.packed = nullptr;
    D.n = n;
    D.seq = dseq; D.pure = dpure;
    D.a_off = da; D.a_len = dal; D.b_off = db; D.b_len = dbl; D.out_off = dout;
    if (fail_here(2) || cudaMemcpyAsync(c->dev, c->host, in_bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        (span_a > 0 && cudaMemcpyAsync(dspan_a, (const void*)spa.first, (size_t)span_a, cudaMemcpyHostToDevice,
                                       c->stream) != cudaSuccess) ||
        (span_b > 0 && cudaMemcpyAsync(dspan_b, (const void*)spb.first, (size_t)span_b, cudaMemcpyHostToDevice,
                                       c->stream) != cudaSuccess)) {
        cudaGetLastError();
        *err = E_H2D;
        return GA_DEVICE_ERROR;
    }
    // the device work: a fixed sequence for a given launch shape (no plan read
    // back), so it is captured once per shape and replayed as a CUDA graph
    auto enqueue = [&]() -> cudaError_t {
        cudaStream_t st = c->stream;
        // sentinel: too-large pairs keep score -1 (never written by a kernel)
        cudaError_t e = cudaMemsetAsync(dsc, 0xff, sizeof(int32_t) * (size_t)n, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(dpos, 0xff, sizeof(int32_t) * 4 * (size_t)n, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(dln, 0, sizeof(int32_t) * (size_t)n, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(der, 0, sizeof(int32_t), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(dctr, 0, sizeof(int32_t) * 8, st);
        if (e == cudaSuccess && span) e = launch_gather_sides(D, dseq, dspan_a, dspan_b, dsa, dsb, st);
        if (e == cudaSuccess && span) e = cudaMemsetAsync(dseq + arena - 64, 0, 64, st);
        if (e == cudaSuccess) e = launch_pack(D, arena, nullptr, dpure, st);
        if (e == cudaSuccess && route) e = launch_sw_route(D, s0.match, s0.gap_open, dfeat, dy, dtry, st);
        if (e == cudaSuccess)
            e = enqueue_plan_sw(D, s0, trace, trace ? cell_limit : -1, -1, dsc, dwork, dscr, dres, T, st, dtry);
        if (e == cudaSuccess)
            e = launch_plan(P, S, D, s0, trace, T, dwork, dsc, dpos, dln, dcg, ddirs, dedge, dctr, der, st, dscr, dres);
        if (e == cudaSuccess && trace)
            e = launch_sw_validate(D, ga_sw_scoring_t{s0.match, s0.mismatch, s0.gap_open, s0.gap_extend}, dsc, dpos,
                                   dln, dcg, dvf, st);
        if (e == cudaSuccess && trace) e = launch_cigar_pack(D, dln, dcg, dpo, dpk, st);
        return e;
    };
    cudaError_t le = cudaErrorLaunchFailure;
    if (!fail_here(3)) {
        if (profiling_on()) {
            le = enqueue();
        } else {
            const std::vector<uint64_t> key = {
                c->dev_gen, (uint64_t)n, (uint64_t)arena, (uint64_t)cig, (uint64_t)pkb,
                (uint64_t)trace | (uint64_t)route << 1 | (uint64_t)span << 2, (uint64_t)span_a, (uint64_t)span_b,
                (uint64_t)cell_limit,
                (uint64_t)(uint32_t)s0.match | (uint64_t)(uint32_t)s0.mismatch << 32,
                (uint64_t)(uint32_t)s0.gap_open | (uint64_t)(uint32_t)s0.gap_extend << 32,
                (uint64_t)T.sw_pack16 | (uint64_t)T.sw_window << 8 | (uint64_t)T.sw_long_log2 << 16 |
                    (uint64_t)T.sw_coop_log2 << 24 | (uint64_t)T.sw_opt16_pct << 32,
                (uint64_t)P.ints[0], (uint64_t)P.ints[1], (uint64_t)P.ints[2], (uint64_t)P.dir[0],
                (uint64_t)P.dir[1], (uint64_t)P.dir[2], (uint64_t)P.edge_slot, (uint64_t)P.max16_cells,
                (uint64_t)P.n_opt, (uint64_t)P.dir_opt, (uint64_t)S.dir_words, (uint64_t)S.max_slots,
                (uint64_t)S.s[0] | (uint64_t)S.s[1] << 32, (uint64_t)S.s[2] | (uint64_t)S.s_esc << 32};
            le = replay_graph(c->swexec, c->swkey, key, c->swlaunches, c->stream, enqueue);
        }
    }
    if (le != cudaSuccess) {
        cudaGetLastError();
        *err = E_LAUNCH;
        return GA_DEVICE_ERROR;
    }
    const size_t out_bytes = (size_t)((char*)(dpk + pkb) - (char*)dsc);
    *d2h = (int64_t)out_bytes;
    if (fail_here(4) || cudaMemcpyAsync(hsc, dsc, out_bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) {
        cudaGetLastError();
        *err = E_D2H;
        return GA_DEVICE_ERROR;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        *err = E_SYNC;
        return GA_DEVICE_ERROR;
    }
    if (*her != 0) { *err = (*her & ERR_SCRATCH) ? E_SCRATCH : E_OVERFLOW; return GA_DEVICE_ERROR; }
    if (trace && fail_here(5)) hln[0] = INT32_MAX;       // test hook: a length past its slot
    SwView v{hsc, hpos, hln, hpk, hpo, slot_end.data(), trace, trace ? hvf : nullptr, base, cig_base};
    std::atomic<bool> bad{false};
    parallel_for(n, 512, [&](int64_t lo, int64_t hi) {
        if (trace && !lengths_fit(hln, slot_end.data(), lo, hi)) { bad = true; return; }
        fin(base + lo, base + hi, v);
    });
    if (bad) { *err = E_BADLEN; return GA_DEVICE_ERROR; }
    return GA_OK;
}

int32_t sw_batch(const ga_sw_request* reqs, int32_t n, int64_t cell_limit, const SwFinish& fin,
                 const char** err, bool learned)
{
    learned = learned && sw_model_loaded();
    *err = nullptr;
    if (n <= 0) return GA_OK;
    if (int32_t st = sw_check(reqs, n, err)) return st;
    const ga_tune T = tune_current();
    // trace, the widest pattern and the cells, in one parallel pass
    struct Part { bool trace = false; int max_n = 0; double cells = 0.0; };
    std::vector<Part> part((size_t)((n + REQ_CHUNK - 1) / REQ_CHUNK + 1));
    const int64_t nch = for_chunks(n, [&](int64_t k, int64_t lo, int64_t hi) {
        Part& p = part[(size_t)k];
        for (int64_t i = lo; i < hi; ++i) {
            p.trace |= reqs[i].with_cigar != 0;
            p.max_n = std::max(p.max_n, (int)reqs[i].pattern_len);
            p.cells += (double)reqs[i].text_len * (double)reqs[i].pattern_len;
        }
    });
    bool trace = false;
    int max_n = 0;
    double cells = 0.0;
    for (int64_t k = 0; k < nch; ++k) {
        trace |= part[(size_t)k].trace;
        max_n = std::max(max_n, part[(size_t)k].max_n);
        cells += part[(size_t)k].cells;
    }
    // The reference's score-only kernel holds 4 warps x 2*(n+1) ints of shared
    // memory per block and refuses the batch above the per-block limit the
    // runtime reports, 48 KiB on CUDA devices (src/api/api.cpp:789-797).  The
    // drop-in entry keeps that limit; the extension entry passes cell_limit < 0.
    if (!trace && cell_limit >= 0 && (int64_t)4 * 2 * (max_n + 1) * 4 > 48 * 1024) {
        *err = E_SW_SMEM;
        return GA_INVALID_ARGUMENT;
    }
    // Large batches run as up to SW_CHUNKS contiguous ranges of about equal
    // cells (one per 2 Gcells), each on its own thread, context and stream:
    // one range's staging and copies, and its results' finish on the host,
    // overlap the others' kernels, whose blocks also fill the SMs a range's
    // tail leaves idle.  (200,000-pair batch end to end: 3 ranges 31.5 ms,
    // 4 30.9, 6 30.2, 8 30.0, 12 29.7.)
    constexpr int SW_CHUNKS = 12;
    const int K = n >= 8 * 1024 ? (int)std::max(1.0, std::min((double)SW_CHUNKS, cells / 2e9)) : 1;
    if (K == 1) return sw_batch_range(reqs, n, 0, 0, trace, T, cell_limit, fin, err, &t_h2d, &t_d2h, 1, -1, learned);
    int32_t cut[SW_CHUNKS + 1];
    int64_t cig_at[SW_CHUNKS + 1];
    cut[0] = 0;
    cig_at[0] = 0;
    {
        double acc = 0.0;
        int k = 1;
        int64_t cg = 0;
        for (int32_t i = 0; i < n && k < K; ++i) {
            acc += (double)reqs[i].text_len * (double)reqs[i].pattern_len;
            cg += (int64_t)reqs[i].text_len + reqs[i].pattern_len;
            if (acc >= cells * k / K) {
                cut[k] = i + 1;
                cig_at[k] = cg;
                ++k;
            }
        }
        for (; k < K; ++k) { cut[k] = n; cig_at[k] = cg; }
        cut[K] = n;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    int32_t st[SW_CHUNKS];
    const char* errs[SW_CHUNKS];
    int64_t h2d[SW_CHUNKS], d2h[SW_CHUNKS];
    auto run = [&](int k) {
        cudaSetDevice(dev);
        st[k] = sw_batch_range(reqs + cut[k], cut[k + 1] - cut[k], cut[k], cig_at[k], trace, T, cell_limit, fin,
                               &errs[k], &h2d[k], &d2h[k], K, k, learned);
    };
    PoolQuiet quiet;
    std::vector<std::thread> th;
    for (int k = 0; k + 1 < K; ++k) th.emplace_back(run, k);
    run(K - 1);
    for (std::thread& x : th) x.join();
    t_h2d = t_d2h = 0;
    for (int k = 0; k < K; ++k) {
        t_h2d += h2d[k];
        t_d2h += d2h[k];
    }
    for (int k = 0; k < K; ++k)
        if (st[k] != GA_OK) {
            *err = errs[k];
            return st[k];
        }
    return GA_OK;
}

// ------------------------------------------------------------ validators --
void wfa_validate(const char* cg, int len, int score, const char* P, int m, const char* T, int n,
                  bool* rescore_ok, bool* wellformed_ok)
{
    int cost = 0, pi = 0, ti = 0;
    bool ok = true;
    for (int q = 0; q < len; ++q) {
        const char op = cg[q];
        if (op == 'M' || op == 'X') {
            if (pi >= m || ti >= n || ((P[pi] == T[ti]) != (op == 'M'))) ok = false;
            cost += op == 'X';
            ++pi;
            ++ti;
        } else if (op == 'I') {
            ++ti;
            ++cost;
        } else if (op == 'D') {
            ++pi;
            ++cost;
        } else {
            ok = false;
        }
    }
    *wellformed_ok = ok && pi == m && ti == n;
    *rescore_ok = cost == score;
}

void sw_validate(const char* cg, int len, const char* T, int m, int si, int ei, const char* P, int n,
                 int sj, int ej, const ga_sw_scoring& sc, int score, bool* rescore_ok, bool* wellformed_ok)
{
    int i = si, j = sj, total = 0, gap = 0;   // gap > 0: run of I, < 0: run of D
    bool ok = true;
    auto close = [&] {
        if (gap) {
            const int L = gap > 0 ? gap : -gap;
            total -= sc.gap_open + (L - 1) * sc.gap_extend;
            gap = 0;
        }
    };
    for (int q = 0; q < len; ++q) {
        const char op = cg[q];
        if (op == 'M' || op == 'X') {
            close();
            if (i > ei || j > ej || i >= m || j >= n || ((T[i] == P[j]) != (op == 'M'))) ok = false;
            total += op == 'M' ? sc.match : sc.mismatch;
            ++i;
            ++j;
        } else if (op == 'I') {
            if (gap < 0) close();
            if (i > ei || i >= m) ok = false;
            ++i;
            ++gap;
        } else if (op == 'D') {
            if (gap > 0) close();
            if (j > ej || j >= n) ok = false;
            ++j;
            --gap;
        } else {
            ok = false;
        }
    }
    close();
    ok = ok && i == ei + 1 && j == ej + 1;
    *wellformed_ok = ok;
    *rescore_ok = ok && total == score;
}

// Sum of both sides' lengths (negative ones as 0) over a batch, in parallel chunks.
template <class R>
static int64_t side_bytes(const R* reqs, int32_t n)
{
    const int64_t nch = ((int64_t)n + REQ_CHUNK - 1) / REQ_CHUNK;
    std::vector<int64_t> part((size_t)std::max<int64_t>(nch, 1), 0);
    parallel_for(nch, 1, [&](int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) {
            int64_t s = 0;
            for (int64_t i = k * REQ_CHUNK, e = std::min<int64_t>(n, (k + 1) * REQ_CHUNK); i < e; ++i)
                s += std::max(0, reqs[i].text_len) + (int64_t)std::max(0, reqs[i].pattern_len);
            part[(size_t)k] = s;
        }
    });
    int64_t s = 0;
    for (int64_t k = 0; k < nch; ++k) s += part[(size_t)k];
    return s;
}

}  // namespace ga

// ================================================================== C ABI ==
using namespace ga;

extern "C" {

int64_t ga_align_cigar_bytes(const ga_align_request* reqs, int32_t n) { return side_bytes(reqs, n); }

int64_t ga_align_sw_cigar_bytes(const ga_sw_request* reqs, int32_t n) { return side_bytes(reqs, n); }

static void set_info(ga_batch_info* info, int32_t st, const char* e, int32_t res, int32_t unres)
{
    if (!info) return;
    info->status = st;
    info->error = e;
    info->resolved_count = res;
    info->unresolved_count = unres;
    info->reserved = 0;
}

int32_t ga_align_batch_ex(const ga_align_request* reqs, int32_t n, ga_align_result* results,
                          char* cigar_buf, int64_t cigar_buf_bytes, const ga_options* opt,
                          ga_batch_info* info)
{
    const ga_align_result dflt{-1, 0, 0, 0, 0, 0, 0};
    auto reset = [&] {
        parallel_for(n, 16384, [&](int64_t lo, int64_t hi) { std::fill(results + lo, results + hi, dflt); });
    };
    const int32_t max_smax =
        (opt && opt->max_smax > 0) ? std::min<int32_t>(opt->max_smax, GA_MAX_SMAX_DEVICE) : GA_MAX_SMAX;
    const char* err = nullptr;
    std::atomic<int32_t> resolved{0};
    auto fin = [&](int64_t lo, int64_t hi, const WfaView& v) {
        int32_t res = 0;
        for (int64_t i = lo; i < hi; ++i) {
            ga_align_result& r = results[i];
            const int64_t q = i - v.base;           // index in the range's outputs
            r = dflt;                               // every pair of the batch passes here once
            r.score = v.score[q];
            r.resolved = r.score >= 0;
            res += r.resolved;
            if (v.trace && r.resolved && v.len[q] > 0) {
                const int64_t at = v.cig_base + v.slot_end[q] - v.len[q];
                v.cigar(q, cigar_buf + at);
                r.cigar_offset = at;
                r.cigar_len = v.len[q];
                bool rs = false, wf = false;
                if (v.vflags) {
                    rs = v.vflags[q] & 1;
                    wf = (v.vflags[q] >> 1) & 1;
                } else {
                    wfa_validate(cigar_buf + at, v.len[q], r.score, reqs[i].pattern, reqs[i].pattern_len,
                                 reqs[i].text, reqs[i].text_len, &rs, &wf);
                }
                r.rescore_ok = rs;
                r.wellformed_ok = wf;
            }
        }
        resolved.fetch_add(res);
    };
    // the reference's request checks come first, then the buffer contract
    // (the CIGAR bytes the batch needs, ga_align_cigar_bytes), both in the
    // entry's first pass over the requests
    const int32_t st = wfa_batch(reqs, n, max_smax, opt ? opt->learned : 0, fin, &err,
                                 cigar_buf ? cigar_buf_bytes : -1);
    if (st != GA_OK) {
        reset();
        set_info(info, st, err, 0, 0);
        return st;
    }
    set_info(info, GA_OK, nullptr, resolved.load(), n - resolved.load());
    return GA_OK;
}

int32_t ga_align_batch(const ga_align_request* reqs, int32_t n, ga_align_result* results,
                       char* cigar_buf, int64_t cigar_buf_bytes, ga_batch_info* info)
{
    return ga_align_batch_ex(reqs, n, results, cigar_buf, cigar_buf_bytes, nullptr, info);
}

int32_t ga_align_sw_batch_ex(const ga_sw_request* reqs, int32_t n, ga_sw_result* results,
                             char* cigar_buf, int64_t cigar_buf_bytes, const ga_options* opt,
                             ga_batch_info* info)
{
    const ga_sw_result dflt{-1, 0, -1, -1, -1, -1, 0, 0, 0, 0, 0};
    int64_t limit = GA_SW_MAX_TRACE_CELLS;
    if (opt && opt->trace_cell_limit != 0) limit = opt->trace_cell_limit;
    // any CIGAR requested, and ga_align_sw_cigar_bytes, in one parallel pass
    std::vector<int64_t> need((size_t)((n + REQ_CHUNK - 1) / REQ_CHUNK + 1), 0);
    std::vector<uint8_t> want(need.size(), 0);
    const int64_t nch = for_chunks(n, [&](int64_t k, int64_t lo, int64_t hi) {
        int64_t s = 0;
        bool w = false;
        for (int64_t i = lo; i < hi; ++i) {
            w |= reqs[i].with_cigar != 0;
            s += std::max(0, reqs[i].text_len) + (int64_t)std::max(0, reqs[i].pattern_len);
        }
        need[(size_t)k] = s;
        want[(size_t)k] = w;
    });
    bool any_cigar = false;
    int64_t cig_need = 0;
    for (int64_t k = 0; k < nch; ++k) { cig_need += need[(size_t)k]; any_cigar |= want[(size_t)k] != 0; }
    const char* err = nullptr;
    std::atomic<int32_t> resolved{0};
    auto fin = [&](int64_t lo, int64_t hi, const SwView& v) {
        int32_t res = 0;
        for (int64_t i = lo; i < hi; ++i) {
            ga_sw_result& r = results[i];
            r = dflt;                               // every pair of the batch passes here once
            const int64_t q = i - v.base;           // index in the range's outputs
            const int s = v.score[q];
            if (s < 0) {                            // declared size limit
                if (v.trace) r.too_large = 1;
                continue;
            }
            r.score = s;
            r.resolved = 1;
            ++res;
            r.end_i = v.pos[4 * q + 2];
            r.end_j = v.pos[4 * q + 3];
            if (s == 0) { r.rescore_ok = r.wellformed_ok = 1; continue; }
            if (!v.trace || !reqs[i].with_cigar) continue;
            r.start_i = v.pos[4 * q];
            r.start_j = v.pos[4 * q + 1];
            const int len = v.len[q];
            if (len > 0) {
                const int64_t at = v.slot_end[q] - len;
                v.cigar(q, cigar_buf + v.cig_base + at);
                r.cigar_offset = v.cig_base + at;
                r.cigar_len = len;
                bool rs = false, wf = false;
                if (v.vflags) {
                    rs = v.vflags[q] & 1;
                    wf = (v.vflags[q] >> 1) & 1;
                } else {
                    sw_validate(cigar_buf + v.cig_base + at, len, reqs[i].text, reqs[i].text_len, r.start_i, r.end_i,
                                reqs[i].pattern, reqs[i].pattern_len, r.start_j, r.end_j, reqs[i].scoring, s,
                                &rs, &wf);
                }
                r.rescore_ok = rs;
                r.wellformed_ok = wf;
            }
        }
        resolved.fetch_add(res);
    };
    int32_t st;
    if (any_cigar && (cigar_buf == nullptr || cigar_buf_bytes < cig_need)) {
        st = sw_check(reqs, n, &err);
        if (st == GA_OK) { st = GA_INVALID_ARGUMENT; err = E_CIGBUF; }
    } else {
        st = sw_batch(reqs, n, limit, fin, &err, opt && opt->learned == 1);
    }
    if (st != GA_OK) {
        for (int32_t i = 0; i < n; ++i) results[i] = dflt;
        set_info(info, st, err, 0, 0);
        return st;
    }
    set_info(info, GA_OK, nullptr, resolved.load(), n - resolved.load());
    return GA_OK;
}

int32_t ga_align_sw_batch(const ga_sw_request* reqs, int32_t n, ga_sw_result* results, char* cigar_buf,
                          int64_t cigar_buf_bytes, ga_batch_info* info)
{
    return ga_align_sw_batch_ex(reqs, n, results, cigar_buf, cigar_buf_bytes, nullptr, info);
}

// ------------------------------------------------------ device-resident --
int32_t ga_wfa_device_ex(const ga_device_batch* b, int32_t smax, int32_t trace, const ga_options* opt,
                         int32_t* out_score, int32_t* out_len, char* out_cigar, void* stream, const char** err)
{
    const char* e = nullptr;
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
    const int route = route_mode(opt ? opt->learned : 0);
    const bool learned = route != 0;
    Ctx* c = acquire_ctx(&e);
    if (!c) { if (err) *err = e; return GA_DEVICE_ERROR; }
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    const ga_tune tuned = tune_current();
    WfaScratch S;
    size_wfa(S, b->n, smax, trace != 0, learned, c->sm_count, tuned.wfa_group);
    Carve k(nullptr);
    carve_wfa(k, S, b->n, b->seq_bytes, trace != 0, learned);
    k.take<int32_t>(1, 4);                                           // error word
    if (!ensure_dev(c, k.off)) { release_ctx(c); if (err) *err = E_ALLOC; return GA_DEVICE_ERROR; }
    Carve d(c->dev);
    carve_wfa(d, S, b->n, b->seq_bytes, trace != 0, learned);
    int32_t* derr = d.take<int32_t>(1, 4);
    PairDesc D;
    D.seq = b->seq; D.packed = nullptr; D.pure = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len;
    D.out_off = b->out_off; D.n = b->n;
    int32_t rc = GA_OK;
    cudaError_t le = cudaMemsetAsync(derr, 0, sizeof(int32_t), st);
    if (le == cudaSuccess) {
        const int lane_smax = tuned.wfa_lane_smax;
        if (learned && !profiling_on())
            le = run_wfa_graph(c, S, D, smax, trace != 0, route, lane_smax, out_score, out_len, out_cigar, derr, st);
        else le = enqueue_wfa(S, D, smax, trace != 0, route, lane_smax, out_score, out_len, out_cigar, derr, st);
        if (learned) note_route(c, S, b->n);
    }
    if (le != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = E_LAUNCH;
        rc = GA_DEVICE_ERROR;
    }
    if (stream) {
        cudaEventRecord(c->done, st);
        c->pending = true;
    } else if (cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = E_SYNC;
        rc = GA_DEVICE_ERROR;
    }
    release_ctx(c);
    return rc;
}

int32_t ga_wfa_route_stats(int32_t* out, int32_t max)
{
    const RouteRecord r = t_route;
    if (!r.c || !out || max < 2) return GA_INVALID_ARGUMENT;
    if (r.c->dev_gen != r.gen) return GA_INVALID_ARGUMENT;
    const int NB = route_buckets();
    std::vector<int32_t> counts(2 * NB + 4);
    int32_t esc[32];
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(counts.data(), r.counts, sizeof(int32_t) * (2 * NB + 4), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(esc, r.ctr + 32, sizeof(int32_t) * 32, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    out[0] = counts[2 * NB + 1];              // lane queue (one pair per lane)
    out[1] = counts[2 * NB];                  // warp queue (one pair per warp)
    int k = 2;
    if (k < max) out[k++] = esc[0];
    if (k < max) out[k++] = counts[2 * NB + 2];   // warp-queue pairs run on whole blocks
    for (; k < max; ++k) out[k] = 0;
    return GA_OK;
}

int32_t ga_wfa_route_items(int32_t* out, int32_t n)
{
    const RouteRecord r = t_route;
    if (!r.c || !out || n != r.n || r.c->dev_gen != r.gen) return GA_INVALID_ARGUMENT;
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(out, r.item, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

int32_t ga_wfa_device(const ga_device_batch* b, int32_t smax, int32_t trace, int32_t* out_score,
                      int32_t* out_len, char* out_cigar, void* stream, const char** err)
{
    return ga_wfa_device_ex(b, smax, trace, nullptr, out_score, out_len, out_cigar, stream, err);
}

int32_t ga_sw_device(const ga_device_batch* b, ga_sw_scoring sc, int32_t trace, int64_t cell_limit,
                     int32_t* out_score, int32_t* out_pos, int32_t* out_len, char* out_cigar, void* stream,
                     const char** err)
{
    return ga_sw_device_ex(b, sc, trace, cell_limit, nullptr, out_score, out_pos, out_len, out_cigar, stream, err);
}

int32_t ga_sw_device_ex(const ga_device_batch* b, ga_sw_scoring sc, int32_t trace, int64_t cell_limit,
                        const ga_options* opt, int32_t* out_score, int32_t* out_pos, int32_t* out_len,
                        char* out_cigar, void* stream, const char** err)
{
    const char* e = nullptr;
    if (!b || b->n < 0 || b->seq_bytes < 0 ||
        (b->n > 0 && (!b->seq || !b->a_off || !b->a_len || !b->b_off || !b->b_len || !out_score || !out_pos ||
                      (trace && (!out_len || !out_cigar || !b->out_off))))) {
        if (err) *err = "invalid device batch";
        return GA_INVALID_ARGUMENT;
    }
    if (b->n == 0) return GA_OK;
    const int32_t n = b->n;
    Ctx* c = acquire_ctx(&e);
    if (!c) { if (err) *err = e; return GA_DEVICE_ERROR; }
    struct Guard { Ctx* c; ~Guard() { release_ctx(c); } } guard{c};
    auto fail = [&](const char* msg) {
        cudaGetLastError();
        if (err) *err = msg;
        return GA_DEVICE_ERROR;
    };
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    const ga_tune T = tune_current();
    // the SW model picks the pairs the 16-bit kernel tries (traceback)
    const bool route = trace && opt && opt->learned == 1 && sw_model_loaded();
    float *dfeat = nullptr, *dy = nullptr;
    uint8_t* dtry = nullptr;
    // purity and the plan on the device, then the launches
    auto plan_layout = [&](char* base, uint8_t** pp, int32_t** scr, int32_t** wk, long long** res) {
        Carve k(base);
        *pp = k.take<uint8_t>(2 * (size_t)n);
        *scr = k.take<int32_t>((size_t)sw_plan_scratch_ints(n));
        *wk = k.take<int32_t>(2 * (size_t)n + 8);
        *res = k.take<long long>(SP_RES);
        if (route) {
            dfeat = k.take<float>(66 * (size_t)n);
            dy = k.take<float>(2 * (size_t)n);
            dtry = k.take<uint8_t>((size_t)n);
        }
        return k.off;
    };
    uint8_t* dpure;
    int32_t *dscr, *dwork;
    long long* dres;
    const size_t plan_bytes = plan_layout(nullptr, &dpure, &dscr, &dwork, &dres);
    if (!ensure_dev(c, plan_bytes + 4096) || !ensure_host(c, sizeof(long long) * SP_RES + 256)) return fail(E_ALLOC);
    long long* hres = reinterpret_cast<long long*>(c->host);
    int32_t* herr = reinterpret_cast<int32_t*>(c->host + sizeof(long long) * SP_RES);
    PairDesc D;
    D.seq = b->seq; D.packed = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len;
    D.out_off = b->out_off; D.n = n;

    // A synchronous traceback call with a cell limit replays the CUDA graph of
    // its launch shape: the first call of a shape reads the plan back to size
    // the per-warp memory and captures the launches in plan mode (sizes read
    // on the device); a replay whose plan needs more memory than that (the
    // pairs behind the same pointers grew) is flagged by the kernels
    // (ERR_SCRATCH) and runs again through the read-back path.
    const bool graph = !stream && trace && cell_limit >= 0 && !profiling_on();
    std::vector<uint64_t> key;
    if (graph) {
        key = {0x5357445645ull, (uint64_t)n, (uint64_t)(uintptr_t)b->seq, (uint64_t)b->seq_bytes,
               (uint64_t)(uintptr_t)b->a_off, (uint64_t)(uintptr_t)b->a_len, (uint64_t)(uintptr_t)b->b_off,
               (uint64_t)(uintptr_t)b->b_len, (uint64_t)(uintptr_t)b->out_off, (uint64_t)(uintptr_t)out_score,
               (uint64_t)(uintptr_t)out_pos, (uint64_t)(uintptr_t)out_len, (uint64_t)(uintptr_t)out_cigar,
               (uint64_t)(uint32_t)sc.match | (uint64_t)(uint32_t)sc.mismatch << 32,
               (uint64_t)(uint32_t)sc.gap_open | (uint64_t)(uint32_t)sc.gap_extend << 32, (uint64_t)cell_limit,
               (uint64_t)T.sw_pack16 | (uint64_t)T.sw_window << 8 | (uint64_t)T.sw_long_log2 << 16 |
                   (uint64_t)T.sw_coop_log2 << 24 | (uint64_t)T.sw_opt16_pct << 32 | (uint64_t)route << 40};
        if (c->swexec && c->swkey.size() == key.size() + 2 && std::equal(key.begin(), key.end(), c->swkey.begin()) &&
            c->swkey[key.size()] == c->dev_gen) {
            int32_t* derr = reinterpret_cast<int32_t*>(c->swkey[key.size() + 1]);
            note_graph_launches(c->swlaunches);
            if (cudaGraphLaunch(c->swexec, st) != cudaSuccess ||
                cudaMemcpyAsync(herr, derr, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return fail(E_SYNC);
            if (!(*herr & ERR_SCRATCH)) return *herr ? fail(E_OVERFLOW) : GA_OK;
            cudaGraphExecDestroy(c->swexec);           // sized for smaller pairs: plan again below
            c->swexec = nullptr;
            c->swkey.clear();
        }
    }

    cudaMemsetAsync(out_score, 0xff, sizeof(int32_t) * n, st);
    cudaMemsetAsync(out_pos, 0xff, sizeof(int32_t) * 4 * (size_t)n, st);
    if (out_len) cudaMemsetAsync(out_len, 0, sizeof(int32_t) * n, st);
    SwPlan P;
    auto plan = [&]() {
        plan_layout(c->dev, &dpure, &dscr, &dwork, &dres);
        D.pure = dpure;
        if (launch_pack(D, b->seq_bytes, nullptr, dpure, st) != cudaSuccess) return false;
        if (route && launch_sw_route(D, sc.match, sc.gap_open, dfeat, dy, dtry, st) != cudaSuccess) return false;
        return device_plan_sw(D, sc, trace != 0, cell_limit, -2, out_score, dwork, dscr, dres, hres, T, st, P, dtry) ==
               cudaSuccess;
    };
    if (!plan()) return fail(E_LAUNCH);
    const SwSlots S = size_sw(P, trace != 0, T, c->sm_count, sw_dir_budget(c, 1));
    auto run_layout = [&](char* base, int32_t** ctr, int32_t** edge, uint32_t** dirs) {
        Carve k(base);
        k.off = plan_bytes;
        *ctr = k.take<int32_t>(64, 256);
        *edge = k.take<int32_t>((size_t)S.max_slots * P.edge_slot);
        *dirs = k.take<uint32_t>((size_t)S.dir_words);
        return k.off;
    };
    int32_t *dctr, *dedge;
    uint32_t* ddirs;
    const uint64_t gen_before = c->dev_gen;
    if (!ensure_dev(c, run_layout(nullptr, &dctr, &dedge, &ddirs))) return fail(E_ALLOC);
    if (c->dev_gen != gen_before && !plan()) return fail(E_LAUNCH);      // the arena moved: plan again in the new one
    run_layout(c->dev, &dctr, &dedge, &ddirs);
    if (graph) {
        // the launches of this shape in plan mode, captured with the memsets,
        // the purity pass and the planner, then replayed (this call included)
        auto enqueue = [&]() -> cudaError_t {
            cudaError_t x = cudaMemsetAsync(out_score, 0xff, sizeof(int32_t) * n, st);
            if (x == cudaSuccess) x = cudaMemsetAsync(out_pos, 0xff, sizeof(int32_t) * 4 * (size_t)n, st);
            if (x == cudaSuccess) x = cudaMemsetAsync(out_len, 0, sizeof(int32_t) * n, st);
            if (x == cudaSuccess) x = cudaMemsetAsync(dctr, 0, 64 * sizeof(int32_t), st);
            if (x == cudaSuccess) x = launch_pack(D, b->seq_bytes, nullptr, dpure, st);
            if (x == cudaSuccess && route) x = launch_sw_route(D, sc.match, sc.gap_open, dfeat, dy, dtry, st);
            if (x == cudaSuccess)
                x = enqueue_plan_sw(D, sc, true, cell_limit, -2, out_score, dwork, dscr, dres, T, st, dtry);
            if (x == cudaSuccess)
                x = launch_plan(P, S, D, sc, true, T, dwork, out_score, out_pos, out_len, out_cigar, ddirs, dedge, dctr,
                                dctr + 32, st, dscr, dres);
            return x;
        };
        std::vector<uint64_t> full = key;
        full.push_back(c->dev_gen);
        full.push_back((uint64_t)(uintptr_t)(dctr + 32));
        if (replay_graph(c->swexec, c->swkey, full, c->swlaunches, st, enqueue) != cudaSuccess ||
            cudaMemcpyAsync(herr, dctr + 32, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return fail(E_SYNC);
        return *herr ? fail((*herr & ERR_SCRATCH) ? E_SCRATCH : E_OVERFLOW) : GA_OK;
    }
    cudaMemsetAsync(dctr, 0, 64 * sizeof(int32_t), st);
    if (launch_plan(P, S, D, sc, trace != 0, T, dwork, out_score, out_pos, out_len, out_cigar, ddirs, dedge, dctr,
                    dctr + 32, st, dscr) != cudaSuccess)
        return fail(E_LAUNCH);
    if (stream) {
        cudaEventRecord(c->done, st);
        c->pending = true;
    } else if (cudaStreamSynchronize(st) != cudaSuccess) {
        return fail(E_SYNC);
    }
    return GA_OK;
}

// ------------------------------------------------------------ provenance --
const char* ga_backend_name(void) { return "cuda-sm_103a"; }

const char* ga_device_name(void)
{
    static std::once_flag once;
    static char name[256] = "none";
    std::call_once(once, [] {
        int n = 0;
        if (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) {
            cudaDeviceProp p;
            if (cudaGetDeviceProperties(&p, 0) == cudaSuccess) std::snprintf(name, sizeof(name), "%s", p.name);
        }
        cudaGetLastError();
    });
    return name;
}

int32_t ga_wfa_validate_device(const ga_device_batch* b, const int32_t* score, const int32_t* len, const char* cigar,
                               uint8_t* flags, void* stream)
{
    if (!b || b->n < 0 || (b->n > 0 && (!b->seq || !b->a_off || !b->a_len || !b->b_off || !b->b_len ||
                                         !b->out_off || !score || !len || !cigar || !flags)))
        return GA_INVALID_ARGUMENT;
    PairDesc D;
    D.seq = b->seq; D.packed = nullptr; D.pure = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len;
    D.out_off = b->out_off; D.n = b->n;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = launch_wfa_validate(D, score, len, cigar, flags, st);
    if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

int32_t ga_sw_validate_device(const ga_device_batch* b, ga_sw_scoring sc, const int32_t* score, const int32_t* pos,
                              const int32_t* len, const char* cigar, uint8_t* flags, void* stream)
{
    if (!b || b->n < 0 || (b->n > 0 && (!b->seq || !b->a_off || !b->a_len || !b->b_off || !b->b_len ||
                                         !b->out_off || !score || !pos || !len || !cigar || !flags)))
        return GA_INVALID_ARGUMENT;
    PairDesc D;
    D.seq = b->seq; D.packed = nullptr; D.pure = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len;
    D.out_off = b->out_off; D.n = b->n;
    const ga_sw_scoring_t s{sc.match, sc.mismatch, sc.gap_open, sc.gap_extend};
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = launch_sw_validate(D, s, score, pos, len, cigar, flags, st);
    if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

int32_t ga_pack_2bit_device(const uint8_t* seq, int64_t seq_bytes, uint64_t* packed, uint32_t* mask, void* stream)
{
    if (seq_bytes < 0 || (seq_bytes & 31) != 0 || (seq_bytes > 0 && (!seq || !packed || !mask)) ||
        ((uintptr_t)seq & 15) != 0)
        return GA_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = launch_pack_arena(seq, seq_bytes, packed, mask, st);
    if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

int32_t ga_device_available(void)
{
    int n = 0;
    const bool ok = cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
    cudaGetLastError();
    return ok ? 1 : 0;
}

int64_t ga_kernel_launches(void) { return g_launches.load(); }

void ga_last_transfer_bytes(int64_t* h2d, int64_t* d2h)
{
    if (h2d) *h2d = t_h2d;
    if (d2h) *d2h = t_d2h;
}

void ga_profile(int32_t on)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (on) {
        for (int k = 0; k < K_COUNT; ++k) { g_prof_ms[k] = 0; g_prof_n[k] = 0; }
        g_prof_done.clear();
    }
    g_prof_on = on != 0;
}

int32_t ga_profile_read(int32_t kernel_id, double* total_ms, int64_t* launches)
{
    if (kernel_id < 0 || kernel_id >= K_COUNT) return GA_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (ProfRec& r : g_prof_done) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            g_prof_ms[r.id] += ms;
            g_prof_n[r.id] += 1;
        }
        cudaGetLastError();
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    g_prof_done.clear();
    if (total_ms) *total_ms = g_prof_ms[kernel_id];
    if (launches) *launches = g_prof_n[kernel_id];
    return GA_OK;
}

const char* ga_profile_kernel_name(int32_t kernel_id)
{
    static const char* names[K_COUNT] = {"pack2", "wfa_score", "wfa_trace", "wfa_lane", "wfa_routed",
                                         "sw32_score", "sw32_trace", "sw16x2_trace", "sw16x2_score", "sw_plan",
                                         "validate", "gene_qc", "int_peak", "kmer_sketch", "mlp", "route"};
    return (kernel_id >= 0 && kernel_id < K_COUNT) ? names[kernel_id] : nullptr;
}

void ga_debug_fail_next(int32_t step) { g_fail_next.store(step); }

}  // extern "C"
