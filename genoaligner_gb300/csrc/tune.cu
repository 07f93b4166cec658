// tune.cu -- the autotuner: per-device kernel settings and the search that
// picks them by timing candidates on a caller's batch.
//
// A setting (ga_tune) chooses how work is laid onto the GPU -- 16-bit pairs
// two per warp (inter-sequence) or one per warp in 32 bits (intra-sequence),
// the traceback window's tile count and so its lanes and columns per tile, the
// cell count where 32-bit pairs switch to the long tile shape, which
// learned-WFA pairs run one per lane and how many lanes the others get -- and
// never what is computed: every
// kernel variant gives the same results.  The search is coordinate-wise: one
// field at a time over its candidates, the others held at the best so far,
// each candidate timed end to end through the public device entry (one
// untimed call, then `reps` timed ones).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "route.cuh"
#include "tune.hpp"

namespace ga {

constexpr int MAX_DEV = 64;
static std::mutex g_tune_mu;
static ga_tune g_tune[MAX_DEV];
static bool g_tune_has[MAX_DEV];
static thread_local const ga_tune* t_candidate = nullptr;

static ga_tune builtin()
{
    ga_tune t;
    std::memset(&t, 0, sizeof(t));
    t.sw_pack16 = 1;
    t.sw_window = CK_TG;
    t.sw_long_log2 = C32_LONG_LOG2;
    t.wfa_lane_smax = LANE_SMAX;
    t.sw_coop_log2 = C32_COOP_LOG2;
    t.sw_opt16_pct = 100;
    t.wfa_group = 16;
    return t;
}

static bool valid(const ga_tune& t)
{
    return (t.sw_pack16 == 0 || t.sw_pack16 == 1) && (t.sw_window == 2 || t.sw_window == 4) &&
           t.sw_long_log2 >= 16 && t.sw_long_log2 <= 30 && t.wfa_lane_smax >= 0 && t.wfa_lane_smax <= LANE_SMAX &&
           t.sw_coop_log2 >= 16 && t.sw_coop_log2 <= 40 && t.sw_opt16_pct >= 50 && t.sw_opt16_pct <= 100 &&
           (t.wfa_group == 8 || t.wfa_group == 16 || t.wfa_group == 32);
}

static bool same(const ga_tune& a, const ga_tune& b)
{
    return a.sw_pack16 == b.sw_pack16 && a.sw_window == b.sw_window && a.sw_long_log2 == b.sw_long_log2 &&
           a.wfa_lane_smax == b.wfa_lane_smax && a.sw_coop_log2 == b.sw_coop_log2 &&
           a.sw_opt16_pct == b.sw_opt16_pct && a.wfa_group == b.wfa_group;
}

static int current_device()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return dev;
}

ga_tune tune_current()
{
    if (t_candidate) return *t_candidate;
    const int dev = current_device();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (dev >= 0 && dev < MAX_DEV && g_tune_has[dev]) return g_tune[dev];
    return builtin();
}

static bool store(int dev, const ga_tune& t)
{
    if (dev < 0 || dev >= MAX_DEV || !valid(t)) return false;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[dev] = t;
    std::memset(g_tune[dev].reserved, 0, sizeof(g_tune[dev].reserved));
    g_tune_has[dev] = true;
    return true;
}

// Times one candidate: `run` is one synchronous call of the public entry.
template <typename Run>
static int32_t time_candidate(const ga_tune& cand, int reps, const Run& run, double* ms, const char** err)
{
    t_candidate = &cand;
    int32_t rc = run(err);                                      // untimed: allocations, graph capture
    double total = 0.0;
    for (int r = 0; r < reps && rc == GA_OK; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        rc = run(err);
        total += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    t_candidate = nullptr;
    *ms = reps > 0 ? total / reps : 0.0;
    return rc;
}

struct Search {
    ga_tune best;
    double best_ms = 1e300;
    std::vector<ga_tune_trial> trials;
};

// One coordinate: every value of field `f` in `vals`, the rest at S.best.
template <typename Run>
static int32_t sweep(Search& S, int32_t ga_tune::*f, const std::vector<int>& vals, int reps, const Run& run,
                     const char** err)
{
    const ga_tune base = S.best;
    ga_tune pick = base;
    double pick_ms = 1e300;
    for (int v : vals) {
        ga_tune cand = base;
        cand.*f = v;
        double ms = 0.0;
        bool seen = false;
        for (const ga_tune_trial& tr : S.trials)
            if (same(tr.tune, cand)) { ms = tr.ms; seen = true; }
        if (!seen) {
            const int32_t rc = time_candidate(cand, reps, run, &ms, err);
            if (rc != GA_OK) return rc;
            S.trials.push_back(ga_tune_trial{cand, ms});
        }
        if (ms < pick_ms) { pick_ms = ms; pick = cand; }
    }
    S.best = pick;
    S.best_ms = pick_ms;
    return GA_OK;
}

static void report(const Search& S, ga_tune* chosen, ga_tune_trial* trials, int32_t max_trials, int32_t* n_trials)
{
    if (chosen) *chosen = S.best;
    int32_t k = 0;
    for (const ga_tune_trial& tr : S.trials) {
        if (trials && k < max_trials) trials[k] = tr;
        ++k;
    }
    if (n_trials) *n_trials = std::min(k, trials ? max_trials : k);
}

}  // namespace ga

using namespace ga;

extern "C" {

int32_t ga_tune_default(ga_tune* out)
{
    if (!out) return GA_INVALID_ARGUMENT;
    *out = builtin();
    return GA_OK;
}

int32_t ga_tune_get(ga_tune* out)
{
    if (!out) return GA_INVALID_ARGUMENT;
    *out = tune_current();
    return GA_OK;
}

int32_t ga_tune_set(const ga_tune* t)
{
    if (!t || !valid(*t)) return GA_INVALID_ARGUMENT;
    return store(current_device(), *t) ? GA_OK : GA_DEVICE_ERROR;
}

int32_t ga_autotune_sw(const ga_device_batch* batch, ga_sw_scoring scoring, int64_t trace_cell_limit,
                       int32_t* out_score, int32_t* out_pos, int32_t* out_len, char* out_cigar, int32_t reps,
                       ga_tune* chosen, ga_tune_trial* trials, int32_t max_trials, int32_t* n_trials,
                       const char** err)
{
    if (err) *err = nullptr;
    if (!batch || batch->n <= 0) {
        if (err) *err = "autotuning needs a non-empty batch";
        return GA_INVALID_ARGUMENT;
    }
    const int dev = current_device();
    if (dev < 0 || dev >= MAX_DEV) {
        if (err) *err = "no CUDA device is available";
        return GA_DEVICE_ERROR;
    }
    if (reps <= 0) reps = 2;
    // the largest pair decides whether the long-shape threshold matters
    const int n = batch->n;
    std::vector<int32_t> al(n), bl(n);
    if (cudaMemcpy(al.data(), batch->a_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(bl.data(), batch->b_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        if (err) *err = "device-to-host copy failed";
        return GA_DEVICE_ERROR;
    }
    int64_t max_cells = 0;
    int max_min_len = 0;
    for (int i = 0; i < n; ++i) {
        max_cells = std::max<int64_t>(max_cells, (int64_t)std::max(al[i], 0) * std::max(bl[i], 0));
        max_min_len = std::max(max_min_len, std::min(al[i], bl[i]));
    }
    auto run = [&](const char** e) {
        return ga_sw_device(batch, scoring, 1, trace_cell_limit, out_score, out_pos, out_len, out_cigar, nullptr, e);
    };
    // coordinate search from the built-in SW setting (the WFA field kept),
    // repeated once when the first pass moved: a field swept early (the
    // variant) is then judged again at the later fields' best values
    Search S;
    S.best = tune_current();
    {
        const ga_tune d = builtin();
        S.best.sw_pack16 = d.sw_pack16; S.best.sw_window = d.sw_window; S.best.sw_long_log2 = d.sw_long_log2;
        S.best.sw_coop_log2 = d.sw_coop_log2; S.best.sw_opt16_pct = d.sw_opt16_pct;
    }
    auto pass = [&]() -> int32_t {
        int32_t rc = sweep(S, &ga_tune::sw_pack16, {1, 0}, reps, run, err);
        if (rc == GA_OK && S.best.sw_pack16) rc = sweep(S, &ga_tune::sw_window, {2, 4}, reps, run, err);
        if (rc == GA_OK && max_cells > ((int64_t)1 << 20)) {
            std::vector<int> vals;
            for (int v = 20; v <= 28; v += 2)
                if (max_cells > ((int64_t)1 << v) || v == 20) vals.push_back(v);
            vals.push_back(30);                                   // no pair in the long shape
            rc = sweep(S, &ga_tune::sw_long_log2, vals, reps, run, err);
        }
        if (rc == GA_OK && max_cells > ((int64_t)1 << 24)) {
            std::vector<int> vals;
            for (int v = 24; v <= 30; v += 3)
                if (max_cells > ((int64_t)1 << v)) vals.push_back(v);
            vals.push_back(40);                                   // every pair on one warp
            rc = sweep(S, &ga_tune::sw_coop_log2, vals, reps, run, err);
        }
        if (rc == GA_OK && S.best.sw_pack16 && max_min_len > 0 &&
            (int64_t)scoring.match * max_min_len + BIAS16 + scoring.gap_open >= 32000)
            rc = sweep(S, &ga_tune::sw_opt16_pct, {100, 85, 75, 65}, reps, run, err);
        return rc;
    };
    const ga_tune start = S.best;
    int32_t rc = pass();
    if (rc == GA_OK && !same(start, S.best)) rc = pass();
    if (rc != GA_OK) return rc;
    store(dev, S.best);
    report(S, chosen, trials, max_trials, n_trials);
    // leave the batch's results in the outputs, computed with the kept setting
    return run(err);
}

int32_t ga_autotune_wfa(const ga_device_batch* batch, int32_t smax, int32_t trace, int32_t* out_score,
                        int32_t* out_len, char* out_cigar, int32_t reps, ga_tune* chosen, ga_tune_trial* trials,
                        int32_t max_trials, int32_t* n_trials, const char** err)
{
    if (err) *err = nullptr;
    if (!batch || batch->n <= 0) {
        if (err) *err = "autotuning needs a non-empty batch";
        return GA_INVALID_ARGUMENT;
    }
    if (!cost_model_loaded()) {
        if (err) *err = "the learned WFA path needs a cost model (ga_cost_model_set)";
        return GA_INVALID_ARGUMENT;
    }
    const int dev = current_device();
    if (dev < 0 || dev >= MAX_DEV) {
        if (err) *err = "no CUDA device is available";
        return GA_DEVICE_ERROR;
    }
    if (reps <= 0) reps = 2;
    ga_options opt;
    std::memset(&opt, 0, sizeof(opt));
    opt.learned = 1;
    opt.max_smax = 1 << 20;
    auto run = [&](const char** e) {
        return ga_wfa_device_ex(batch, smax, trace, &opt, out_score, out_len, out_cigar, nullptr, e);
    };
    Search S;
    S.best = tune_current();
    int32_t rc = sweep(S, &ga_tune::wfa_lane_smax, {0, 8, 15, 23, LANE_SMAX}, reps, run, err);
    if (rc == GA_OK && routed_group(smax, 8) == 8) rc = sweep(S, &ga_tune::wfa_group, {32, 16, 8}, reps, run, err);
    if (rc != GA_OK) return rc;
    store(dev, S.best);
    report(S, chosen, trials, max_trials, n_trials);
    return run(err);
}

int32_t ga_tune_save(const char* path)
{
    if (!path) return GA_INVALID_ARGUMENT;
    std::vector<std::pair<int, ga_tune>> rows;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (int d = 0; d < MAX_DEV; ++d)
            if (g_tune_has[d]) rows.push_back({d, g_tune[d]});
    }
    FILE* f = std::fopen(path, "w");
    if (!f) return GA_INVALID_ARGUMENT;
    std::fprintf(f, "# genoaligner_gb300 tune v4: device name <TAB> sw_pack16 sw_window sw_long_log2 wfa_lane_smax "
                    "sw_coop_log2 sw_opt16_pct wfa_group\n");
    for (const auto& r : rows) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, r.first) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        std::fprintf(f, "%s\t%d %d %d %d %d %d %d\n", p.name, r.second.sw_pack16, r.second.sw_window,
                     r.second.sw_long_log2, r.second.wfa_lane_smax, r.second.sw_coop_log2, r.second.sw_opt16_pct,
                     r.second.wfa_group);
    }
    return std::fclose(f) == 0 ? GA_OK : GA_INVALID_ARGUMENT;
}

int32_t ga_tune_load(const char* path)
{
    if (!path) return GA_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "r");
    if (!f) return GA_INVALID_ARGUMENT;
    std::vector<std::pair<std::string, ga_tune>> rows;
    char line[512];
    bool ok = true;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        char* tab = std::strchr(line, '\t');
        ga_tune t = builtin();
        // six fields (files written before wfa_group existed: the built-in group) or seven
        const int got = tab ? std::sscanf(tab + 1, "%d %d %d %d %d %d %d", &t.sw_pack16, &t.sw_window,
                                          &t.sw_long_log2, &t.wfa_lane_smax, &t.sw_coop_log2, &t.sw_opt16_pct,
                                          &t.wfa_group)
                            : 0;
        if ((got != 6 && got != 7) || !valid(t)) {
            ok = false;
            break;
        }
        rows.push_back({std::string(line, tab), t});
    }
    std::fclose(f);
    if (!ok) return GA_INVALID_ARGUMENT;
    const int dev = current_device();
    if (dev < 0) return GA_OK;                       // nothing to apply without a device
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
        cudaGetLastError();
        return GA_OK;
    }
    for (const auto& r : rows)
        if (r.first == p.name) store(dev, r.second);
    return GA_OK;
}

}  // extern "C"
