// group.cu -- grouped real-field transforms of many functions of uneven bandwidth.
//
// A group fixes a list of functions (function f has bandwidth bw[f]: any bandwidth of the split
// path, i.e. 16 .. 256 or a power of two up to 512, at most 16 distinct ones) and a split
// precision.  Functions are binned by bandwidth into classes; each class owns class-contiguous
// intermediate arrays (split_layout).  One transform runs as
//   forward : the phi-DFT of the classes (FST_semi_memo.c:81-90), then their weighted DCT-II
//             (seminaive.c:161-176), then ONE persistent tcgen05 contraction launch over the work
//             items of every class (seminaive.c:183-197);
//   inverse : ONE persistent contraction launch (seminaive.c:74-98), then the DCT-III with the
//             naive-order recombination, then the DFT over the orders (FST_semi_memo.c:334-350).
// Each FFT stage of the power-of-two classes is a grouped launch (k_stage_group: a block decodes
// its class and runs that class's transform length) over a tier of classes: the short transforms
// (bw <= 64), compiled for the per-length kernels' small register budgets, and the long ones
// (bw >= 128).  The two tiers run concurrently on two streams, so those classes take at most two
// launches per stage whatever their number.  A class of another bandwidth (transform length 32 R
// with R not a power of two, or a chirp-z length) runs each stage as its own launch on the
// long tier's stream.  The sequence is captured once as a CUDA graph (on an internal stream, the tiers as
// parallel branches) and replayed on the caller's stream; the first call with a given set of
// pointers runs eagerly and captures, later calls replay.
//
// Shapes (the N extent of each class's contraction tile, the depth of the contraction's table-copy
// ring, resident blocks per SM the DCT stages are sized for) come from an autotuner that
// times the group's whole forward + inverse sequence on its own sizes and keeps the fastest;
// results are cached per (device, precision, class sizes) in memory and, when $S2G_TUNE_CACHE
// names a file, on disk.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "s2g_internal.h"

namespace s2g {

static constexpr int kGroupMaxClasses = 16;

// Bandwidths whose FFT stages the grouped stage kernel runs (transform lengths 32 R, R a power of two).
static bool stage_groupable(int B) { return B >= 16 && B <= 512 && (B & (B - 1)) == 0; }

struct GroupClass {
    int B = 0, N = 0, NB = 0;
    Tables* t = nullptr;
    std::vector<int> funcs;     // member functions, in the caller's order
    int64_t* gmap = nullptr;    // device: member i -> grid offset (elements)
    int64_t* cmap = nullptr;    // device: member i -> coefficient offset
    float* buf0 = nullptr;      // X (forward) / F (inverse): [2][N][B][SX]  (split_layout)
    float* buf1 = nullptr;      // C (forward) / Fc (inverse): [2][N][B][2 BH]
};

struct GroupGraph {
    cudaGraphExec_t exec = nullptr;
    const void* ptr[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    unsigned long long kernels = 0;
};

}  // namespace s2g

struct s2g_group_s {
    int device = -1, precision = 0, nfunc = 0;
    std::vector<int> bw;
    std::vector<int64_t> goff, coff;
    int64_t grid_total = 0, coef_total = 0;
    std::vector<s2g::GroupClass> cls;
    void* mem = nullptr;        // one device allocation: maps, intermediates, counters
    int* counters = nullptr;    // [0] forward, [1] inverse contraction work counters
    int table_stages = 0;       // contraction: table-copy ring depth, 0 = as many as fit
    int dct_ctas = 0;           // DCT stages: resident blocks per SM they are sized for, 0 = as many as fit
    cudaStream_t cap = nullptr;
    cudaStream_t side = nullptr;               // the short-transform tier's stream
    cudaEvent_t fork = nullptr, join = nullptr;
    s2g::GroupGraph graphs[3];  // forward, inverse, forward+inverse
    std::string tuning;         // description of the chosen tile shapes
};

namespace s2g {

// ---- launch sequences (eager or under capture) ----

// Short transforms (bw <= 64) form one tier of the FFT stages, the rest the other.
static constexpr int kShortTierMaxBw = 64;

// FFT stage `which` of every class, from in(c) to out(c): the long tier on st, the short tier on the
// side stream (forked from and joined back into st).
template <typename In, typename Out>
static int group_stages(s2g_group g, const int* which, int nstage, In in, Out out, cudaStream_t st) {
    const int nc = (int)g->cls.size();
    StageSpec lo[kGroupMaxClasses], hi[kGroupMaxClasses];
    int nlo = 0, nhi = 0;
    for (int w = 0; w < nstage; ++w) {
        nlo = nhi = 0;
        for (int c = 0; c < nc; ++c) {
            GroupClass& k = g->cls[c];
            if (!stage_groupable(k.B)) continue;
            const bool rows = which[w] == 0 || which[w] == 3;
            const StageSpec q{k.t, k.N, in(w, c), out(w, c), rows ? k.gmap : nullptr};
            if (k.B <= kShortTierMaxBw) lo[nlo++] = q;
            else hi[nhi++] = q;
        }
        if (w == 0 && nlo && nhi) {
            S2G_CUDA(cudaEventRecord(g->fork, st));
            S2G_CUDA(cudaStreamWaitEvent(g->side, g->fork, 0));
        }
        const int dc = (which[w] == 1 || which[w] == 2) ? g->dct_ctas : 0;
        if (nhi) S2G_TRY(split_stage_group(which[w], hi, nhi, dc, st));
        if (nlo) S2G_TRY(split_stage_group(which[w], lo, nlo, dc, nhi ? g->side : st));
        // the other classes: one launch each, in stage order on st
        for (int c = 0; c < nc; ++c) {
            GroupClass& k = g->cls[c];
            if (stage_groupable(k.B)) continue;
            S2G_TRY(split_stage_one(which[w], k.t, k.N, in(w, c), out(w, c), k.gmap, st));
        }
    }
    if (nlo && nhi) {
        S2G_CUDA(cudaEventRecord(g->join, g->side));
        S2G_CUDA(cudaStreamWaitEvent(st, g->join, 0));
    }
    return S2G_OK;
}

static int group_fwd_seq(s2g_group g, const float* grid, float* rc, float* ic, cudaStream_t st) {
    const int nc = (int)g->cls.size();
    const int which[2] = {0, 1};  // grid -> X -> C
    S2G_TRY(group_stages(
        g, which, 2, [&](int w, int c) -> const void* { return w == 0 ? (const void*)grid : g->cls[c].buf0; },
        [&](int w, int c) -> void* { return w == 0 ? g->cls[c].buf0 : g->cls[c].buf1; }, st));
    LegSpec spec[kGroupMaxClasses] = {};
    for (int c = 0; c < nc; ++c) {
        GroupClass& k = g->cls[c];
        LegSpec& q = spec[c];
        q.t = k.t;
        q.N = k.N;
        q.NB = k.NB;
        q.C = k.buf1;
        q.X = k.buf0;
        q.rc = rc;
        q.ic = ic;
        q.cmap = k.cmap;
    }
    return split_leg(true, g->precision, spec, nc, g->counters, g->table_stages, st);
}

static int group_inv_seq(s2g_group g, const float* rc, const float* ic, float* grid, cudaStream_t st) {
    const int nc = (int)g->cls.size();
    LegSpec spec[kGroupMaxClasses] = {};
    for (int c = 0; c < nc; ++c) {
        GroupClass& k = g->cls[c];
        LegSpec& q = spec[c];
        q.t = k.t;
        q.N = k.N;
        q.NB = k.NB;
        q.rc_in = rc;
        q.ic_in = ic;
        q.Fc = k.buf1;
        q.F = k.buf0;
        q.cmap = k.cmap;
    }
    S2G_TRY(split_leg(false, g->precision, spec, nc, g->counters + 1, g->table_stages, st));
    const int which[2] = {2, 3};  // Fc -> F -> grid
    return group_stages(
        g, which, 2, [&](int w, int c) -> const void* { return w == 0 ? g->cls[c].buf1 : g->cls[c].buf0; },
        [&](int w, int c) -> void* { return w == 0 ? (void*)g->cls[c].buf0 : (void*)grid; }, st);
}

static int group_seq(s2g_group g, int kind, const void* const* ptr, cudaStream_t st) {
    if (kind == 0) return group_fwd_seq(g, (const float*)ptr[0], (float*)ptr[1], (float*)ptr[2], st);
    if (kind == 1) return group_inv_seq(g, (const float*)ptr[0], (const float*)ptr[1], (float*)ptr[2], st);
    S2G_TRY(group_fwd_seq(g, (const float*)ptr[0], (float*)ptr[1], (float*)ptr[2], st));
    return group_inv_seq(g, (const float*)ptr[1], (const float*)ptr[2], (float*)ptr[3], st);
}

static void drop_graph(GroupGraph& gr) {
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
    gr = GroupGraph{};
}

// Runs sequence `kind` on `st`: replays its graph when the pointers match the captured ones;
// otherwise runs eagerly on `st` and captures a new graph (on the internal stream) for later calls.
static int group_run(s2g_group g, int kind, const void* const* ptr, int nptr, cudaStream_t st) {
    GroupGraph& gr = g->graphs[kind];
    bool same = gr.exec != nullptr;
    for (int i = 0; i < nptr && same; ++i) same = gr.ptr[i] == ptr[i];
    if (same) {
        S2G_CUDA(cudaGraphLaunch(gr.exec, st));
        launches_add(gr.kernels);
        return S2G_OK;
    }
    drop_graph(gr);
    S2G_TRY(group_seq(g, kind, ptr, st));
    // capture for the next call with these pointers (the capture runs nothing)
    cudaGraph_t graph = nullptr;
    S2G_CUDA(cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal));
    capture_count_begin();
    const int r = group_seq(g, kind, ptr, g->cap);
    const unsigned long long nk = capture_count_end();
    const cudaError_t e = cudaStreamEndCapture(g->cap, &graph);
    if (r != S2G_OK) {
        if (graph) cudaGraphDestroy(graph);
        return r;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t ei = cudaGraphInstantiate(&gr.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        gr.exec = nullptr;
        return cuda_fail(ei, "cudaGraphInstantiate");
    }
    for (int i = 0; i < nptr; ++i) gr.ptr[i] = ptr[i];
    gr.kernels = nk;
    return S2G_OK;
}

// ---- autotuner ----

static std::mutex g_tune_mu;
static std::map<std::string, std::string> g_tune;  // key -> "cps NB0 NB1 ..."
static bool g_tune_loaded = false;

static std::string tune_key(s2g_group g) {
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, g->device);
    std::string k = std::string(prop.name) + "|v3|p" + std::to_string(g->precision);
    for (auto& c : g->cls) k += "|" + std::to_string(c.B) + "x" + std::to_string(c.N);
    for (auto& ch : k)
        if (ch == ' ') ch = '_';
    return k;
}

static void tune_load() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = getenv("S2G_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = fopen(path, "r");
    if (!f) return;
    char line[1024];
    while (fgets(line, sizeof line, f)) {
        char* sp = strchr(line, ' ');
        if (!sp) continue;
        *sp = 0;
        std::string v(sp + 1);
        while (!v.empty() && (v.back() == '\n' || v.back() == '\r')) v.pop_back();
        g_tune[line] = v;
    }
    fclose(f);
}

static void tune_store(const std::string& key, const std::string& val) {
    g_tune[key] = val;
    const char* path = getenv("S2G_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %s\n", key.c_str(), val.c_str());
    fclose(f);
}

static std::string tune_value(s2g_group g) {
    std::string v = std::to_string(g->table_stages) + " " + std::to_string(g->dct_ctas);
    for (auto& c : g->cls) v += " " + std::to_string(c.NB);
    return v;
}

static bool tune_apply(s2g_group g, const std::string& v) {
    std::vector<int> x;
    const char* p = v.c_str();
    char* end = nullptr;
    for (;;) {
        const long a = strtol(p, &end, 10);
        if (end == p) break;
        x.push_back((int)a);
        p = end;
    }
    if (x.size() != g->cls.size() + 2) return false;
    g->table_stages = x[0];
    g->dct_ctas = x[1];
    for (size_t c = 0; c < g->cls.size(); ++c) g->cls[c].NB = x[c + 2];
    return true;
}

static void tune_describe(s2g_group g) {
    std::string d = "{\"table_stages\": " + std::to_string(g->table_stages) +
                    ", \"dct_ctas_per_sm\": " + std::to_string(g->dct_ctas) + ", \"tile_n\": {";
    for (size_t c = 0; c < g->cls.size(); ++c) {
        if (c) d += ", ";
        d += "\"" + std::to_string(g->cls[c].B) + "\": " + std::to_string(g->cls[c].NB);
    }
    g->tuning = d + "}}";
}

// Candidate N extents of a class's contraction tile: the whole table-row extent and its
// halvings down to 32 (multiples of 16).
static std::vector<int> nb_candidates(int B) {
    const int full = std::max(16, ((B / 2) + 15) & ~15);
    std::vector<int> v{0};
    for (int n = full / 2; n >= 32; n /= 2) v.push_back(n);
    return v;
}

// Times the group's forward + inverse sequence with the current shapes on the internal stream
// (ms, best of reps; eager launches, so shape changes need no new graph).
static int time_group(s2g_group g, const float* grid, float* rc, float* ic, float* grid_out, int reps, float* ms) {
    cudaEvent_t a, b;
    S2G_CUDA(cudaEventCreate(&a));
    S2G_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    int r = S2G_OK;
    for (int it = 0; it < reps + 1 && r == S2G_OK; ++it) {
        cudaEventRecord(a, g->cap);
        r = group_fwd_seq(g, grid, rc, ic, g->cap);
        if (r == S2G_OK) r = group_inv_seq(g, rc, ic, grid_out, g->cap);
        cudaEventRecord(b, g->cap);
        if (cudaEventSynchronize(b) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "autotune");
        float t = 0;
        cudaEventElapsedTime(&t, a, b);
        if (it > 0) best = std::min(best, t);  // first run warms caches
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = best;
    return r;
}

static int group_autotune(s2g_group g, int force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load();
    const std::string key = tune_key(g);
    if (!force) {
        auto it = g_tune.find(key);
        if (it != g_tune.end() && tune_apply(g, it->second)) {
            tune_describe(g);
            return S2G_OK;
        }
    }
    // synthetic samples and coefficients (zero): the kernels' cost does not depend on values
    float* rc = nullptr;
    const size_t nbuf = 2 * (size_t)g->coef_total + 2 * (size_t)g->grid_total;
    S2G_CUDA(cudaMalloc(&rc, sizeof(float) * nbuf));
    float* ic = rc + g->coef_total;
    float* grid = ic + g->coef_total;
    float* grid_out = grid + g->grid_total;
    S2G_CUDA(cudaMemsetAsync(rc, 0, sizeof(float) * nbuf, g->cap));
    int r = S2G_OK;
    float best = 0;
    g->table_stages = 0;
    g->dct_ctas = 0;
    for (auto& c : g->cls) c.NB = 0;
    auto timed = [&](float* ms) { return time_group(g, grid, rc, ic, grid_out, 3, ms); };
    r = timed(&best);
    // coordinate descent: classes with the most work first, then the persistent grid size
    std::vector<int> order(g->cls.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int x, int y) {
        const double wx = (double)g->cls[x].N * g->cls[x].B * g->cls[x].B * g->cls[x].B;
        const double wy = (double)g->cls[y].N * g->cls[y].B * g->cls[y].B * g->cls[y].B;
        return wx > wy;
    });
    for (int ci : order) {
        if (r != S2G_OK) break;
        GroupClass& c = g->cls[ci];
        int keep = c.NB;
        for (int nb : nb_candidates(c.B)) {
            if (nb == keep) continue;
            c.NB = nb;
            float ms = 0;
            r = timed(&ms);
            if (r != S2G_OK) break;
            if (ms < best * 0.98f) best = ms, keep = nb;
        }
        c.NB = keep;
    }
    for (int ts : {2, 3, 4, 6}) {
        if (r != S2G_OK) break;
        const int keep = g->table_stages;
        g->table_stages = ts;
        float ms = 0;
        r = timed(&ms);
        if (r == S2G_OK && ms < best * 0.98f) best = ms;
        else g->table_stages = keep;
    }
    for (int dc : {1, 2, 3, 4}) {
        if (r != S2G_OK) break;
        const int keep = g->dct_ctas;
        g->dct_ctas = dc;
        float ms = 0;
        r = timed(&ms);
        if (r == S2G_OK && ms < best * 0.98f) best = ms;
        else g->dct_ctas = keep;
    }
    cudaStreamSynchronize(g->cap);
    cudaFree(rc);
    if (r != S2G_OK) return r;
    tune_store(key, tune_value(g));
    tune_describe(g);
    for (auto& gr : g->graphs) drop_graph(gr);
    return S2G_OK;
}

static void group_free(s2g_group g) {
    if (!g) return;
    if (g->device >= 0) cudaSetDevice(g->device);
    if (g->cap) cudaStreamSynchronize(g->cap);
    for (auto& gr : g->graphs) drop_graph(gr);
    if (g->side) cudaStreamSynchronize(g->side);
    if (g->side) cudaStreamDestroy(g->side);
    if (g->cap) cudaStreamDestroy(g->cap);
    if (g->fork) cudaEventDestroy(g->fork);
    if (g->join) cudaEventDestroy(g->join);
    cudaFree(g->mem);
    for (auto& c : g->cls) put_tables(c.t);
    delete g;
}

}  // namespace s2g

using namespace s2g;

extern "C" {

int s2g_group_create(s2g_group* out, int nfunc, const int* bw, int precision) {
    if (!out) return fail(S2G_ERR_ARG, "NULL group pointer");
    *out = nullptr;
    if (nfunc < 1 || !bw) return fail(S2G_ERR_ARG, "a group needs nfunc >= 1 bandwidths (got %d)", nfunc);
    if (precision != S2G_PREC_BF16X3 && precision != S2G_PREC_BF16X2 && precision != S2G_PREC_FP16X2)
        return fail(S2G_ERR_ARG, "precision %d is not a split (tensor-core) mode", precision);
    for (int f = 0; f < nfunc; ++f)
        if (bw[f] < 16 || bw[f] > 512 || (bw[f] > 256 && (bw[f] & (bw[f] - 1))))
            return fail(S2G_ERR_UNSUPPORTED,
                        "function %d: bandwidth %d is neither in [16, 256] nor a power of two up to 512", f, bw[f]);
    {
        std::vector<int> distinct(bw, bw + nfunc);
        std::sort(distinct.begin(), distinct.end());
        const long nd = std::unique(distinct.begin(), distinct.end()) - distinct.begin();
        if (nd > kGroupMaxClasses)
            return fail(S2G_ERR_UNSUPPORTED, "%ld distinct bandwidths in one group (at most %d)", nd, kGroupMaxClasses);
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(S2G_ERR_NOGPU, "no CUDA device");
    s2g_group g = new s2g_group_s();
    g->device = dev;
    g->precision = precision;
    g->nfunc = nfunc;
    g->bw.assign(bw, bw + nfunc);
    g->goff.resize(nfunc);
    g->coff.resize(nfunc);
    for (int f = 0; f < nfunc; ++f) {
        g->goff[f] = g->grid_total;
        g->coff[f] = g->coef_total;
        g->grid_total += 4 * (int64_t)bw[f] * bw[f];
        g->coef_total += (int64_t)bw[f] * bw[f];
    }
    // classes in increasing bandwidth
    for (int B = 16; B <= 512; ++B) {
        GroupClass c;
        c.B = B;
        for (int f = 0; f < nfunc; ++f)
            if (bw[f] == B) c.funcs.push_back(f);
        if (c.funcs.empty()) continue;
        c.N = (int)c.funcs.size();
        g->cls.push_back(c);
    }
    int r = S2G_OK;
    for (auto& c : g->cls) {
        if (r == S2G_OK) r = get_tables(c.B, c.B, &c.t);
        else c.t = nullptr;
    }
    // device memory: maps, intermediates (256-byte aligned pieces), two counters
    auto rnd = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t total = 256;
    auto x_floats = [](const GroupClass& c) { return 2 * (size_t)c.N * c.B * split_layout(c.B).SX; };
    auto c_floats = [](const GroupClass& c) { return 2 * (size_t)c.N * c.B * 2 * split_layout(c.B).BH; };
    for (auto& c : g->cls) {
        total += 2 * rnd(sizeof(int64_t) * c.N);
        total += rnd(sizeof(float) * x_floats(c)) + rnd(sizeof(float) * c_floats(c));
    }
    if (r == S2G_OK && cudaMalloc(&g->mem, total) != cudaSuccess)
        r = fail(S2G_ERR_NOMEM, "group: cudaMalloc of %zu bytes failed", total);
    if (r == S2G_OK) {
        char* p = (char*)g->mem;
        g->counters = (int*)p;
        p += 256;
        std::vector<int64_t> gm, cm;
        for (auto& c : g->cls) {
            c.gmap = (int64_t*)p;
            p += rnd(sizeof(int64_t) * c.N);
            c.cmap = (int64_t*)p;
            p += rnd(sizeof(int64_t) * c.N);
            c.buf0 = (float*)p;
            p += rnd(sizeof(float) * x_floats(c));
            c.buf1 = (float*)p;
            p += rnd(sizeof(float) * c_floats(c));
            gm.clear();
            cm.clear();
            for (int f : c.funcs) gm.push_back(g->goff[f]), cm.push_back(g->coff[f]);
            if (cudaMemcpy(c.gmap, gm.data(), sizeof(int64_t) * c.N, cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(c.cmap, cm.data(), sizeof(int64_t) * c.N, cudaMemcpyHostToDevice) != cudaSuccess) {
                r = cuda_fail(cudaGetLastError(), "group maps");
                break;
            }
        }
    }
    auto ck = [&](cudaError_t e, const char* w) {
        if (e != cudaSuccess && r == S2G_OK) r = cuda_fail(e, w);
    };
    if (r == S2G_OK) {
        ck(cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&g->join, cudaEventDisableTiming), "cudaEventCreate");
    }
    // operands packed now, so that no later call allocates (a graph capture cannot)
    for (auto& c : g->cls)
        if (r == S2G_OK) r = split_prepare(c.t, precision);
    if (r != S2G_OK) {
        group_free(g);
        return r;
    }
    tune_describe(g);
    *out = g;
    return S2G_OK;
}

int s2g_group_destroy(s2g_group g) {
    group_free(g);
    return S2G_OK;
}

int s2g_group_layout(s2g_group g, int64_t* grid_offsets, int64_t* coeff_offsets, int64_t* grid_total,
                     int64_t* coeff_total) {
    if (!g) return fail(S2G_ERR_ARG, "NULL group");
    if (grid_offsets) memcpy(grid_offsets, g->goff.data(), sizeof(int64_t) * g->nfunc);
    if (coeff_offsets) memcpy(coeff_offsets, g->coff.data(), sizeof(int64_t) * g->nfunc);
    if (grid_total) *grid_total = g->grid_total;
    if (coeff_total) *coeff_total = g->coef_total;
    return S2G_OK;
}

static int group_check(s2g_group g) {
    if (!g) return fail(S2G_ERR_ARG, "NULL group");
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(S2G_ERR_NOGPU, "no CUDA device");
    if (dev != g->device) return fail(S2G_ERR_ARG, "group made on device %d used on device %d", g->device, dev);
    return S2G_OK;
}

int s2g_group_fst(s2g_group g, const float* grid, float* rcoeffs, float* icoeffs, void* stream) {
    S2G_TRY(group_check(g));
    if (!grid || !rcoeffs || !icoeffs) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rcoeffs, icoeffs}));
    const void* p[3] = {grid, rcoeffs, icoeffs};
    return group_run(g, 0, p, 3, (cudaStream_t)stream);
}

int s2g_group_inv_fst(s2g_group g, const float* rcoeffs, const float* icoeffs, float* grid, void* stream) {
    S2G_TRY(group_check(g));
    if (!grid || !rcoeffs || !icoeffs) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rcoeffs, icoeffs}));
    const void* p[3] = {rcoeffs, icoeffs, grid};
    return group_run(g, 1, p, 3, (cudaStream_t)stream);
}

int s2g_group_fst_inv(s2g_group g, const float* grid, float* rcoeffs, float* icoeffs, float* grid_out,
                      void* stream) {
    S2G_TRY(group_check(g));
    if (!grid || !rcoeffs || !icoeffs || !grid_out) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rcoeffs, icoeffs, grid_out}));
    const void* p[4] = {grid, rcoeffs, icoeffs, grid_out};
    return group_run(g, 2, p, 4, (cudaStream_t)stream);
}

int s2g_group_autotune(s2g_group g, int force) {
    S2G_TRY(group_check(g));
    return group_autotune(g, force);
}

int s2g_group_set_tiles(s2g_group g, int table_stages, const int* tile_n) {
    S2G_TRY(group_check(g));
    if (table_stages < 0 || table_stages == 1 || table_stages > 8)
        return fail(S2G_ERR_ARG, "table_stages %d: 0 or 2..8", table_stages);
    for (size_t c = 0; tile_n && c < g->cls.size(); ++c)
        if (tile_n[c] < 0 || tile_n[c] > 256 || tile_n[c] % 16)
            return fail(S2G_ERR_ARG, "tile_n[%zu] = %d: a multiple of 16 in [0, 256]", c, tile_n[c]);
    g->table_stages = table_stages;
    for (size_t c = 0; c < g->cls.size(); ++c) g->cls[c].NB = tile_n ? tile_n[c] : 0;
    for (auto& gr : g->graphs) drop_graph(gr);
    tune_describe(g);
    return S2G_OK;
}

int s2g_group_set_dct_ctas(s2g_group g, int dct_ctas_per_sm) {
    S2G_TRY(group_check(g));
    if (dct_ctas_per_sm < 0 || dct_ctas_per_sm > 8)
        return fail(S2G_ERR_ARG, "dct_ctas_per_sm %d outside [0, 8]", dct_ctas_per_sm);
    g->dct_ctas = dct_ctas_per_sm;
    for (auto& gr : g->graphs) drop_graph(gr);
    tune_describe(g);
    return S2G_OK;
}

int s2g_group_describe(s2g_group g, char* buf, size_t len) {
    if (!g || !buf || len == 0) return fail(S2G_ERR_ARG, "NULL argument");
    std::string d = "{\"classes\": [";
    for (size_t c = 0; c < g->cls.size(); ++c) {
        if (c) d += ", ";
        d += "[" + std::to_string(g->cls[c].B) + ", " + std::to_string(g->cls[c].N) + "]";
    }
    d += "], \"tiles\": " + g->tuning + ", \"graph_kernels\": [" + std::to_string(g->graphs[0].kernels) + ", " +
         std::to_string(g->graphs[1].kernels) + ", " + std::to_string(g->graphs[2].kernels) + "]}";
    if (d.size() + 1 > len) return fail(S2G_ERR_ARG, "buffer of %zu bytes too small (%zu needed)", len, d.size() + 1);
    memcpy(buf, d.c_str(), d.size() + 1);
    return S2G_OK;
}

int s2g_group_sync_status(s2g_group g) {
    S2G_TRY(group_check(g));
    S2G_CUDA(cudaStreamSynchronize(g->cap));
    S2G_CUDA(cudaDeviceSynchronize());
    int r = S2G_OK;
    for (auto& c : g->cls) {
        const int v = split_device_status(c.t, 1);
        if (v != S2G_OK && r == S2G_OK) r = v;
    }
    return r;
}

}  // extern "C"
