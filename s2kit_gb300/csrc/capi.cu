// capi.cu -- the C ABI (include/s2kit_gb300.h): S2kit memo-path drop-ins on host buffers
// and the batched device-pointer API.  All transforms run on the GPU; there is no CPU path.
#include <limits.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <algorithm>
#include <vector>

#include "s2g_common.cuh"
#include "s2g_internal.h"

namespace s2g {

static thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

// name of the kernel this thread launched last (for launch-error messages)
static thread_local const char* t_kernel = "";

int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? S2G_ERR_NOMEM : S2G_ERR_CUDA, "%s: %s (last kernel launched: %s)",
                what, cudaGetErrorString(e), t_kernel);
}

// ---------------------------------------------------------------------------------
// Launch counting and optional per-kernel event timing.
static std::atomic<unsigned long long> g_launches{0};
static std::atomic<int> g_prof_on{0};
struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
};
static std::mutex g_prof_mu;
static std::vector<ProfRec> g_prof_recs;
static std::vector<cudaEvent_t> g_prof_pool;
static thread_local std::vector<size_t> t_prof_open;

static cudaEvent_t prof_event() {
    if (!g_prof_pool.empty()) {
        cudaEvent_t e = g_prof_pool.back();
        g_prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// While this thread captures a graph, launches are counted into the graph instead of the
// process total (each replay adds them) and are not bracketed by events.
static thread_local bool t_capturing = false;
static thread_local unsigned long long t_captured = 0;

void capture_count_begin() {
    t_capturing = true;
    t_captured = 0;
}

unsigned long long capture_count_end() {
    t_capturing = false;
    return t_captured;
}

void launches_add(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void prof_begin(const char* name, cudaStream_t st) {
    t_kernel = name;
    if (t_capturing) {
        ++t_captured;
        return;
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    ProfRec r{name, prof_event(), prof_event()};
    cudaEventRecord(r.a, st);
    g_prof_recs.push_back(r);
    t_prof_open.push_back(g_prof_recs.size() - 1);
}

void prof_end(cudaStream_t st) {
    if (t_capturing || !g_prof_on.load(std::memory_order_relaxed) || t_prof_open.empty()) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    const size_t i = t_prof_open.back();
    t_prof_open.pop_back();
    if (i < g_prof_recs.size()) cudaEventRecord(g_prof_recs[i].b, st);
}

int Scratch::ensure(size_t need) {
    if (need <= bytes) return S2G_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t want = need + need / 8;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return cuda_fail(e, "cudaMalloc(scratch)");
    }
    bytes = want;
    return S2G_OK;
}

void Scratch::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

// ---------------------------------------------------------------------------------
// Parameter checks shared by every entry point.
static int check_bw(int bw) {
    if (bw < 2) return fail(S2G_ERR_ARG, "bandwidth %d < 2", bw);
    const bool pow2 = (bw & (bw - 1)) == 0;
    if (pow2 && bw > 2048) return fail(S2G_ERR_UNSUPPORTED, "bandwidth %d > 2048", bw);
    if (!pow2 && bw > 512) return fail(S2G_ERR_UNSUPPORTED, "non power-of-two bandwidth %d > 512", bw);
    return S2G_OK;
}

static int check_cutoff(int bw, int cutoff) {
    // cutoff 0 makes the reference apply DLTNaive to the order-0 cosine table
    // (SemiNaive_Naive_Pml_Table always builds order 0 as a cosine table, cospml.c:455-456)
    if (cutoff < 1 || cutoff > bw) return fail(S2G_ERR_ARG, "cutoff %d outside [1, bw=%d]", cutoff, bw);
    return S2G_OK;
}

static int current_device(int* dev) {
    cudaError_t e = cudaGetDevice(dev);
    if (e != cudaSuccess) return fail(S2G_ERR_NOGPU, "no CUDA device: %s", cudaGetErrorString(e));
    return S2G_OK;
}

// Device used by the host-buffer drop-ins: $S2G_DEVICE or 0.
static int dropin_device() {
    static int dev = -1;
    if (dev < 0) {
        const char* s = getenv("S2G_DEVICE");
        dev = s ? atoi(s) : 0;
    }
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return fail(S2G_ERR_NOGPU, "cudaSetDevice(%d): %s", dev, cudaGetErrorString(e));
    return S2G_OK;
}

// ---------------------------------------------------------------------------------
// Device table cache, keyed by (device, bw, cutoff).
static std::mutex g_tab_mu;
static std::map<std::tuple<int, int, int>, Tables*> g_tables;

static void free_tables(Tables* t);

// Returns the tables with one reference taken for the caller (released with put_tables); the
// cache holds its own reference, so s2g_cache_clear() never frees tables a plan still uses.
int get_tables(int bw, int cutoff, Tables** out) {
    int dev;
    S2G_TRY(current_device(&dev));
    std::lock_guard<std::mutex> lk(g_tab_mu);
    auto key = std::make_tuple(dev, bw, cutoff);
    auto it = g_tables.find(key);
    if (it != g_tables.end()) {
        ++it->second->refs;
        *out = it->second;
        return S2G_OK;
    }
    Tables* t = new Tables();
    t->bw = bw;
    t->cutoff = cutoff;
    t->device = dev;
    cudaStream_t st;
    S2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int r = build_tables(t, st);
    cudaStreamDestroy(st);
    if (r != S2G_OK) {
        free_tables(t);
        return r;
    }
    t->refs = 2;  // the cache and the caller
    g_tables[key] = t;
    *out = t;
    return S2G_OK;
}

void put_tables(Tables* t) {
    if (!t) return;
    std::lock_guard<std::mutex> lk(g_tab_mu);
    if (--t->refs == 0) free_tables(t);
}

void free_split(Tables* t);

static void free_tables(Tables* t) {
    if (!t) return;
    cudaFree(t->fwd);
    cudaFree(t->inv);
    cudaFree(t->off);
    cudaFree(t->weights);
    cudaFree(t->sinv);
    cudaFree(t->tw_S);
    cudaFree(t->tw_D);
    free_split(t);
    delete[] t->h_off;
    delete t;
}

// Caller tables uploaded by the drop-ins, keyed by the table-pointer array and contents
// fingerprint (first and last entry of every order).
struct Upload {
    double* d = nullptr;
    uint64_t fp = 0;
};
static std::map<std::tuple<int, const void*, int, int, int>, Upload> g_uploads;

static int64_t order_size(int bw, int cutoff, int m) {
    return (m < cutoff) ? table_size(m, bw) : 2 * (int64_t)bw * (bw - m);
}

static uint64_t fingerprint(double** tab, int bw, int cutoff) {
    uint64_t h = 1469598103934665603ull;
    for (int m = 0; m < bw; ++m) {
        const int64_t n = order_size(bw, cutoff, m);
        if (n <= 0) continue;
        uint64_t a, b;
        memcpy(&a, &tab[m][0], 8);
        memcpy(&b, &tab[m][n - 1], 8);
        h = (h ^ a) * 1099511628211ull;
        h = (h ^ b) * 1099511628211ull;
        h = (h ^ (uint64_t)(uintptr_t)tab[m]) * 1099511628211ull;
    }
    return h;
}

// Uploads (or finds) the caller's packed table `tab` (kind 0 forward, 1 transposed).
static int upload_table(const Tables* t, double** tab, int kind, double** d_out) {
    if (!tab) return fail(S2G_ERR_ARG, "NULL table");
    const int bw = t->bw, cutoff = t->cutoff;
    for (int m = 0; m < bw; ++m)
        if (!tab[m] && order_size(bw, cutoff, m) > 0) return fail(S2G_ERR_ARG, "NULL table entry for order %d", m);
    const uint64_t fp = fingerprint(tab, bw, cutoff);
    std::lock_guard<std::mutex> lk(g_tab_mu);
    auto key = std::make_tuple(t->device, (const void*)tab, bw, cutoff, kind);
    auto it = g_uploads.find(key);
    if (it != g_uploads.end() && it->second.fp == fp) {
        *d_out = it->second.d;
        return S2G_OK;
    }
    double* d = (it != g_uploads.end()) ? it->second.d : nullptr;
    if (!d) S2G_CUDA(cudaMalloc(&d, sizeof(double) * (size_t)(t->total > 0 ? t->total : 1)));
    for (int m = 0; m < bw; ++m) {
        const int64_t n = order_size(bw, cutoff, m);
        if (n > 0) S2G_CUDA(cudaMemcpy(d + t->h_off[m], tab[m], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    }
    g_uploads[key] = Upload{d, fp};
    *d_out = d;
    return S2G_OK;
}

// Per-thread device scratch for the drop-ins.
struct DropinScratch {
    Scratch s;
    ~DropinScratch() { s.release(); }
};
static thread_local DropinScratch g_dscratch;

// Carve `n` doubles out of a scratch area.
struct Carve {
    char* base;
    size_t used = 0;
    double* take(size_t n) {
        double* p = (double*)(base + used);
        used += ((n * sizeof(double) + 255) / 256) * 256;
        return p;
    }
};

static size_t rnd(size_t n) { return ((n * sizeof(double) + 255) / 256) * 256; }

static void report(const char* fn, int r) {
    if (r != S2G_OK) fprintf(stderr, "s2kit_gb300: %s failed (%d): %s\n", fn, r, g_last_error.c_str());
}

// ---------------------------------------------------------------------------------
// Drop-in implementations (return a status; the exported void wrappers print it).

// fly: the on-the-fly family (no Legendre table on the device; `table` unused).
static int do_fst(double* rdata, double* idata, double* rcoeffs, double* icoeffs, int bw, double** table,
                  int fmt, int cutoff, double* weights, bool fly = false) {
    S2G_TRY(check_bw(bw));
    S2G_TRY(check_cutoff(bw, cutoff));
    if (!rdata || !idata || !rcoeffs || !icoeffs) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(dropin_device());
    Tables* base;
    S2G_TRY(get_tables(bw, fly ? 0 : cutoff, &base));
    TabRef tref_{base};
    Tables view = *base;
    view.split = nullptr;
    if (table) S2G_TRY(upload_table(base, table, 0, &view.fwd));  // null: the device's own table (on the fly)
    const size_t S = 2 * (size_t)bw, ng = S * S, nc = (size_t)bw * bw;
    const size_t need = 2 * rnd(ng) + 2 * rnd(nc) + rnd(4 * (size_t)bw) + f64_work_bytes(bw, 1, fmt) + 256;
    S2G_TRY(g_dscratch.s.ensure(need));
    Carve c{(char*)g_dscratch.s.ptr};
    double *dr = c.take(ng), *di = c.take(ng), *cr = c.take(nc), *ci = c.take(nc), *dw = c.take(4 * bw);
    void* work = c.take(f64_work_bytes(bw, 1, fmt) / sizeof(double));
    S2G_CUDA(cudaMemcpy(dr, rdata, ng * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(di, idata, ng * 8, cudaMemcpyHostToDevice));
    if (weights) {
        S2G_CUDA(cudaMemcpy(dw, weights, 4 * (size_t)bw * 8, cudaMemcpyHostToDevice));
        view.weights = dw;
    }
    if (fly)
        S2G_TRY(fst_f64_fly(&view, dr, di, cr, ci, 1, fmt, work, 0));
    else
        S2G_TRY(fst_f64(&view, dr, di, cr, ci, 1, fmt, cutoff, work, 0));
    S2G_CUDA(cudaMemcpy(rcoeffs, cr, nc * 8, cudaMemcpyDeviceToHost));
    S2G_CUDA(cudaMemcpy(icoeffs, ci, nc * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

static int do_inv_fst(double* rcoeffs, double* icoeffs, double* rdata, double* idata, int bw, double** ttable,
                      int fmt, int cutoff, bool fly = false) {
    S2G_TRY(check_bw(bw));
    S2G_TRY(check_cutoff(bw, cutoff));
    if (!rdata || !idata || !rcoeffs || !icoeffs) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(dropin_device());
    Tables* base;
    S2G_TRY(get_tables(bw, fly ? 0 : cutoff, &base));
    TabRef tref_{base};
    Tables view = *base;
    view.split = nullptr;
    if (ttable) S2G_TRY(upload_table(base, ttable, 1, &view.inv));  // null: the device's own table
    const size_t S = 2 * (size_t)bw, ng = S * S, nc = (size_t)bw * bw;
    const size_t need = 2 * rnd(ng) + 2 * rnd(nc) + f64_work_bytes(bw, 1, fmt) + 256;
    S2G_TRY(g_dscratch.s.ensure(need));
    Carve c{(char*)g_dscratch.s.ptr};
    double *dr = c.take(ng), *di = c.take(ng), *cr = c.take(nc), *ci = c.take(nc);
    void* work = c.take(f64_work_bytes(bw, 1, fmt) / sizeof(double));
    S2G_CUDA(cudaMemcpy(cr, rcoeffs, nc * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(ci, icoeffs, nc * 8, cudaMemcpyHostToDevice));
    if (fly)
        S2G_TRY(inv_fst_f64_fly(&view, cr, ci, dr, di, 1, fmt, work, 0));
    else
        S2G_TRY(inv_fst_f64(&view, cr, ci, dr, di, 1, fmt, cutoff, work, 0));
    S2G_CUDA(cudaMemcpy(rdata, dr, ng * 8, cudaMemcpyDeviceToHost));
    S2G_CUDA(cudaMemcpy(idata, di, ng * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

static int do_fzt(double* rdata, double* idata, double* rres, double* ires, int bw, double* cos_pml_table, int fmt,
                  double* weights, bool fly = false) {
    S2G_TRY(check_bw(bw));
    if (!rdata || !idata || !rres || !ires) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(dropin_device());
    Tables* base;
    S2G_TRY(get_tables(bw, fly ? 0 : bw, &base));
    TabRef tref_{base};
    Tables view = *base;
    view.split = nullptr;
    const size_t S = 2 * (size_t)bw, ng = S * S, nt = (size_t)table_size(0, bw);
    const size_t need = 2 * rnd(ng) + 2 * rnd(S) + rnd(nt) + rnd(4 * (size_t)bw) + f64_work_bytes(bw, 1, REAL) + 256;
    S2G_TRY(g_dscratch.s.ensure(need));
    Carve c{(char*)g_dscratch.s.ptr};
    double *dr = c.take(ng), *di = c.take(ng), *rr = c.take(S), *ri = c.take(S), *tab = c.take(nt),
           *dw = c.take(4 * bw);
    void* work = c.take(f64_work_bytes(bw, 1, REAL) / sizeof(double));
    S2G_CUDA(cudaMemcpy(dr, rdata, ng * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(di, idata, ng * 8, cudaMemcpyHostToDevice));
    if (cos_pml_table) {  // null: the device's own order-0 table (on the fly)
        S2G_CUDA(cudaMemcpy(tab, cos_pml_table, nt * 8, cudaMemcpyHostToDevice));
        view.fwd = tab;
    }
    if (weights) {
        S2G_CUDA(cudaMemcpy(dw, weights, 4 * (size_t)bw * 8, cudaMemcpyHostToDevice));
        view.weights = dw;
    }
    if (fly)
        S2G_TRY(fzt_f64_fly(&view, dr, di, rr, ri, 1, fmt, work, 0));
    else
        S2G_TRY(fzt_f64(&view, dr, di, rr, ri, 1, fmt, work, 0));
    S2G_CUDA(cudaMemcpy(rres, rr, (size_t)bw * 8, cudaMemcpyDeviceToHost));
    if (fmt == COMPLEX) {
        S2G_CUDA(cudaMemcpy(ires, ri, (size_t)bw * 8, cudaMemcpyDeviceToHost));
    } else {
        memset(ires, 0, sizeof(double) * S);  // 2*bw zeros, FST_semi_memo.c:406
    }
    return S2G_OK;
}

// t without Legendre tables (cutoff 0): the on-the-fly kernels.
static int conv_device(const Tables* t, const double* dr, const double* di, const double* fr, const double* fi,
                       double* rr, double* ri, int batch, Scratch& scr, cudaStream_t st) {
    const bool fly = (t->cutoff == 0);
    const int bw = t->bw;
    const size_t nc = (size_t)bw * bw;
    const size_t work = f64_work_bytes(bw, batch, REAL);
    const size_t need = 4 * rnd(nc * batch) + 2 * rnd(2 * (size_t)bw * batch) + work + 256;
    S2G_TRY(scr.ensure(need));
    Carve c{(char*)scr.ptr};
    double *cr = c.take(nc * batch), *ci = c.take(nc * batch), *tr = c.take(nc * batch), *ti = c.take(nc * batch);
    double *hr = c.take(2 * (size_t)bw * batch), *hi = c.take(2 * (size_t)bw * batch);
    void* w = c.take(work / sizeof(double));
    if (fly) {
        S2G_TRY(fst_f64_fly(t, dr, di, cr, ci, batch, REAL, w, st));
        S2G_TRY(fzt_f64_fly(t, fr, fi, hr, hi, batch, REAL, w, st));
    } else {
        S2G_TRY(fst_f64(t, dr, di, cr, ci, batch, REAL, bw, w, st));
        S2G_TRY(fzt_f64(t, fr, fi, hr, hi, batch, REAL, w, st));
    }
    S2G_TRY(transmult_f64(cr, ci, hr, hi, tr, ti, bw, batch, st));
    if (fly)
        S2G_TRY(inv_fst_f64_fly(t, tr, ti, rr, ri, batch, REAL, w, st));
    else
        S2G_TRY(inv_fst_f64(t, tr, ti, rr, ri, batch, REAL, bw, w, st));
    return S2G_OK;
}

static int do_conv(double* rdata, double* idata, double* rfilter, double* ifilter, double* rres, double* ires,
                   int bw, bool fly = false) {
    S2G_TRY(check_bw(bw));
    if (!rdata || !idata || !rfilter || !ifilter || !rres || !ires) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(dropin_device());
    Tables* t;
    S2G_TRY(get_tables(bw, fly ? 0 : bw, &t));
    TabRef tref_{t};
    const size_t S = 2 * (size_t)bw, ng = S * S;
    static thread_local DropinScratch io;
    S2G_TRY(io.s.ensure(6 * rnd(ng) + 256));
    Carve c{(char*)io.s.ptr};
    double *dr = c.take(ng), *di = c.take(ng), *fr = c.take(ng), *fi = c.take(ng), *orr = c.take(ng),
           *oi = c.take(ng);
    S2G_CUDA(cudaMemcpy(dr, rdata, ng * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(di, idata, ng * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(fr, rfilter, ng * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(fi, ifilter, ng * 8, cudaMemcpyHostToDevice));
    S2G_TRY(conv_device(t, dr, di, fr, fi, orr, oi, 1, g_dscratch.s, 0));
    S2G_CUDA(cudaMemcpy(rres, orr, ng * 8, cudaMemcpyDeviceToHost));
    S2G_CUDA(cudaMemcpy(ires, oi, ng * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

// 1-D Legendre transforms with the caller's tables.
static int do_dlt(int kind, const double* in, int bw, int m, double* out, const double* table, const double* aux) {
    S2G_TRY(check_bw(bw));
    if (m < 0 || m >= bw) return fail(S2G_ERR_ARG, "order %d outside [0, bw)", m);
    if (!in || !out || !table) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(dropin_device());
    Tables* t;
    S2G_TRY(get_tables(bw, bw, &t));
    TabRef tref_{t};
    const size_t S = 2 * (size_t)bw;
    const size_t nt = (kind <= 1) ? (size_t)table_size(m, bw) : S * (size_t)(bw - m);
    const size_t nin = (kind == 0 || kind == 2) ? S : (size_t)(bw - m);
    const size_t nout = (kind == 0 || kind == 2) ? (size_t)(bw - m) : S;
    const size_t naux = (kind == 1) ? S : 4 * (size_t)bw;
    S2G_TRY(g_dscratch.s.ensure(rnd(nt) + rnd(nin) + rnd(nout) + rnd(naux) + 256));
    Carve c{(char*)g_dscratch.s.ptr};
    double *dt = c.take(nt), *di = c.take(nin), *dout = c.take(nout), *da = c.take(naux);
    if (nt) S2G_CUDA(cudaMemcpy(dt, table, nt * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(di, in, nin * 8, cudaMemcpyHostToDevice));
    if (aux) S2G_CUDA(cudaMemcpy(da, aux, naux * 8, cudaMemcpyHostToDevice));
    switch (kind) {
        case 0: S2G_TRY(dlt_semi_f64(di, bw, m, dout, dt, aux ? da : t->weights, t->tw_S, t->tw_D, 0)); break;
        case 1: S2G_TRY(inv_dlt_semi_f64(di, bw, m, dout, dt, aux ? da : t->sinv, t->tw_S, t->tw_D, 0)); break;
        case 2: S2G_TRY(dlt_naive_f64(di, bw, m, aux ? da : t->weights, dout, dt, 0)); break;
        default: S2G_TRY(inv_dlt_naive_f64(di, bw, m, dout, dt, 0)); break;
    }
    S2G_CUDA(cudaMemcpy(out, dout, nout * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

// Table builders: generate on the device into a temporary buffer and copy to the caller.
static int do_gen_tables(int bw, int cutoff, int which, double* resultspace, double** src, int64_t* total_out) {
    // which: 0 forward (seminaive below cutoff, naive above), 1 transposed from `src`
    S2G_TRY(check_bw(bw));
    if (cutoff < 0 || cutoff > bw) return fail(S2G_ERR_ARG, "cutoff %d outside [0, bw]", cutoff);
    S2G_TRY(dropin_device());
    std::vector<int64_t> off(bw);
    int64_t total = 0;
    for (int m = 0; m < bw; ++m) {
        off[m] = total;
        total += order_size(bw, cutoff, m);
    }
    *total_out = total;
    double *dfwd = nullptr, *dinv = nullptr;
    int64_t* doff = nullptr;
    struct Guard {
        double** a; double** b; int64_t** c;
        ~Guard() { cudaFree(*a); cudaFree(*b); cudaFree(*c); }
    } g{&dfwd, &dinv, &doff};
    S2G_CUDA(cudaMalloc(&dfwd, sizeof(double) * (size_t)(total > 0 ? total : 1)));
    S2G_CUDA(cudaMalloc(&dinv, sizeof(double) * (size_t)(total > 0 ? total : 1)));
    S2G_CUDA(cudaMalloc(&doff, sizeof(int64_t) * bw));
    S2G_CUDA(cudaMemcpy(doff, off.data(), sizeof(int64_t) * bw, cudaMemcpyHostToDevice));
    if (which == 0) {
        S2G_TRY(generate_cos_pml_device(bw, 0, cutoff, dfwd, doff, 0));
        S2G_TRY(generate_pml_device(bw, cutoff, bw, dfwd, doff, 0));
        S2G_CUDA(cudaMemcpy(resultspace, dfwd, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost));
        return S2G_OK;
    }
    for (int m = 0; m < bw; ++m) {
        const int64_t n = order_size(bw, cutoff, m);
        if (n > 0) S2G_CUDA(cudaMemcpy(dfwd + off[m], src[m], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    }
    S2G_TRY(transpose_cos_pml_device(bw, 0, cutoff, dfwd, dinv, doff, 0));
    if (cutoff < bw)  // the naive orders are stored untransposed (cospml.c:506-515)
        S2G_CUDA(cudaMemcpy(dinv + off[cutoff], dfwd + off[cutoff], sizeof(double) * (size_t)(total - off[cutoff]),
                            cudaMemcpyDeviceToDevice));
    S2G_CUDA(cudaMemcpy(resultspace, dinv, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

static double** pointer_array(int bw, int cutoff, double* resultspace, int extra) {
    double** p = (double**)malloc(sizeof(double*) * (size_t)(bw + extra));
    if (!p) return nullptr;
    int64_t o = 0;
    for (int m = 0; m < bw; ++m) {
        p[m] = resultspace + o;
        o += order_size(bw, cutoff, m);
    }
    for (int k = 0; k < extra; ++k) p[bw + k] = resultspace + o;
    return p;
}

// Single-order generation / transposition / sampled table into caller memory.
static int do_order(int kind, int bw, int m, const double* in, double* out) {
    S2G_TRY(check_bw(bw));
    if (m < 0 || m >= bw) return fail(S2G_ERR_ARG, "order %d outside [0, bw)", m);
    if (!out) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(dropin_device());
    const size_t n = (kind == 2) ? 2 * (size_t)bw * (bw - m) : (size_t)table_size(m, bw);
    std::vector<int64_t> zero(bw, 0);
    S2G_TRY(g_dscratch.s.ensure(2 * rnd(n) + rnd(bw) + 256));
    Carve c{(char*)g_dscratch.s.ptr};
    double *a = c.take(n), *b = c.take(n);
    int64_t* doff = (int64_t*)c.take(bw);
    S2G_CUDA(cudaMemcpy(doff, zero.data(), sizeof(int64_t) * bw, cudaMemcpyHostToDevice));
    if (kind == 0) {
        S2G_TRY(generate_cos_pml_device(bw, m, m + 1, a, doff, 0));
    } else if (kind == 1) {
        if (!in) return fail(S2G_ERR_ARG, "NULL table");
        S2G_CUDA(cudaMemcpy(b, in, n * 8, cudaMemcpyHostToDevice));
        S2G_TRY(transpose_cos_pml_device(bw, m, m + 1, b, a, doff, 0));
    } else {
        S2G_TRY(generate_pml_device(bw, m, m + 1, a, doff, 0));
    }
    S2G_CUDA(cudaMemcpy(out, a, n * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

static int do_vec(int kind, int n, int m, const double* in, double* out) {
    // kind 0 acos nodes, 1 cos nodes, 2 Pmm_L2(m, in), 3 weights (n = bw)
    if (n < 1 || !out) return fail(S2G_ERR_ARG, "bad vector request");
    S2G_TRY(dropin_device());
    const size_t len = (kind == 3) ? 4 * (size_t)n : (size_t)n;
    S2G_TRY(g_dscratch.s.ensure(2 * rnd(len) + 256));
    Carve c{(char*)g_dscratch.s.ptr};
    double *a = c.take(len), *b = c.take(len);
    if (kind == 2) {
        if (!in) return fail(S2G_ERR_ARG, "NULL eval points");
        S2G_CUDA(cudaMemcpy(b, in, (size_t)n * 8, cudaMemcpyHostToDevice));
        S2G_TRY(pmm_device(m, b, n, a, 0));
    } else if (kind == 3) {
        S2G_TRY(generate_weights_device(n, a, 0));
    } else {
        S2G_TRY(nodes_device(n, a, kind, 0));
    }
    S2G_CUDA(cudaMemcpy(out, a, len * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

static int do_transmult(const double* rd, const double* id, const double* rf, const double* iff, double* rr,
                        double* ir, int bw) {
    if (bw < 1 || !rd || !id || !rf || !iff || !rr || !ir) return fail(S2G_ERR_ARG, "bad TransMult arguments");
    S2G_TRY(dropin_device());
    const size_t nc = (size_t)bw * bw;
    S2G_TRY(g_dscratch.s.ensure(4 * rnd(nc) + 2 * rnd(bw) + 256));
    Carve c{(char*)g_dscratch.s.ptr};
    double *a = c.take(nc), *b = c.take(nc), *o1 = c.take(nc), *o2 = c.take(nc), *f1 = c.take(bw), *f2 = c.take(bw);
    S2G_CUDA(cudaMemcpy(a, rd, nc * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(b, id, nc * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(f1, rf, (size_t)bw * 8, cudaMemcpyHostToDevice));
    S2G_CUDA(cudaMemcpy(f2, iff, (size_t)bw * 8, cudaMemcpyHostToDevice));
    S2G_TRY(transmult_f64(a, b, f1, f2, o1, o2, bw, 1, 0));
    S2G_CUDA(cudaMemcpy(rr, o1, nc * 8, cudaMemcpyDeviceToHost));
    S2G_CUDA(cudaMemcpy(ir, o2, nc * 8, cudaMemcpyDeviceToHost));
    return S2G_OK;
}

}  // namespace s2g

using namespace s2g;

// =================================== exported =========================================
extern "C" {

void FSTSemiMemo(double* rdata, double* idata, double* rcoeffs, double* icoeffs, const int bw,
                 double** seminaive_naive_table, double* workspace, DataFormat data_format, const int cutoff,
                 fftw_plan* DCT_plan, fftw_plan* FFT_plan, double* weights) {
    (void)workspace; (void)DCT_plan; (void)FFT_plan;
    report("FSTSemiMemo",
           do_fst(rdata, idata, rcoeffs, icoeffs, bw, seminaive_naive_table, (int)data_format, cutoff, weights));
}

void InvFSTSemiMemo(double* rcoeffs, double* icoeffs, double* rdata, double* idata, const int bw,
                    double** transpose_seminaive_naive_table, double* workspace, DataFormat data_format,
                    const int cutoff, fftw_plan* inv_DCT_plan, fftw_plan* inv_FFT_plan) {
    (void)workspace; (void)inv_DCT_plan; (void)inv_FFT_plan;
    report("InvFSTSemiMemo", do_inv_fst(rcoeffs, icoeffs, rdata, idata, bw, transpose_seminaive_naive_table,
                                        (int)data_format, cutoff));
}

void FZTSemiMemo(double* rdata, double* idata, double* rres, double* ires, const int bw, double* cos_pml_table,
                 double* workspace, DataFormat data_format, fftw_plan* DCT_plan, double* weights) {
    (void)workspace; (void)DCT_plan;
    report("FZTSemiMemo", do_fzt(rdata, idata, rres, ires, bw, cos_pml_table, (int)data_format, weights));
}

void ConvOn2SphereSemiMemo(double* rdata, double* idata, double* rfilter, double* ifilter, double* rres,
                           double* ires, const int bw, double* workspace) {
    (void)workspace;
    report("ConvOn2SphereSemiMemo", do_conv(rdata, idata, rfilter, ifilter, rres, ires, bw));
}

// On-the-fly family (src/FST_semi_fly.c): like the reference, no Legendre table outlives an
// order; here none is written at all, the recurrence runs inside the contraction kernels
// (fst_f64_fly and companions).
void FSTSemiFly(double* rdata, double* idata, double* rcoeffs, double* icoeffs, const int bw, double* workspace,
                DataFormat data_format, const int cutoff, fftw_plan* DCT_plan, fftw_plan* FFT_plan,
                double* weights) {
    (void)workspace; (void)DCT_plan; (void)FFT_plan;
    report("FSTSemiFly",
           do_fst(rdata, idata, rcoeffs, icoeffs, bw, nullptr, (int)data_format, cutoff, weights, true));
}

void InvFSTSemiFly(double* rcoeffs, double* icoeffs, double* rdata, double* idata, const int bw, double* workspace,
                   DataFormat data_format, const int cutoff, fftw_plan* inv_DCT_plan, fftw_plan* inv_FFT_plan) {
    (void)workspace; (void)inv_DCT_plan; (void)inv_FFT_plan;
    report("InvFSTSemiFly", do_inv_fst(rcoeffs, icoeffs, rdata, idata, bw, nullptr, (int)data_format, cutoff, true));
}

void FZTSemiFly(double* rdata, double* idata, double* rres, double* ires, const int bw, double* workspace,
                DataFormat data_format, fftw_plan* DCT_plan, double* weights) {
    (void)workspace; (void)DCT_plan;
    report("FZTSemiFly", do_fzt(rdata, idata, rres, ires, bw, nullptr, (int)data_format, weights, true));
}

void ConvOn2SphereSemiFly(double* rdata, double* idata, double* rfilter, double* ifilter, double* rres,
                          double* ires, const int bw, double* workspace) {
    (void)workspace;
    report("ConvOn2SphereSemiFly", do_conv(rdata, idata, rfilter, ifilter, rres, ires, bw, true));
}

void DLTSemi(double* data, const int bw, const int m, double* result, double* workspace, double* cos_pml_table,
             double* weights, fftw_plan* plan) {
    (void)workspace; (void)plan;
    report("DLTSemi", do_dlt(0, data, bw, m, result, cos_pml_table, weights));
}

void InvDLTSemi(double* coeffs, const int bw, const int m, double* result, double* trans_cos_pml_table,
                double* sin_values, double* workspace, fftw_plan* plan) {
    (void)workspace; (void)plan;
    report("InvDLTSemi", do_dlt(1, coeffs, bw, m, result, trans_cos_pml_table, sin_values));
}

void DLTNaive(double* data, const int bw, const int m, double* weights, double* result, double* pml_table,
              double* workspace) {
    (void)workspace;
    report("DLTNaive", do_dlt(2, data, bw, m, result, pml_table, weights));
}

void InvDLTNaive(double* coeffs, const int bw, const int m, double* result, double* pml_table) {
    report("InvDLTNaive", do_dlt(3, coeffs, bw, m, result, pml_table, nullptr));
}

void GenerateWeightsForDLT(const int bw, double* weights) {
    report("GenerateWeightsForDLT", do_vec(3, bw, 0, nullptr, weights));
}

void GenerateCosPmlTable(const int bw, const int m, double* tablespace, double* workspace) {
    (void)workspace;
    report("GenerateCosPmlTable", do_order(0, bw, m, nullptr, tablespace));
}

void TransposeCosPmlTable(const int bw, const int m, double* cos_pml_table, double* result) {
    report("TransposeCosPmlTable", do_order(1, bw, m, cos_pml_table, result));
}

void GeneratePmlTable(const int bw, const int m, double* pml_table, double* workspace) {
    (void)workspace;
    report("GeneratePmlTable", do_order(2, bw, m, nullptr, pml_table));
}

double** Spharmonic_Pml_Table(const int bw, double* resultspace, double* workspace) {
    (void)workspace;
    int64_t total;
    int r = do_gen_tables(bw, bw, 0, resultspace, nullptr, &total);
    report("Spharmonic_Pml_Table", r);
    return r == S2G_OK ? pointer_array(bw, bw, resultspace, 0) : nullptr;
}

double** Transpose_Spharmonic_Pml_Table(double** spharmonic_pml_table, const int bw, double* resultspace) {
    int64_t total;
    int r = do_gen_tables(bw, bw, 1, resultspace, spharmonic_pml_table, &total);
    report("Transpose_Spharmonic_Pml_Table", r);
    return r == S2G_OK ? pointer_array(bw, bw, resultspace, 0) : nullptr;
}

double** SemiNaive_Naive_Pml_Table(const int bw, const int m, double* resultspace, double* workspace) {
    (void)workspace;
    int64_t total;
    int r = (m < 1) ? fail(S2G_ERR_ARG, "cutoff %d < 1", m) : do_gen_tables(bw, m, 0, resultspace, nullptr, &total);
    report("SemiNaive_Naive_Pml_Table", r);
    return r == S2G_OK ? pointer_array(bw, m, resultspace, 1) : nullptr;
}

double** Transpose_SemiNaive_Naive_Pml_Table(double** seminaive_naive_pml_table, const int bw, const int m,
                                             double* resultspace, double* workspace) {
    (void)workspace;
    int64_t total;
    int r = (m < 1) ? fail(S2G_ERR_ARG, "cutoff %d < 1", m)
                    : do_gen_tables(bw, m, 1, resultspace, seminaive_naive_pml_table, &total);
    report("Transpose_SemiNaive_Naive_Pml_Table", r);
    return r == S2G_OK ? pointer_array(bw, m, resultspace, 1) : nullptr;
}

void Pmm_L2(const int m, double* eval_points, const int n, double* result) {
    report("Pmm_L2", do_vec(2, n, m, eval_points, result));
}

void AcosOfChebyshevNodes(const int n, double* eval_points) {
    report("AcosOfChebyshevNodes", do_vec(0, n, 0, nullptr, eval_points));
}

void ChebyshevNodes(const int n, double* eval_points) {
    report("ChebyshevNodes", do_vec(1, n, 0, nullptr, eval_points));
}

void TransMult(double* rdatacoeffs, double* idatacoeffs, double* rfiltercoeffs, double* ifiltercoeffs,
               double* rres, double* ires, const int bw) {
    report("TransMult", do_transmult(rdatacoeffs, idatacoeffs, rfiltercoeffs, ifiltercoeffs, rres, ires, bw));
}

// ---- integer layout helpers --------------------------------------------------------
static int clamp_int(int64_t v) { return v > INT_MAX ? INT_MAX : (int)v; }

int TableSize(const int m, const int bw) { return clamp_int(table_size(m, bw)); }

int Spharmonic_TableSize(const int bw) {
    // cospml.c:85-92: closed-form upper bound up to bw 512, exact sum beyond
    if (bw <= 512) return (((4 * bw * bw * bw) + (6 * bw * bw) - (8 * bw)) / 24) + bw;
    int64_t s = 0;
    for (int m = 0; m < bw; ++m) s += table_size(m, bw);
    return clamp_int(s);
}

int Reduced_SpharmonicTableSize(const int bw, const int m) {
    int64_t s = 0;
    for (int i = 0; i < m; ++i) s += table_size(i, bw);
    return clamp_int(s);
}

int Reduced_Naive_TableSize(const int bw, const int m) {
    int64_t s = 0;
    for (int i = m; i < bw; ++i) s += bw - i;
    return clamp_int(2 * (int64_t)bw * s);
}

int TableOffset(int m, int l) { return clamp_int(table_offset(m, l)); }
int RowSize(const int m, const int l) { return row_size(m, l); }
int Transpose_RowSize(const int row, const int m, const int bw) { return transpose_row_size(row, m, bw); }
int IndexOfHarmonicCoeff(const int m, const int l, const int bw) { return index_of_harmonic_coeff(m, l, bw); }

// ---- Part 2 ------------------------------------------------------------------------
const char* s2g_last_error(void) { return g_last_error.c_str(); }
const char* s2g_version(void) { return "s2kit_gb300 0.1 (sm_103a)"; }

// ---- table files: the device tables of (bw, cutoff) saved to disk and loaded back ----
// Layout: 64-byte header {magic "S2GTAB1\0", int32 bw, int32 cutoff, int64 doubles per table,
// uint64 FNV-1a hash of the payload, 32 reserved bytes}, then the forward table and the
// transposed table (FP64, host byte order), exactly the device copies.
namespace {
struct TabFileHeader {
    char magic[8];
    int32_t bw, cutoff;
    int64_t total;
    uint64_t hash;
    int64_t reserved[4];
};
static_assert(sizeof(TabFileHeader) == 64, "table file header");
const char kTabMagic[8] = {'S', '2', 'G', 'T', 'A', 'B', '1', '\0'};

uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    return h;
}

int64_t tables_total(int bw, int cutoff) {
    int64_t n = 0;
    for (int m = 0; m < bw; ++m) n += order_size(bw, cutoff, m);
    return n;
}
}  // namespace

int s2g_tables_save(int bw, int cutoff, const char* path) {
    S2G_TRY(check_bw(bw));
    S2G_TRY(check_cutoff(bw, cutoff));
    if (!path) return fail(S2G_ERR_ARG, "NULL path");
    S2G_TRY(dropin_device());
    Tables* t;
    S2G_TRY(get_tables(bw, cutoff, &t));
    TabRef tref_{t};
    std::vector<double> buf(2 * (size_t)t->total);
    S2G_CUDA(cudaMemcpy(buf.data(), t->fwd, sizeof(double) * t->total, cudaMemcpyDeviceToHost));
    S2G_CUDA(cudaMemcpy(buf.data() + t->total, t->inv, sizeof(double) * t->total, cudaMemcpyDeviceToHost));
    TabFileHeader h{};
    memcpy(h.magic, kTabMagic, 8);
    h.bw = bw, h.cutoff = cutoff, h.total = t->total;
    h.hash = fnv1a(buf.data(), sizeof(double) * buf.size());
    FILE* fp = fopen(path, "wb");
    if (!fp) return fail(S2G_ERR_ARG, "cannot write %s", path);
    const bool ok = fwrite(&h, sizeof h, 1, fp) == 1 && fwrite(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
    if (fclose(fp) != 0 || !ok) return fail(S2G_ERR_ARG, "writing %s failed", path);
    return S2G_OK;
}

int s2g_tables_load(const char* path, int* bw_out, int* cutoff_out) {
    if (!path) return fail(S2G_ERR_ARG, "NULL path");
    FILE* fp = fopen(path, "rb");
    if (!fp) return fail(S2G_ERR_ARG, "cannot open %s", path);
    TabFileHeader h{};
    if (fread(&h, sizeof h, 1, fp) != 1 || memcmp(h.magic, kTabMagic, 8) != 0) {
        fclose(fp);
        return fail(S2G_ERR_ARG, "%s is not a table file", path);
    }
    int r = check_bw(h.bw);
    if (r == S2G_OK) r = check_cutoff(h.bw, h.cutoff);
    if (r == S2G_OK && h.total != tables_total(h.bw, h.cutoff))
        r = fail(S2G_ERR_ARG, "%s: %lld doubles per table, bw %d cutoff %d needs %lld", path, (long long)h.total,
                 h.bw, h.cutoff, (long long)tables_total(h.bw, h.cutoff));
    if (r != S2G_OK) {
        fclose(fp);
        return r;
    }
    std::vector<double> buf(2 * (size_t)h.total);
    const bool got = fread(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
    fclose(fp);
    if (!got) return fail(S2G_ERR_ARG, "%s is truncated", path);
    if (fnv1a(buf.data(), sizeof(double) * buf.size()) != h.hash)
        return fail(S2G_ERR_ARG, "%s: payload hash mismatch (corrupt file)", path);
    S2G_TRY(dropin_device());
    int dev;
    S2G_TRY(current_device(&dev));
    {
        std::lock_guard<std::mutex> lk(g_tab_mu);
        const auto key = std::make_tuple(dev, (int)h.bw, (int)h.cutoff);
        if (g_tables.count(key))
            return fail(S2G_ERR_ARG, "tables for bw %d cutoff %d already exist on device %d (s2g_cache_clear first)",
                        h.bw, h.cutoff, dev);
        Tables* t = new Tables();
        t->bw = h.bw, t->cutoff = h.cutoff, t->device = dev;
        cudaStream_t st;
        S2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        r = build_tables(t, st, buf.data(), buf.data() + h.total);
        cudaStreamDestroy(st);
        if (r != S2G_OK) {
            free_tables(t);
            return r;
        }
        t->refs = 1;  // the cache's own reference
        g_tables[key] = t;
    }
    if (bw_out) *bw_out = h.bw;
    if (cutoff_out) *cutoff_out = h.cutoff;
    return S2G_OK;
}

int s2g_cache_clear(void) {
    std::lock_guard<std::mutex> lk(g_tab_mu);
    for (auto& kv : g_tables)
        if (--kv.second->refs == 0) free_tables(kv.second);
    g_tables.clear();
    for (auto& kv : g_uploads) cudaFree(kv.second.d);
    g_uploads.clear();
    return S2G_OK;
}

// A host range that a queued copy of the host-buffer pipeline reads (H2D) or writes (D2H),
// with the event recorded after that copy.
struct HostDep {
    uintptr_t lo, hi;
    bool write;
    cudaEvent_t ev;
};

struct s2g_plan_s {
    int bw, cutoff, device;
    bool fly = false;  // s2g_plan_create_fly: no Legendre table, on-the-fly kernels
    Tables* t;
    Scratch work;
    Scratch io;
    Scratch cx;  // the two real fields' coefficients of COMPLEX split transforms
    cudaStream_t streams[3];
    cudaEvent_t events[6];
    // host-buffer pipeline state, kept across asynchronous calls
    std::vector<HostDep> deps;        // queued copies from or into host memory
    std::vector<cudaEvent_t> ev_free;  // recycled events
    unsigned long long seq = 0;        // chunks issued; staging buffer = seq & 1
    size_t stage = 0;                  // bytes of one staging buffer
    int host_pending = 0;              // host-buffer work may still be queued
};

// Waits for every queued host-buffer transfer and transform of the plan.
static int drain_host(s2g_plan p) {
    if (!p->host_pending) return S2G_OK;
    for (auto s : p->streams) S2G_CUDA(cudaStreamSynchronize(s));
    for (auto& d : p->deps) p->ev_free.push_back(d.ev);
    p->deps.clear();
    p->host_pending = 0;
    return S2G_OK;
}

// Drops the dependencies whose copies have completed.
static void prune_deps(s2g_plan p) {
    size_t k = 0;
    for (auto& d : p->deps) {
        if (cudaEventQuery(d.ev) == cudaSuccess)
            p->ev_free.push_back(d.ev);
        else
            p->deps[k++] = d;
    }
    p->deps.resize(k);
    if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();  // a query's "not yet", not a fault
}

// Makes stream s wait for the queued copies that conflict with host range [ptr, ptr + bytes):
// a read waits for earlier writes into the range, a write also for earlier reads out of it.
static int wait_host_range(s2g_plan p, cudaStream_t s, const void* ptr, size_t bytes, bool write) {
    const uintptr_t lo = (uintptr_t)ptr, hi = lo + bytes;
    for (auto& d : p->deps)
        if (d.lo < hi && lo < d.hi && (write || d.write)) S2G_CUDA(cudaStreamWaitEvent(s, d.ev, 0));
    return S2G_OK;
}

// Records that the copy just queued on s reads (or writes) host range [ptr, ptr + bytes).
static int note_host_range(s2g_plan p, cudaStream_t s, const void* ptr, size_t bytes, bool write) {
    cudaEvent_t e;
    if (!p->ev_free.empty()) {
        e = p->ev_free.back();
        p->ev_free.pop_back();
    } else {
        S2G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const cudaError_t r = cudaEventRecord(e, s);
    if (r != cudaSuccess) {
        p->ev_free.push_back(e);
        return cuda_fail(r, "cudaEventRecord");
    }
    p->deps.push_back({(uintptr_t)ptr, (uintptr_t)ptr + bytes, write, e});
    return S2G_OK;
}

int s2g_plan_create(s2g_plan* plan, int bw, int cutoff) {
    if (!plan) return fail(S2G_ERR_ARG, "NULL plan pointer");
    *plan = nullptr;
    S2G_TRY(check_bw(bw));
    S2G_TRY(check_cutoff(bw, cutoff));
    int dev;
    S2G_TRY(current_device(&dev));
    Tables* t;
    S2G_TRY(get_tables(bw, cutoff, &t));
    TabRef tref_{t};
    s2g_plan p = new s2g_plan_s();
    p->bw = bw;
    p->cutoff = cutoff;
    p->device = dev;
    p->t = t;
    for (auto& s : p->streams) S2G_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    for (auto& e : p->events) S2G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    tref_.t = nullptr;  // the plan keeps the reference
    *plan = p;
    return S2G_OK;
}

int s2g_plan_create_fly(s2g_plan* plan, int bw) {
    if (!plan) return fail(S2G_ERR_ARG, "NULL plan pointer");
    *plan = nullptr;
    S2G_TRY(check_bw(bw));
    int dev;
    S2G_TRY(current_device(&dev));
    Tables* t;
    S2G_TRY(get_tables(bw, 0, &t));
    TabRef tref_{t};
    s2g_plan p = new s2g_plan_s();
    p->bw = bw;
    p->cutoff = bw;
    p->device = dev;
    p->fly = true;
    p->t = t;
    for (auto& s : p->streams) S2G_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    for (auto& e : p->events) S2G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    tref_.t = nullptr;
    *plan = p;
    return S2G_OK;
}

int s2g_plan_destroy(s2g_plan p) {
    if (!p) return S2G_OK;
    cudaSetDevice(p->device);
    for (auto s : p->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    for (auto e : p->events) cudaEventDestroy(e);
    for (auto& d : p->deps) cudaEventDestroy(d.ev);
    for (auto e : p->ev_free) cudaEventDestroy(e);
    p->work.release();
    p->io.release();
    p->cx.release();
    put_tables(p->t);
    delete p;
    return S2G_OK;
}

size_t s2g_plan_workspace_size(s2g_plan p, int batch, int precision) {
    if (!p || batch < 1) return 0;
    if (precision == S2G_PREC_FP64) return f64_work_bytes(p->bw, batch, COMPLEX) + 256;
    return split_work_bytes(p->bw, batch);
}

// Device-buffer calls share the plan's scratch with the host-buffer pipeline, so they first wait
// for host-buffer work still queued (host = true: the pipeline itself, which orders its own work).
// fly_ok: the entry point also runs on an on-the-fly plan (the FP64 transforms); the others need
// the plan's Legendre tables.
static int plan_check(s2g_plan p, int batch, bool host = false, bool fly_ok = false) {
    if (!p) return fail(S2G_ERR_ARG, "NULL plan");
    if (batch < 1) return fail(S2G_ERR_ARG, "batch %d < 1", batch);
    if (p->fly && !fly_ok)
        return fail(S2G_ERR_ARG, "an on-the-fly plan runs only s2g_fst, s2g_inv_fst, s2g_fzt and s2g_conv");
    int dev;
    S2G_TRY(current_device(&dev));
    if (dev != p->device) return fail(S2G_ERR_ARG, "plan made on device %d used on device %d", p->device, dev);
    if (!host) S2G_TRY(drain_host(p));
    return S2G_OK;
}

int s2g_fst(s2g_plan p, const double* rdata, const double* idata, double* rcoeffs, double* icoeffs, int batch,
            DataFormat fmt, void* stream) {
    S2G_TRY(plan_check(p, batch, false, true));
    if (!rdata || !rcoeffs || !icoeffs || (fmt == COMPLEX && !idata)) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(p->work.ensure(f64_work_bytes(p->bw, batch, fmt)));
    if (p->fly) return fst_f64_fly(p->t, rdata, idata, rcoeffs, icoeffs, batch, fmt, p->work.ptr, (cudaStream_t)stream);
    return fst_f64(p->t, rdata, idata, rcoeffs, icoeffs, batch, fmt, p->cutoff, p->work.ptr, (cudaStream_t)stream);
}

int s2g_inv_fst(s2g_plan p, const double* rcoeffs, const double* icoeffs, double* rdata, double* idata, int batch,
                DataFormat fmt, void* stream) {
    S2G_TRY(plan_check(p, batch, false, true));
    if (!rdata || !rcoeffs || !icoeffs || (fmt == COMPLEX && !idata)) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(p->work.ensure(f64_work_bytes(p->bw, batch, fmt)));
    if (p->fly)
        return inv_fst_f64_fly(p->t, rcoeffs, icoeffs, rdata, idata, batch, fmt, p->work.ptr, (cudaStream_t)stream);
    return inv_fst_f64(p->t, rcoeffs, icoeffs, rdata, idata, batch, fmt, p->cutoff, p->work.ptr,
                       (cudaStream_t)stream);
}

int s2g_fzt(s2g_plan p, const double* rdata, const double* idata, double* rres, double* ires, int batch,
            DataFormat fmt, void* stream) {
    S2G_TRY(plan_check(p, batch, false, true));
    if (!rdata || !rres || !ires || (fmt == COMPLEX && !idata)) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(p->work.ensure(f64_work_bytes(p->bw, batch, REAL)));
    if (p->fly) return fzt_f64_fly(p->t, rdata, idata, rres, ires, batch, fmt, p->work.ptr, (cudaStream_t)stream);
    return fzt_f64(p->t, rdata, idata, rres, ires, batch, fmt, p->work.ptr, (cudaStream_t)stream);
}

int s2g_transmult(int bw, const double* rd, const double* id, const double* rf, const double* iff, double* rr,
                  double* ir, int batch, void* stream) {
    if (bw < 1 || batch < 1 || !rd || !id || !rf || !iff || !rr || !ir) return fail(S2G_ERR_ARG, "bad arguments");
    return transmult_f64(rd, id, rf, iff, rr, ir, bw, batch, (cudaStream_t)stream);
}

int s2g_conv(s2g_plan p, const double* rdata, const double* idata, const double* rfilter, const double* ifilter,
             double* rres, double* ires, int batch, void* stream) {
    S2G_TRY(plan_check(p, batch, false, true));
    if (p->cutoff != p->bw) return fail(S2G_ERR_ARG, "s2g_conv needs a plan with cutoff == bw");
    if (!rdata || !rfilter || !rres || !ires) return fail(S2G_ERR_ARG, "NULL argument");
    return conv_device(p->t, rdata, idata, rfilter, ifilter, rres, ires, batch, p->work, (cudaStream_t)stream);
}

int s2g_fst_real_f32(s2g_plan p, const float* grid, float* rc, float* ic, int batch, int precision, void* stream) {
    S2G_TRY(plan_check(p, batch));
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rc, ic}));
    S2G_TRY(p->work.ensure(split_work_bytes(p->bw, batch)));
    return fst_split(p->t, grid, rc, ic, batch, precision, p->work.ptr, (cudaStream_t)stream);
}

int s2g_inv_fst_real_f32(s2g_plan p, const float* rc, const float* ic, float* grid, int batch, int precision,
                         void* stream) {
    S2G_TRY(plan_check(p, batch));
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rc, ic}));
    S2G_TRY(p->work.ensure(split_work_bytes(p->bw, batch)));
    return inv_fst_split(p->t, rc, ic, grid, batch, precision, p->work.ptr, (cudaStream_t)stream);
}

int s2g_fst_complex_f32(s2g_plan p, const float* rgrid, const float* igrid, float* rc, float* ic, int batch,
                        int precision, void* stream) {
    S2G_TRY(plan_check(p, batch));
    if (!rgrid || !igrid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({rgrid, igrid, rc, ic}));
    S2G_TRY(p->work.ensure(split_work_bytes(p->bw, batch)));
    S2G_TRY(p->cx.ensure(split_complex_bytes(p->bw, batch)));
    return fst_split_complex(p->t, rgrid, igrid, rc, ic, batch, precision, p->work.ptr, p->cx.ptr,
                             (cudaStream_t)stream);
}

int s2g_inv_fst_complex_f32(s2g_plan p, const float* rc, const float* ic, float* rgrid, float* igrid, int batch,
                            int precision, void* stream) {
    S2G_TRY(plan_check(p, batch));
    if (!rgrid || !igrid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({rgrid, igrid, rc, ic}));
    S2G_TRY(p->work.ensure(split_work_bytes(p->bw, batch)));
    S2G_TRY(p->cx.ensure(split_complex_bytes(p->bw, batch)));
    return inv_fst_split_complex(p->t, rc, ic, rgrid, igrid, batch, precision, p->work.ptr, p->cx.ptr,
                                 (cudaStream_t)stream);
}

int s2g_fst_refined(s2g_plan p, const double* grid, double* rc, double* ic, int batch, int precision,
                    void* stream) {
    S2G_TRY(plan_check(p, batch));
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rc, ic}));
    S2G_TRY(p->work.ensure(refine_work_bytes(p->bw, batch)));
    S2G_TRY(p->io.ensure(refine_io_bytes(p->bw, batch)));
    return fst_refined(p->t, grid, rc, ic, batch, precision, p->io.ptr, p->work.ptr, (cudaStream_t)stream);
}

int s2g_inv_fst_refined(s2g_plan p, const double* rc, const double* ic, double* grid, int batch, int precision,
                        void* stream) {
    S2G_TRY(plan_check(p, batch));
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    S2G_TRY(check_aligned16({grid, rc, ic}));
    S2G_TRY(p->work.ensure(refine_work_bytes(p->bw, batch)));
    S2G_TRY(p->io.ensure(refine_io_bytes(p->bw, batch)));
    return inv_fst_refined(p->t, rc, ic, grid, batch, precision, p->io.ptr, p->work.ptr, (cudaStream_t)stream);
}

int s2g_plan_sync_status(s2g_plan p) {
    if (!p) return fail(S2G_ERR_ARG, "NULL plan");
    S2G_CUDA(cudaSetDevice(p->device));
    S2G_TRY(drain_host(p));
    S2G_CUDA(cudaDeviceSynchronize());
    return split_device_status(p->t, 1);
}

// Host-buffer variants: chunks of the batch flow H2D (stream 0) -> compute (stream 1) -> D2H
// (stream 2) through double-buffered device staging, so copies overlap the transforms.  The
// staging buffers, their events and the chunk sequence live in the plan, so an asynchronous call
// queues behind the previous one and its uploads overlap the previous call's downloads.  Copies
// from or into host memory that a queued copy of an earlier call writes or reads wait for it
// (per chunk, through the plan's list of queued host ranges).
static int host_pipeline(s2g_plan p, int fwd, const float* in0, const float* in1, float* out0, float* out1,
                         int batch, int precision, bool async) {
    S2G_TRY(plan_check(p, batch, true));
    const size_t S = 2 * (size_t)p->bw, ng = S * S, nc = (size_t)p->bw * p->bw;
    const size_t in_per = fwd ? ng : 2 * nc, out_per = fwd ? 2 * nc : ng;
    // 64 functions per chunk: the contraction's 64-function tiles are full, and the fill and drain
    // (the first upload and the last download overlap nothing) stay short; 32 left every tile
    // half empty (-14% end to end), 96 and 128 lengthen the fill and drain
    int chunk = batch < 64 ? batch : 64;
    while (chunk > 1 && (size_t)chunk * (in_per + out_per) * 4 * 2 > ((size_t)4 << 30)) chunk /= 2;
    // one staging layout for both directions, so queued chunks of an earlier call keep their buffers
    const size_t stage = (size_t)chunk * std::max(ng, 2 * nc) * 4;
    if (stage != p->stage || p->io.bytes < 4 * stage + 1024 || p->work.bytes < split_work_bytes(p->bw, chunk)) {
        S2G_TRY(drain_host(p));  // a new layout or a larger buffer: nothing queued may still use the old one
        S2G_TRY(p->io.ensure(4 * stage + 1024));
        S2G_TRY(p->work.ensure(split_work_bytes(p->bw, chunk)));
        p->stage = stage;
    }
    prune_deps(p);
    if (p->deps.size() > 4096) S2G_TRY(drain_host(p));
    char* base = (char*)p->io.ptr;
    float* din[2] = {(float*)base, (float*)(base + stage)};
    float* dout[2] = {(float*)(base + 2 * stage), (float*)(base + 3 * stage)};
    cudaStream_t h2d = p->streams[0], comp = p->streams[1], d2h = p->streams[2];
    cudaEvent_t in_ready[2] = {p->events[0], p->events[1]};
    cudaEvent_t done[2] = {p->events[2], p->events[3]};
    cudaEvent_t out_free[2] = {p->events[4], p->events[5]};
    p->host_pending = 1;
    const int nchunks = (batch + chunk - 1) / chunk;
    for (int c = 0; c < nchunks; ++c) {
        const int b = (int)(p->seq++ & 1);
        const int f0 = c * chunk, n = (batch - f0 < chunk) ? batch - f0 : chunk;
        S2G_CUDA(cudaStreamWaitEvent(h2d, done[b], 0));  // the transform that last read din[b]
        if (fwd) {
            const float* src = in0 + (size_t)f0 * ng;
            const size_t by = (size_t)n * ng * 4;
            S2G_TRY(wait_host_range(p, h2d, src, by, false));
            S2G_CUDA(cudaMemcpyAsync(din[b], src, by, cudaMemcpyHostToDevice, h2d));
            S2G_TRY(note_host_range(p, h2d, src, by, false));
        } else {
            const size_t by = (size_t)n * nc * 4;
            const float* s0 = in0 + (size_t)f0 * nc;
            const float* s1 = in1 + (size_t)f0 * nc;
            S2G_TRY(wait_host_range(p, h2d, s0, by, false));
            S2G_TRY(wait_host_range(p, h2d, s1, by, false));
            S2G_CUDA(cudaMemcpyAsync(din[b], s0, by, cudaMemcpyHostToDevice, h2d));
            S2G_CUDA(cudaMemcpyAsync(din[b] + (size_t)n * nc, s1, by, cudaMemcpyHostToDevice, h2d));
            S2G_TRY(note_host_range(p, h2d, s0, by, false));
            S2G_TRY(note_host_range(p, h2d, s1, by, false));
        }
        S2G_CUDA(cudaEventRecord(in_ready[b], h2d));
        S2G_CUDA(cudaStreamWaitEvent(comp, in_ready[b], 0));
        S2G_CUDA(cudaStreamWaitEvent(comp, out_free[b], 0));  // the download that last read dout[b]
        if (fwd)
            S2G_TRY(fst_split(p->t, din[b], dout[b], dout[b] + (size_t)n * nc, n, precision, p->work.ptr, comp));
        else
            S2G_TRY(inv_fst_split(p->t, din[b], din[b] + (size_t)n * nc, dout[b], n, precision, p->work.ptr, comp));
        S2G_CUDA(cudaEventRecord(done[b], comp));
        S2G_CUDA(cudaStreamWaitEvent(d2h, done[b], 0));
        if (fwd) {
            const size_t by = (size_t)n * nc * 4;
            float* o0 = out0 + (size_t)f0 * nc;
            float* o1 = out1 + (size_t)f0 * nc;
            S2G_TRY(wait_host_range(p, d2h, o0, by, true));
            S2G_TRY(wait_host_range(p, d2h, o1, by, true));
            S2G_CUDA(cudaMemcpyAsync(o0, dout[b], by, cudaMemcpyDeviceToHost, d2h));
            S2G_CUDA(cudaMemcpyAsync(o1, dout[b] + (size_t)n * nc, by, cudaMemcpyDeviceToHost, d2h));
            S2G_TRY(note_host_range(p, d2h, o0, by, true));
            S2G_TRY(note_host_range(p, d2h, o1, by, true));
        } else {
            const size_t by = (size_t)n * ng * 4;
            float* o0 = out0 + (size_t)f0 * ng;
            S2G_TRY(wait_host_range(p, d2h, o0, by, true));
            S2G_CUDA(cudaMemcpyAsync(o0, dout[b], by, cudaMemcpyDeviceToHost, d2h));
            S2G_TRY(note_host_range(p, d2h, o0, by, true));
        }
        S2G_CUDA(cudaEventRecord(out_free[b], d2h));
    }
    return async ? S2G_OK : drain_host(p);
}

int s2g_fst_real_f32_host(s2g_plan p, const float* grid, float* rc, float* ic, int batch, int precision) {
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    return host_pipeline(p, 1, grid, nullptr, rc, ic, batch, precision, false);
}

int s2g_inv_fst_real_f32_host(s2g_plan p, const float* rc, const float* ic, float* grid, int batch, int precision) {
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    return host_pipeline(p, 0, rc, ic, grid, nullptr, batch, precision, false);
}

int s2g_fst_real_f32_host_async(s2g_plan p, const float* grid, float* rc, float* ic, int batch, int precision) {
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    return host_pipeline(p, 1, grid, nullptr, rc, ic, batch, precision, true);
}

int s2g_inv_fst_real_f32_host_async(s2g_plan p, const float* rc, const float* ic, float* grid, int batch,
                                    int precision) {
    if (!grid || !rc || !ic) return fail(S2G_ERR_ARG, "NULL argument");
    return host_pipeline(p, 0, rc, ic, grid, nullptr, batch, precision, true);
}

int s2g_plan_wait(s2g_plan p) {
    if (!p) return fail(S2G_ERR_ARG, "NULL plan");
    S2G_CUDA(cudaSetDevice(p->device));
    return drain_host(p);
}

int s2g_prof_enable(int on) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto& r : g_prof_recs) {
        cudaEventSynchronize(r.b);
        g_prof_pool.push_back(r.a);
        g_prof_pool.push_back(r.b);
    }
    g_prof_recs.clear();
    g_prof_on.store(on ? 1 : 0);
    return S2G_OK;
}

int s2g_prof_report(char* buf, size_t len) {
    if (!buf || len < 3) return fail(S2G_ERR_ARG, "report buffer too small");
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::map<std::string, std::pair<long, double>> agg;
    for (auto& r : g_prof_recs) {
        S2G_CUDA(cudaEventSynchronize(r.b));
        float ms = 0.f;
        S2G_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        auto& a = agg[r.name];
        a.first += 1;
        a.second += ms;
    }
    std::string out = "{";
    for (auto& kv : agg) {
        char tmp[256];
        snprintf(tmp, sizeof(tmp), "%s\"%s\": [%ld, %.6f]", out.size() > 1 ? ", " : "", kv.first.c_str(),
                 kv.second.first, kv.second.second);
        out += tmp;
    }
    out += "}";
    if (out.size() + 1 > len) return fail(S2G_ERR_ARG, "report buffer too small (%zu needed)", out.size() + 1);
    memcpy(buf, out.c_str(), out.size() + 1);
    return S2G_OK;
}

unsigned long long s2g_launch_count(void) { return g_launches.load(); }

}  // extern "C"
